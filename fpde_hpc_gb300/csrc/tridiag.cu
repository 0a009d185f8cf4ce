// Batched Thomas solves (fpde_tridiag_solve): one thread per line, FP64, the reference's
// recurrences (al1 fpde_hpc_1d.cpp:4002-4027, bt1 :4585-4590, back-substitution and the
// boundary closures of U1 :4678-4725). Bt[i+1] is parked in u[i] during the forward sweep
// and Al[i+1] in a scratch array laid out [i][line] so that neighbouring lines coalesce.
#include "common.cuh"
#include "kernels.cuh"

namespace fpde {

__device__ __forceinline__ double right_closure(int kind, double gN, double dLN, double AlN, double BtN,
                                                double uNm1_old)
{
    if (kind == FPDE_BC_DIRICHLET) return gN;
    if (fabs(BtN) > 1e-15) {
        if (fabs(1.0 - AlN) > 1e-15) return (BtN + gN * dLN) / (1.0 - AlN);
        return uNm1_old;
    }
    if (fabs(1.0 - AlN) > 1e-15) return 0.0;
    return uNm1_old;
}

__global__ void k_thomas_lines(const double *__restrict__ a, const double *__restrict__ b,
                               const double *__restrict__ r, const double *__restrict__ om,
                               double *__restrict__ u, double *__restrict__ als, int64_t n_lines, int64_t N,
                               int64_t se, int64_t sl, int lk, const double *__restrict__ lv, int rk,
                               const double *__restrict__ rv, double dLN)
{
    const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n_lines) return;
    const int64_t base = l * sl;
    const double g0 = lv ? lv[l] : 0.0, gN = rv ? rv[l] : 0.0;
    const double uNm1_old = u[base + (N - 1) * se];
    double al = (lk == FPDE_BC_FLUX) ? 1.0 : 0.0;   // Al[1]
    double bt = g0;                                  // Bt[1]
    als[1 * n_lines + l] = al;
    u[base] = bt;
    for (int64_t i = 1; i < N; ++i) {
        const int64_t o = base + i * se;
        const double A = a[o], B = b[o], R = r[o], O = om[o];
        al = B / (R - A * al);
        bt = (al / B) * (A * bt - O);
        als[(i + 1) * n_lines + l] = al;
        u[o] = bt;
    }
    double U = right_closure(rk, gN, dLN, al, bt, uNm1_old);
    u[base + N * se] = U;
    for (int64_t i = N - 1; i >= 0; --i) {
        const int64_t o = base + i * se;
        U = als[(i + 1) * n_lines + l] * U + u[o];
        u[o] = U;
    }
}

int launch_thomas_lines(cudaStream_t st, const double *a, const double *b, const double *r, const double *om,
                        double *u, double *als, int64_t n_lines, int64_t N, int64_t se, int64_t sl, int lk,
                        const double *lv, int rk, const double *rv, double dLN)
{
    unsigned blocks = (unsigned)((n_lines + 127) / 128);
    k_thomas_lines<<<blocks, 128, 0, st>>>(a, b, r, om, u, als, n_lines, N, se, sl, lk, lv, rk, rv, dLN);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

}  // namespace fpde

using namespace fpde;

extern "C" int fpde_tridiag_solve(fpde_ctx *ctx, const double *a, const double *b, const double *r,
                                  const double *om, double *u, int64_t n_lines, int64_t N,
                                  int64_t stride_elem, int64_t stride_line, int left_kind,
                                  const double *left_val, int right_kind, const double *right_val,
                                  double dLN, int on_device)
{
    clear_error();
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    FPDE_CHECK_ARG(a && b && r && om && u, "null array");
    FPDE_CHECK_ARG(n_lines > 0 && N >= 2 && stride_elem > 0 && stride_line >= 0, "bad shape");
    FPDE_CHECK_ARG((left_kind == 0 || left_kind == 1) && (right_kind == 0 || right_kind == 1), "bad boundary kind");
    cudaStream_t st = ctx->stream;
    const int64_t extent = (n_lines - 1) * stride_line + N * stride_elem + 1;   // elements touched
    double *als = nullptr;
    if ((rc = dev_alloc((void **)&als, (size_t)(N + 1) * n_lines * sizeof(double)))) return rc;
    const double *da = a, *db = b, *dr = r, *dom = om, *dlv = left_val, *drv = right_val;
    double *du = u;
    std::vector<void *> tmp;
    auto up = [&](const double *h, int64_t n, const double **d) -> int {
        void *p = nullptr;
        int e = dev_alloc(&p, (size_t)n * sizeof(double));
        if (e) return e;
        tmp.push_back(p);
        cudaMemcpyAsync(p, h, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st);
        *d = (const double *)p;
        return 0;
    };
    if (!on_device) {
        if ((rc = up(a, extent, &da)) || (rc = up(b, extent, &db)) || (rc = up(r, extent, &dr)) ||
            (rc = up(om, extent, &dom)) || (left_val && (rc = up(left_val, n_lines, &dlv))) ||
            (right_val && (rc = up(right_val, n_lines, &drv))) || (rc = up(u, extent, (const double **)&du))) {
            for (void *p : tmp) dev_free(p);
            dev_free(als);
            return rc;
        }
    }
    rc = launch_thomas_lines(st, da, db, dr, dom, du, als, n_lines, N, stride_elem, stride_line, left_kind, dlv,
                             right_kind, drv, dLN);
    if (!rc && !on_device) {
        cudaError_t e = cudaMemcpyAsync(u, du, (size_t)extent * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) rc = set_error(FPDE_ERR_CUDA, "copy back: %s", cudaGetErrorString(e));
    }
    cudaError_t e = cudaStreamSynchronize(st);
    for (void *p : tmp) dev_free(p);
    dev_free(als);
    if (!rc && e != cudaSuccess) rc = set_error(FPDE_ERR_CUDA, "tridiag: %s", cudaGetErrorString(e));
    return rc;
}

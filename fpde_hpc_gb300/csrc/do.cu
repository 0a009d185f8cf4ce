// Distributed-order (DO) Caputo derivative of sampled series on the GPU.
//
// fr_do.cpp evaluates, for every node pt and time t, one L1 Caputo sum per order a_q
// (GPU DOC :146-236, one thread per order and node looping over t and j), divides by
// Gamma(2-a_q) and integrates over the orders (Sum :238-252). The sums are linear in the
// increments, so with the fused lag weights c[l] (fpde_do_weights) the whole operator is
//   DF[pt][t] = sum_{j in [max(j0,0), min(t, maxt))} (F[pt][j+1] - F[pt][j]) / tau * c[t-j-1]
// for t in [t0, ntau): one FP64 Toeplitz product per node, with no per-order table, no
// do1 intermediate of na x ntau values per node and no second kernel.
//
// Layout: F and DF node-major with time contiguous (F[pt*ldf + j], the reference's
// F[pt*total_ntau + j] and do2[pt*ntau2 + t]). One thread per (t, node): a warp covers 32
// consecutive t of one node, so F[j] is a broadcast load and c[t-j-1] a coalesced one.
#include "common.cuh"

namespace fpde {

__global__ void __launch_bounds__(128) k_do_derivative(const double *__restrict__ F, int64_t nodes, int64_t ldf,
                                                       int ntau, const double *__restrict__ c, int t0, int j0,
                                                       int maxt, double inv_tau, double *__restrict__ DF,
                                                       int64_t ldd, int append)
{
    const int t = t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntau) return;
    for (int64_t pt = blockIdx.y; pt < nodes; pt += gridDim.y) {
        const double *f = F + pt * ldf;
        const int jlo = j0 > 0 ? j0 : 0;
        const int jhi = (maxt == -1) ? t : (t < maxt ? t : maxt);
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int j = jlo;
        for (; j + 4 <= jhi; j += 4) {
            const double f0 = __ldg(f + j), f1 = __ldg(f + j + 1), f2 = __ldg(f + j + 2), f3 = __ldg(f + j + 3),
                         f4 = __ldg(f + j + 4);
            s0 = fma(f1 - f0, __ldg(c + (t - j - 1)), s0);
            s1 = fma(f2 - f1, __ldg(c + (t - j - 2)), s1);
            s2 = fma(f3 - f2, __ldg(c + (t - j - 3)), s2);
            s3 = fma(f4 - f3, __ldg(c + (t - j - 4)), s3);
        }
        for (; j < jhi; ++j) s0 = fma(__ldg(f + j + 1) - __ldg(f + j), __ldg(c + (t - j - 1)), s0);
        const double v = ((s0 + s1) + (s2 + s3)) * inv_tau;
        double *o = DF + pt * ldd + t;
        *o = append ? *o + v : v;
    }
}

}  // namespace fpde

using namespace fpde;

extern "C" int fpde_do_derivative(fpde_ctx *ctx, const double *F, int64_t nodes, int64_t ldf, int ntau, double tau,
                                  const double *c, int t0, int j0, int maxt, double *DF, int64_t ldd, int append)
{
    clear_error();
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    FPDE_CHECK_ARG(F && c && DF, "null pointer");
    FPDE_CHECK_ARG(nodes >= 0 && ntau >= 0 && t0 >= 0 && maxt >= -1, "bad sizes");
    FPDE_CHECK_ARG(tau > 0.0, "tau must be positive");
    FPDE_CHECK_ARG(ldf >= ntau && ldd >= ntau, "leading dimensions must cover ntau");
    if (nodes == 0 || t0 >= ntau) return FPDE_OK;
    dim3 grid((unsigned)((ntau - t0 + 127) / 128), (unsigned)(nodes < 65535 ? nodes : 65535));
    k_do_derivative<<<grid, 128, 0, ctx->stream>>>(F, nodes, ldf, ntau, c, t0, j0, maxt, 1.0 / tau, DF, ldd,
                                                   append);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

// The reference's Sum kernel in each of its history modes (fpde_hpc_1d.cpp:1407-1478, the
// sum_alg define; the CPU form is time_summing :4108-4151), on time-major snapshots
// old[t*OS + id]:
//   sum_alg 0  every term kb_3_cache[t] (old[t+1] - old[t]) / tau[t], newest first;
//   sum_alg 1  restricted summing: the same terms from the newest down to where the weight
//              falls below sum_param (time_summing's rule, or the GPU kernel's whole chunks);
//   sum_alg 2  series expansion: P moments per node updated with the newest increment, and
//              the history sum as their dot product with the binomial series coefficients.
//
// k_sum_window (sum_alg 0/1): the window (terms from the newest) is the same for every node; for
// sum_alg 1 a one-CTA kernel finds it from the weights on the device (no host round trip). One thread per node; the CTA's 256 threads first turn
// a chunk of 256 weights into kb/tau (one division per weight and CTA, not per node), then
// every thread walks the chunk's terms carrying the newer snapshot in a register: one 8-byte
// load, one FP64 subtraction and one FP64 FMA per node and term. GB300 issues FP64 at about
// two lanes per clock per SM, so the two FP64 operations per term, not HBM, bound the kernel
// (ncu: FP64 pipe ~90% busy, DRAM ~1/3). The snapshots are close, so the difference needs FP64;
// a float-float accumulation of the products (tried) was slower and ~10x less accurate.
//
// k_sum_series (sum_alg 2): 128 nodes per CTA. The CTA's moment tile (128 x P doubles,
// node-major as the reference's Htmp[id*P + j]) is staged through shared memory with
// coalesced loads and stores; each thread updates its node's P moments and forms the dot
// product in the reference's order j = 0 .. P-1. Rows of the tile are padded to an odd
// number of doubles so the per-node accesses are free of bank conflicts.
#include <algorithm>
#include <climits>
#include <cmath>

#include "common.cuh"

namespace fpde {

constexpr int SW_T = 256;         // threads (nodes) per CTA and weights per chunk of k_sum_window
constexpr int SS_T = 128;         // nodes per CTA of k_sum_series
constexpr int SERIES_PMAX = 128;  // most moments per node

// S[id] = sum over the newest L terms (L = *Ld when Ld is given, else Lh) (t = nt-1 .. nt-L, nt = old_size - 1) of
// kb[t] (old[t+1] - old[t]) / tau[t], newest first.
__global__ void __launch_bounds__(SW_T) k_sum_window(double *__restrict__ S, const double *__restrict__ old,
                                                     int old_size, int64_t OS, int64_t nodes,
                                                     const double *__restrict__ tau, const double *__restrict__ kb,
                                                     int Lh, const int *__restrict__ Ld)
{
    __shared__ double sw[SW_T];
    const int L = Ld ? *Ld : Lh;
    const int64_t id = (int64_t)blockIdx.x * SW_T + threadIdx.x;
    const bool in = id < nodes;
    const int nt = old_size - 1;
    double s = 0.0;
    double prev = (in && L > 0) ? old[(int64_t)nt * OS + id] : 0.0;
    for (int g0 = 0; g0 < L; g0 += SW_T) {               // terms g0 .. g0+SW_T-1 counted from the newest
        __syncthreads();
        const int t = nt - 1 - (g0 + (int)threadIdx.x);
        sw[threadIdx.x] = (g0 + (int)threadIdx.x < L) ? kb[t] / tau[t] : 0.0;
        __syncthreads();
        const int kend = min(SW_T, L - g0);
        if (in) {
            int64_t row = (int64_t)(nt - 1 - g0) * OS + id;
            for (int q = 0; q < kend; ++q, row -= OS) {
                const double cur = old[row];
                s = fma(sw[q], prev - cur, s);
                prev = cur;
            }
        }
    }
    if (in) S[id] = s;
}

// Terms the restricted rules use, counted from the newest, into *L (one CTA):
//   bs == 0: time_summing (:4110-4131): stop before the first |kb[t]| < thr;
//   bs  > 0: the GPU Sum kernel (:1422-1455): whole chunks of bs terms (weights before t = 0
//            count as 0), stopping after the first chunk whose bs weights are all below thr.
constexpr int WL_T = 1024;
__global__ void __launch_bounds__(WL_T) k_window_len(const double *__restrict__ kb, int nt, double thr, int bs,
                                                     int *__restrict__ L)
{
    __shared__ int first;
    if (threadIdx.x == 0) first = INT_MAX;
    __syncthreads();
    if (bs == 0) {
        for (int g = threadIdx.x; g < nt; g += WL_T)
            if (fabs(kb[nt - 1 - g]) < thr) atomicMin(&first, g);
    } else {
        const int nchunks = (nt + bs - 1) / bs;
        for (int m = threadIdx.x; m < nchunks; m += WL_T) {
            bool all_small = true;
            for (int q = 0; q < bs && all_small; ++q) {
                const int t = nt - 1 - (m * bs + q);
                const double kv = t >= 0 ? kb[t] : 0.0;
                if (!(fabs(kv) < thr)) all_small = false;
            }
            if (all_small) atomicMin(&first, m);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int n = nt;
        if (first != INT_MAX) n = bs == 0 ? first : (int)min((long long)nt, ((long long)first + 1) * bs);
        *L = n;
    }
}

struct SeriesCoef {
    double pw[SERIES_PMAX];   // gt^(j+1), formed by repeated multiplication (0 where not finite)
    double v[SERIES_PMAX];    // v_0 = gtj^-alpha, v_j = v_{j-1} (alpha + j - 1) / (j gtj) (0 where not finite)
};

__global__ void __launch_bounds__(SS_T) k_sum_series(double *__restrict__ S, const double *__restrict__ old,
                                                     int64_t OS, int64_t nodes, double *__restrict__ H, int P,
                                                     const double *__restrict__ row2, const double *__restrict__ tau_t,
                                                     const SeriesCoef cf)
{
    extern __shared__ double tile[];                     // [SS_T][Ps]
    __shared__ double sc[SERIES_PMAX], sv[SERIES_PMAX];
    const int Ps = P | 1;
    const int64_t n0 = (int64_t)blockIdx.x * SS_T;
    const int nn = (int)(nodes - n0 < SS_T ? nodes - n0 : SS_T);
    for (int j = threadIdx.x; j < P; j += SS_T) {
        double r = row2[j];
        if (!isfinite(r)) r = 0.0;
        sc[j] = cf.pw[j] * r;
        sv[j] = cf.v[j];
    }
    const double *Hb = H + n0 * P;
    for (int e = threadIdx.x; e < nn * P; e += SS_T) tile[(e / P) * Ps + (e % P)] = Hb[e];
    __syncthreads();
    if (threadIdx.x < nn) {
        const int64_t id = n0 + threadIdx.x;
        double d = old[OS + id] - old[id];
        if (!isfinite(d)) d = 0.0;
        double *h = tile + threadIdx.x * Ps;
        double acc = 0.0;
        for (int j = 0; j < P; ++j) {
            const double hj = fma(sc[j], d, h[j]);
            h[j] = hj;
            acc = fma(sv[j], hj, acc);
        }
        S[id] = acc / *tau_t;
    }
    __syncthreads();
    double *Hw = H + n0 * P;
    for (int e = threadIdx.x; e < nn * P; e += SS_T) Hw[e] = tile[(e / P) * Ps + (e % P)];
}

static size_t series_smem(int P) { return (size_t)SS_T * (P | 1) * sizeof(double); }

}  // namespace fpde

using namespace fpde;

extern "C" {

int fpde_sum(fpde_ctx *ctx, int sum_alg, int bs, int64_t OS, int64_t nodes, double *S, const double *old,
             int old_size, const double *tau, double *Htmp, const double *row2_precalc, const double *kb_3_cache,
             double sum_param, double gtj, double gt, double alpha, int tstep, int on_device)
{
    clear_error();
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    FPDE_CHECK_ARG(sum_alg >= 0 && sum_alg <= 2, "sum_alg must be 0, 1 or 2");
    FPDE_CHECK_ARG(on_device >= 0 && on_device <= 2, "on_device must be 0, 1 or 2");
    FPDE_CHECK_ARG(S && old && old_size >= 1 && nodes > 0 && OS >= nodes, "bad arguments");
    FPDE_CHECK_ARG(sum_alg != 1 || (bs >= 0 && bs <= 65536), "bs must be 0 .. 65536");
    // the reference truncates: (int)sum_param moments (time_summing :4137, Sum kernel :1462-1474)
    const int P = (sum_alg == 2 && std::isfinite(sum_param) && sum_param >= 1.0 && sum_param < 1e9)
                      ? (int)sum_param : 0;
    if (sum_alg == 2) {
        FPDE_CHECK_ARG(P >= 1 && P <= SERIES_PMAX,
                       "sum_alg 2: sum_param (moments per node) must be 1 .. 128");
        FPDE_CHECK_ARG(Htmp && row2_precalc && tau && tstep >= 0, "sum_alg 2: Htmp, row2_precalc and tau required");
    } else {
        FPDE_CHECK_ARG(old_size < 2 || (tau && kb_3_cache), "tau/kb_3_cache required for old_size >= 2");
    }
    cudaStream_t st = ctx->stream;
    const int nt = old_size - 1;
    const int nold = sum_alg == 2 ? std::min(old_size, 2) : old_size;
    double *dS = S, *dold = (double *)old, *dtau = (double *)tau, *dkb = (double *)kb_3_cache;
    double *dH = Htmp, *drow2 = (double *)row2_precalc;
    std::vector<void *> mine;
    auto take = [&](double **p, size_t n) -> int {
        int r = dev_alloc((void **)p, n * sizeof(double));
        if (!r) mine.push_back(*p);
        return r;
    };
    auto release = [&]() { for (void *p : mine) dev_free(p); };
    if (!on_device) {
        rc = take(&dS, nodes) || take(&dold, (size_t)nold * OS);
        if (!rc && sum_alg == 2) rc = take(&dH, (size_t)nodes * P) || take(&drow2, P) || take(&dtau, 1);
        if (!rc && sum_alg != 2 && nt > 0) rc = take(&dtau, nt) || take(&dkb, nt);
        if (rc) { release(); return rc; }
        cudaMemcpyAsync(dold, old, (size_t)nold * OS * sizeof(double), cudaMemcpyHostToDevice, st);
        if (sum_alg == 2) {
            cudaMemcpyAsync(dH, Htmp, (size_t)nodes * P * sizeof(double), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(drow2, row2_precalc, (size_t)P * sizeof(double), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dtau, tau + tstep, sizeof(double), cudaMemcpyHostToDevice, st);
        } else if (nt > 0) {
            cudaMemcpyAsync(dtau, tau, (size_t)nt * sizeof(double), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dkb, kb_3_cache, (size_t)nt * sizeof(double), cudaMemcpyHostToDevice, st);
        }
    }
    cudaError_t e = cudaSuccess;
    int launched = 0;
    if (sum_alg == 2) {
        if (old_size < 2) {
            e = cudaMemsetAsync(dS, 0, (size_t)nodes * sizeof(double), st);
        } else {
            // coefficients in the reference's order (time_summing :4141-4150 and
            // _kb_row2_fixed_coefs :1159-1180): powers by repeated multiplication, the series
            // coefficients by the recurrence; v_0 from the C library's pow as on the host
            SeriesCoef cf;
            double mult = gt, v = std::pow(gtj, -alpha);
            for (int j = 0; j < P; ++j) {
                cf.pw[j] = std::isfinite(mult) ? mult : 0.0;
                cf.v[j] = std::isfinite(v) ? v : 0.0;
                mult *= gt;
                const double i = (double)(j + 1);
                v *= -(-alpha - i + 1.0) / (i * gtj);
            }
            const size_t smem = series_smem(P);
            e = smem_opt_in((const void *)k_sum_series, (int)series_smem(SERIES_PMAX));
            if (e == cudaSuccess) {
                const double *tt = on_device ? dtau + tstep : dtau;
                k_sum_series<<<(unsigned)((nodes + SS_T - 1) / SS_T), SS_T, smem, st>>>(dS, dold, OS, nodes, dH, P,
                                                                                       drow2, tt, cf);
                e = cudaGetLastError();
                launched = 1;
            }
        }
    } else {
        // the window is the same for every node; sum_alg 1 finds it on the device
        const int *Ld = nullptr;
        if (sum_alg == 1 && nt > 0) {
            k_window_len<<<1, WL_T, 0, st>>>(dkb, nt, sum_param, bs, ctx->d_scratch);
            e = cudaGetLastError();
            Ld = ctx->d_scratch;
            launched = 1;
        }
        if (e == cudaSuccess) {
            k_sum_window<<<(unsigned)((nodes + SW_T - 1) / SW_T), SW_T, 0, st>>>(dS, dold, old_size, OS, nodes, dtau,
                                                                                dkb, nt, Ld);
            e = cudaGetLastError();
            launched += 1;
        }
    }
    if (e == cudaSuccess && launched) count_launches(launched);
    if (!on_device) {
        cudaMemcpyAsync(S, dS, (size_t)nodes * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (sum_alg == 2) cudaMemcpyAsync(Htmp, dH, (size_t)nodes * P * sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        release();
    }
    if (e != cudaSuccess) return set_error(FPDE_ERR_CUDA, "Sum (sum_alg %d) launch: %s", sum_alg, cudaGetErrorString(e));
    if (on_device != 2) FPDE_CUDA(cudaStreamSynchronize(st));
    return FPDE_OK;
}

}  // extern "C"

// Context, errors, L1 weights, the stored history and its FP64 sum.
//
// History layout in HBM: increments D_t = u^{t+1} - u^t, time-major, one row of P doubles
// per step (P = nodes rounded up to 512), so that appending a step writes one contiguous
// row and the history sum streams rows with coalesced 16-byte loads.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>
#include <string>

#include "common.cuh"
#include "kernels.cuh"
#include "ff.cuh"

namespace fpde {

static thread_local std::string g_err;
static thread_local int64_t g_launches = 0;

int set_error(int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}
void clear_error() { g_err.clear(); }
void count_launches(int64_t n) { g_launches += n; }

int ctx_enter(fpde_ctx *ctx)
{
    FPDE_CHECK_ARG(ctx, "null context");
    FPDE_CUDA(cudaSetDevice(ctx->device));
    return FPDE_OK;
}

int dev_alloc(void **p, size_t bytes)
{
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return set_error(FPDE_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    return FPDE_OK;
}

void dev_free(void *p)
{
    if (p) cudaFree(p);
}

int ctx_check_flags(fpde_ctx *ctx, const char *where)
{
    unsigned flags = 0;
    FPDE_CUDA(cudaMemcpyAsync(&flags, ctx->d_flags, sizeof flags, cudaMemcpyDeviceToHost, ctx->stream));
    FPDE_CUDA(cudaStreamSynchronize(ctx->stream));
    if (flags) {
        FPDE_CUDA(cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned), ctx->stream));
        FPDE_CUDA(cudaMemsetAsync(ctx->d_barrier, 0, 64 * 2 * sizeof(unsigned), ctx->stream));
        FPDE_CUDA(cudaStreamSynchronize(ctx->stream));
        if (flags & (DEVERR_BARRIER_TIMEOUT | DEVERR_MBAR_TIMEOUT))
            return set_error(FPDE_ERR_TIMEOUT, "%s: device wait timed out (flags 0x%x)", where, flags);
        if (flags & DEVERR_SOLVER)
            return set_error(FPDE_ERR_NUMERIC, "%s: iterative solve broke down or ran past its time limit (flags 0x%x)",
                             where, flags);
        return set_error(FPDE_ERR_ARG, "%s: device reported a bad shape (flags 0x%x)", where, flags);
    }
    return FPDE_OK;
}

// ------------------------------------------------------------------ weights

// int over an interval of length d ending a >= 0 before the evaluation time:
// ((a+d)^e - a^e)/e = a^e expm1(e log1p(d/a)) / e, e = 1 - alpha.
double l1_interval_weight(double alpha, double a, double d)
{
    double e = 1.0 - alpha;
    if (a <= 0.0) return std::pow(d, e) / e;
    return std::pow(a, e) * std::expm1(e * std::log1p(d / a)) / e;
}

double l1_lag(double alpha, int64_t j)
{
    double e = 1.0 - alpha;
    if (j == 0) return 1.0;
    double x = (double)j;
    return std::pow(x, e) * std::expm1(e * std::log1p(1.0 / x));
}

// ------------------------------------------------------------------ kernels

// Partial history sums: part[ks][i] = sum_{t in split ks} wt[t] * D[t][i], two nodes per
// thread (16-byte loads), eight rows in flight per thread.
__global__ void __launch_bounds__(256) k_l1_partial(const double2 *__restrict__ D, int64_t P2, int n,
                                                    const double *__restrict__ wt,
                                                    double2 *__restrict__ part)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int ks = blockIdx.y, KS = gridDim.y;
    const int t0 = (int)((int64_t)n * ks / KS), t1 = (int)((int64_t)n * (ks + 1) / KS);
    if (i >= P2) return;
    double ax = 0.0, ay = 0.0;
    int t = t0;
    for (; t + 8 <= t1; t += 8) {
        double2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = __ldcs(D + (int64_t)(t + u) * P2 + i);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const double w = __ldg(wt + t + u);
            ax = fma(w, v[u].x, ax);
            ay = fma(w, v[u].y, ay);
        }
    }
    for (; t < t1; ++t) {
        const double2 v = __ldcs(D + (int64_t)t * P2 + i);
        const double w = __ldg(wt + t);
        ax = fma(w, v.x, ax);
        ay = fma(w, v.y, ay);
    }
    part[(int64_t)ks * P2 + i] = make_double2(ax, ay);
}

__global__ void k_reduce_partials(const double *__restrict__ part, int KS, int64_t P, int64_t nodes,
                                  double *__restrict__ S)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nodes) return;
    double s = 0.0;
    for (int k = 0; k < KS; ++k) s += part[(int64_t)k * P + i];
    S[i] = s;
}

// u - last -> D row; last <- u
__global__ void k_append(const double *__restrict__ u, double *__restrict__ last,
                         double *__restrict__ row, int64_t nodes, int64_t P)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    if (i < nodes) {
        double v = u[i];
        row[i] = v - last[i];
        last[i] = v;
    } else {
        row[i] = 0.0;
    }
}

__global__ void k_copy_pad(const double *__restrict__ u, double *__restrict__ last, int64_t nodes, int64_t P)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P) last[i] = (i < nodes) ? u[i] : 0.0;
}

// The reference's Sum contract over snapshots (sum_alg 0), newest interval first.
__global__ void k_sum_snapshots(double *__restrict__ S, const double *__restrict__ old, int old_size,
                                int64_t OS, int64_t nodes, const double *__restrict__ tau,
                                const double *__restrict__ kb)
{
    int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nodes) return;
    double s = 0.0;
    for (int t = old_size - 2; t >= 0; --t) {
        double diff = old[(int64_t)(t + 1) * OS + id] - old[(int64_t)t * OS + id];
        s += kb[t] * diff / tau[t];
    }
    S[id] = s;
}

int launch_l1_partial(cudaStream_t st, const double *D, int64_t P, int n, const double *wt,
                      double *part, int KS)
{
    if (n <= 0) return FPDE_OK;
    dim3 grid((unsigned)((P / 2 + 255) / 256), (unsigned)KS);
    k_l1_partial<<<grid, 256, 0, st>>>((const double2 *)D, P / 2, n, wt, (double2 *)part);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

// u - last -> D row (FP64 and float pairs); last <- u
__global__ void k_append_ff(const double *__restrict__ u, double *__restrict__ last, double *__restrict__ row,
                            float2 *__restrict__ rowf, int64_t nodes, int64_t P)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    double d = 0.0;
    if (i < nodes) {
        const double v = u[i];
        d = v - last[i];
        last[i] = v;
    }
    row[i] = d;
    rowf[i] = d2ff(d);
}

int launch_append_ff(cudaStream_t st, const double *u, double *last, double *row, float2 *rowf, int64_t nodes,
                     int64_t P)
{
    k_append_ff<<<(unsigned)((P + 255) / 256), 256, 0, st>>>(u, last, row, rowf, nodes, P);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

int launch_append(cudaStream_t st, const double *u, double *last, double *row, int64_t nodes, int64_t P)
{
    k_append<<<(unsigned)((P + 255) / 256), 256, 0, st>>>(u, last, row, nodes, P);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

int device_sm_count()
{
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
    if (dev < 64 && cached[dev] > 0) return cached[dev];
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    if (dev < 64) cached[dev] = sms;
    return sms;
}

cudaError_t smem_opt_in(const void *fn, int bytes)
{
    static std::mutex mu;
    static std::set<std::pair<int, const void *>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count({dev, fn})) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) done.insert({dev, fn});
    return e;
}

int choose_splits(int n, int64_t P)
{
    // Split the rows so that ~32 CTAs per SM are in flight (the stream needs many loads
    // outstanding), with at least 64 rows per split.
    int64_t ctas_per_split = (P / 2 + 255) / 256;
    int64_t ks_par = ((int64_t)device_sm_count() * 32 + ctas_per_split - 1) / ctas_per_split;
    int64_t ks_rows = (n + 63) / 64;
    int64_t ks = ks_par < ks_rows ? ks_par : ks_rows;
    if (ks > KS_MAX) ks = KS_MAX;
    if (ks < 1) ks = 1;
    return (int)ks;
}

}  // namespace fpde

using namespace fpde;

// ====================================================================== C ABI

struct fpde_hist {
    fpde_ctx *ctx = nullptr;
    int64_t nodes = 0, P = 0, max_steps = 0;
    int precision = 0;
    double *D = nullptr;      // [max_steps][P]
    double *last = nullptr;   // [P]
    double *part = nullptr;   // [KS_MAX][P]
    double *w = nullptr;      // [max_steps]
    double *S = nullptr;      // [P]
    double *io = nullptr;     // [P] staging for host inputs
    int64_t n = 0;
    bool has_base = false;
};

extern "C" {

const char *fpde_last_error_string(void) { return fpde::g_err.c_str(); }
int64_t fpde_kernel_launch_count(void) { return fpde::g_launches; }

int fpde_ctx_create(int device, fpde_ctx **out)
{
    clear_error();
    FPDE_CHECK_ARG(out, "null output pointer");
    *out = nullptr;
    int ndev = 0;
    FPDE_CUDA(cudaGetDeviceCount(&ndev));
    FPDE_CHECK_ARG(device >= 0 && device < ndev, "device index out of range");
    FPDE_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    FPDE_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10)
        return set_error(FPDE_ERR_UNSUPPORTED, "device %d is sm_%d%d; this library is built for sm_103a",
                         device, prop.major, prop.minor);
    fpde_ctx *c = new fpde_ctx();
    c->device = device;
    c->sm_count = prop.multiProcessorCount;
    c->cc_major = prop.major;
    c->cc_minor = prop.minor;
    c->smem_optin = prop.sharedMemPerBlockOptin;
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return set_error(FPDE_ERR_CUDA, "stream create: %s", cudaGetErrorString(e)); }
    c->stream = c->own_stream;
    if (dev_alloc((void **)&c->d_flags, 64) || dev_alloc((void **)&c->d_barrier, 64 * 2 * sizeof(unsigned)) ||
        dev_alloc((void **)&c->d_scratch, 16 * sizeof(int))) {
        dev_free(c->d_flags);
        dev_free(c->d_barrier);
        cudaStreamDestroy(c->own_stream);
        delete c;
        return FPDE_ERR_NOMEM;
    }
    cudaMemset(c->d_flags, 0, 64);
    cudaMemset(c->d_barrier, 0, 64 * 2 * sizeof(unsigned));
    FPDE_CUDA(cudaDeviceSynchronize());
    *out = c;
    return FPDE_OK;
}

int fpde_ctx_destroy(fpde_ctx *ctx)
{
    if (!ctx) return FPDE_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    while (!ctx->lines.empty()) fpde_line_destroy(*ctx->lines.begin());
    while (!ctx->hists.empty()) fpde_history_destroy(*ctx->hists.begin());
    dev_free(ctx->d_flags);
    dev_free(ctx->d_barrier);
    dev_free(ctx->d_scratch);
    cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return FPDE_OK;
}

int fpde_ctx_set_stream(fpde_ctx *ctx, void *s)
{
    FPDE_CHECK_ARG(ctx, "null context");
    ctx->stream = s ? (cudaStream_t)s : ctx->own_stream;
    return FPDE_OK;
}

int fpde_ctx_synchronize(fpde_ctx *ctx)
{
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    FPDE_CUDA(cudaStreamSynchronize(ctx->stream));
    return ctx_check_flags(ctx, "synchronize");
}

int fpde_ctx_sm_count(const fpde_ctx *ctx, int *out)
{
    FPDE_CHECK_ARG(ctx && out, "null argument");
    *out = ctx->sm_count;
    return FPDE_OK;
}

int fpde_weights_l1(double alpha, const double *time, int n, double *kb, double *kkk0)
{
    FPDE_CHECK_ARG(time && n >= 0, "bad arguments");
    FPDE_CHECK_ARG(alpha > 0.0 && alpha <= 1.0, "alpha must be in (0, 1]");
    FPDE_CHECK_ARG(kb || n == 0, "kb is null");
    double T1 = time[n + 1];
    if (alpha == 1.0) {
        for (int t = 0; t < n; ++t) kb[t] = 0.0;
        if (kkk0) *kkk0 = 1.0;
        return FPDE_OK;
    }
    for (int t = 0; t < n; ++t) kb[t] = l1_interval_weight(alpha, T1 - time[t + 1], time[t + 1] - time[t]);
    if (kkk0) *kkk0 = l1_interval_weight(alpha, 0.0, T1 - time[n]);
    return FPDE_OK;
}

int fpde_weights_l1_lags(double alpha, int n, double *b)
{
    FPDE_CHECK_ARG(b && n >= 0, "bad arguments");
    FPDE_CHECK_ARG(alpha > 0.0 && alpha < 1.0, "alpha must be in (0, 1)");
    for (int j = 0; j < n; ++j) b[j] = l1_lag(alpha, j);
    return FPDE_OK;
}

int fpde_restricted_lags(const double *kb_lag, int n, double eps, int *max_lag)
{
    FPDE_CHECK_ARG(max_lag && n >= 0 && (kb_lag || n == 0), "bad arguments");
    FPDE_CHECK_ARG(std::isfinite(eps) && eps >= 0.0, "eps must be >= 0");
    int j = 0;
    while (j < n && !(std::fabs(kb_lag[j]) < eps)) ++j;    // kb_lag[j]: lag j + 1
    *max_lag = j;
    return FPDE_OK;
}

int fpde_gamma(double x, double *out)
{
    FPDE_CHECK_ARG(out, "null output");
    FPDE_CHECK_ARG(x > 0.0, "Gamma argument must be positive");
    *out = std::tgamma(x);
    return FPDE_OK;
}

int fpde_do_weights(int n_orders, const double *a, const double *qw, const double *gnorm, double tau, int n,
                    double *c)
{
    clear_error();
    FPDE_CHECK_ARG(n_orders > 0 && a && qw && c && n >= 0, "bad arguments");
    FPDE_CHECK_ARG(tau > 0.0, "tau must be positive");
    for (int q = 0; q < n_orders; ++q) {
        FPDE_CHECK_ARG(a[q] >= 0.0 && a[q] <= 1.0, "orders must lie in [0, 1]");
        FPDE_CHECK_ARG(!gnorm || gnorm[q] != 0.0, "zero normaliser");
    }
    // per order: qw * tau^{1-a} / Gamma(2-a), then the lag factors b_l(a) summed over orders
    std::vector<double> f(n_orders);
    for (int q = 0; q < n_orders; ++q)
        f[q] = qw[q] * std::pow(tau, 1.0 - a[q]) / (gnorm ? gnorm[q] : std::tgamma(2.0 - a[q]));
    for (int l = 0; l < n; ++l) {
        double s = 0.0;
        for (int q = 0; q < n_orders; ++q) s += f[q] * l1_lag(a[q], l);
        c[l] = s;
    }
    return FPDE_OK;
}

int fpde_history_create(fpde_ctx *ctx, int64_t nodes, int64_t max_steps, int precision, fpde_hist **out)
{
    clear_error();
    FPDE_CHECK_ARG(out, "null output pointer");
    *out = nullptr;
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    FPDE_CHECK_ARG(nodes > 0 && max_steps > 0, "nodes and max_steps must be positive");
    FPDE_CHECK_ARG(precision == FPDE_PREC_FP64, "this history interface stores FP64 increments");
    fpde_hist *h = new fpde_hist();
    h->ctx = ctx;
    h->nodes = nodes;
    h->P = (nodes + 511) / 512 * 512;
    h->max_steps = max_steps;
    h->precision = precision;
    size_t rows = (size_t)max_steps * (size_t)h->P * sizeof(double);
    if (dev_alloc((void **)&h->D, rows) || dev_alloc((void **)&h->last, h->P * sizeof(double)) ||
        dev_alloc((void **)&h->part, (size_t)KS_MAX * h->P * sizeof(double)) ||
        dev_alloc((void **)&h->w, (size_t)max_steps * sizeof(double)) ||
        dev_alloc((void **)&h->S, h->P * sizeof(double)) || dev_alloc((void **)&h->io, h->P * sizeof(double))) {
        std::string keep = fpde_last_error_string();
        fpde_history_destroy(h);
        return set_error(FPDE_ERR_NOMEM, "%s", keep.c_str());
    }
    ctx->hists.insert(h);
    *out = h;
    return FPDE_OK;
}

int fpde_history_destroy(fpde_hist *h)
{
    if (!h) return FPDE_OK;
    if (h->ctx) {
        cudaSetDevice(h->ctx->device);
        cudaStreamSynchronize(h->ctx->stream);
        h->ctx->hists.erase(h);
    }
    dev_free(h->D); dev_free(h->last); dev_free(h->part); dev_free(h->w); dev_free(h->S); dev_free(h->io);
    delete h;
    return FPDE_OK;
}

int fpde_history_reset(fpde_hist *h)
{
    FPDE_CHECK_ARG(h, "null history");
    h->n = 0;
    h->has_base = false;
    return FPDE_OK;
}

int fpde_history_length(const fpde_hist *h, int64_t *n)
{
    FPDE_CHECK_ARG(h && n, "null argument");
    *n = h->n;
    return FPDE_OK;
}

int fpde_history_append(fpde_hist *h, const double *u, int on_device)
{
    clear_error();
    FPDE_CHECK_ARG(h && u, "null argument");
    int rc = ctx_enter(h->ctx);
    if (rc) return rc;
    cudaStream_t st = h->ctx->stream;
    const double *src = u;
    if (!on_device) {
        FPDE_CUDA(cudaMemcpyAsync(h->io, u, h->nodes * sizeof(double), cudaMemcpyHostToDevice, st));
        src = h->io;
    }
    unsigned blocks = (unsigned)((h->P + 255) / 256);
    if (!h->has_base) {
        k_copy_pad<<<blocks, 256, 0, st>>>(src, h->last, h->nodes, h->P);
        FPDE_LAUNCHED(1);
        h->has_base = true;
    } else {
        if (h->n >= h->max_steps) return set_error(FPDE_ERR_CAPACITY, "history full (%lld steps)", (long long)h->max_steps);
        k_append<<<blocks, 256, 0, st>>>(src, h->last, h->D + h->n * h->P, h->nodes, h->P);
        FPDE_LAUNCHED(1);
        h->n++;
    }
    if (!on_device) FPDE_CUDA(cudaStreamSynchronize(st));
    return FPDE_OK;
}

int fpde_l1_sum(fpde_hist *h, const double *kb, const double *tau, double scale, double *S, int out_on_device)
{
    clear_error();
    FPDE_CHECK_ARG(h && S, "null argument");
    FPDE_CHECK_ARG(kb || h->n == 0, "kb is null");
    int rc = ctx_enter(h->ctx);
    if (rc) return rc;
    cudaStream_t st = h->ctx->stream;
    int n = (int)h->n;
    std::vector<double> w(n > 0 ? n : 1);
    for (int t = 0; t < n; ++t) w[t] = scale * (kb[t] / (tau ? tau[t] : 1.0));
    double *dst = out_on_device ? S : h->S;
    if (n == 0) {
        FPDE_CUDA(cudaMemsetAsync(dst, 0, h->nodes * sizeof(double), st));
    } else {
        FPDE_CUDA(cudaMemcpyAsync(h->w, w.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
        int KS = choose_splits(n, h->P);
        rc = launch_l1_partial(st, h->D, h->P, n, h->w, h->part, KS);
        if (rc) return rc;
        k_reduce_partials<<<(unsigned)((h->nodes + 255) / 256), 256, 0, st>>>(h->part, KS, h->P, h->nodes, dst);
        FPDE_LAUNCHED(1);
    }
    if (!out_on_device) {
        FPDE_CUDA(cudaMemcpyAsync(S, h->S, h->nodes * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    FPDE_CUDA(cudaStreamSynchronize(st));
    return FPDE_OK;
}

int fpde_sum_snapshots(fpde_ctx *ctx, double *S, const double *old, int old_size, int64_t OS,
                       int64_t nodes, const double *tau, const double *kb, int on_device)
{
    clear_error();
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    FPDE_CHECK_ARG(S && old && old_size >= 1 && OS >= nodes && nodes > 0, "bad arguments");
    FPDE_CHECK_ARG(old_size < 2 || (tau && kb), "tau/kb required for old_size >= 2");
    cudaStream_t st = ctx->stream;
    double *dS = S, *dold = (double *)old, *dtau = (double *)tau, *dkb = (double *)kb;
    int nt = old_size > 1 ? old_size - 1 : 1;
    if (!on_device) {
        if ((rc = dev_alloc((void **)&dS, nodes * sizeof(double)))) return rc;
        if ((rc = dev_alloc((void **)&dold, (size_t)old_size * OS * sizeof(double)))) { dev_free(dS); return rc; }
        if ((rc = dev_alloc((void **)&dtau, nt * sizeof(double)))) { dev_free(dS); dev_free(dold); return rc; }
        if ((rc = dev_alloc((void **)&dkb, nt * sizeof(double)))) { dev_free(dS); dev_free(dold); dev_free(dtau); return rc; }
        cudaMemcpyAsync(dold, old, (size_t)old_size * OS * sizeof(double), cudaMemcpyHostToDevice, st);
        if (old_size >= 2) {
            cudaMemcpyAsync(dtau, tau, (old_size - 1) * sizeof(double), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dkb, kb, (old_size - 1) * sizeof(double), cudaMemcpyHostToDevice, st);
        }
    }
    k_sum_snapshots<<<(unsigned)((nodes + 255) / 256), 256, 0, st>>>(dS, dold, old_size, OS, nodes, dtau, dkb);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) count_launches(1);
    if (!on_device) {
        cudaMemcpyAsync(S, dS, nodes * sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        dev_free(dS); dev_free(dold); dev_free(dtau); dev_free(dkb);
    }
    if (e != cudaSuccess) return set_error(FPDE_ERR_CUDA, "Sum launch: %s", cudaGetErrorString(e));
    FPDE_CUDA(cudaStreamSynchronize(st));
    return FPDE_OK;
}

}  // extern "C"

// Generalized-kernel L1 weights on the device (the reference's kb, fpde_hpc_1d.cpp:2167-2301,
// with g(t) of func_in_kernel, :1889-1930: t, sqrt(t), t^2, t^p): for step n with T = time[n+1]
//   kb_t(n) = int_{time[t]}^{time[t+1]} (g(T) - g(s))^{-alpha} ds,  t = 0..n-1,
// and kkk0(n), the same integral over the newest interval [time[n], T].
//
// With g = t^p and non-uniform steps these weights are not a function of the lag, so every
// step needs a fresh row. The reference evaluates each weight by truncated series
// (_kb_row :1933, _kb_row2 :2000) on the host, one at a time under an OpenMP critical
// section; here one thread evaluates one weight by quadrature in FP64:
//   - Gauss-Legendre when the interval lies at least 4 widths from both points where the
//     integrand is not smooth (s = T, and s = 0 when p is not a positive integer): 16 points,
//     8 beyond 32 widths (the error falls like rho^-2m, rho ~ 4 x the distance in widths);
//   - the double-exponential rule (nodes k/8, |k| <= 28) otherwise: it absorbs endpoint
//     singularities of the derivatives;
//   - on the newest interval the factor delta^-alpha (delta = T - s) is integrated
//     analytically on the last 1/16 of the interval (delta = h y^(1/(1-alpha)), leaving a
//     smooth integrand in y), and the double-exponential rule covers the rest.
// g(T) - g(s) is formed as -T^p expm1(p log1p(-delta/T)) while delta < T/2, so no
// cancellation occurs near T. The rule's nodes are formed on the host and passed by value.
#include <cmath>

#include "common.cuh"

namespace fpde {

constexpr int WG_DE = 57;
constexpr int WG_GL = 16;
constexpr int WG_GL8 = 8;

struct WeightRule {
    double u[WG_DE], v[WG_DE], w[WG_DE];   // double-exponential: u in (0,1), v = 1 - u, weights
    double x[WG_GL], gw[WG_GL];            // Gauss-Legendre on (0,1), 16 points
    double x8[WG_GL8], gw8[WG_GL8];        // and 8 points
};

__device__ __forceinline__ double wg_gdiff(double delta, double s, double T, double p, double Tp)
{
    if (p == 1.0) return delta;
    if (delta < 0.5 * T) return -Tp * expm1(p * log1p(-delta / T));
    return Tp - pow(s, p);
}

__device__ double wg_interval(const WeightRule &r, double s0, double s1, double T, double p, double alpha, double Tp,
                              bool smooth0)
{
    const double wdt = s1 - s0, d1 = T - s1;
    if (d1 == 0.0) {
        const double hw = wdt * 0.0625, q = 1.0 / (1.0 - alpha), R0 = pow(p * pow(T, p - 1.0), -alpha);
        double a = 0.0, b = 0.0;
        const double rest = wdt - hw;
        for (int k = 0; k < WG_DE; ++k) {
            const double delta = hw * pow(r.u[k], q);
            a += r.w[k] * (delta > 0.0 ? pow(wg_gdiff(delta, T - delta, T, p, Tp) / delta, -alpha) : R0);
            const double d2 = hw + rest * r.u[k], s2 = s0 + rest * r.v[k];
            b += r.w[k] * pow(wg_gdiff(d2, s2, T, p, Tp), -alpha);
        }
        return pow(hw, 1.0 - alpha) / (1.0 - alpha) * a + rest * b;
    }
    double sum = 0.0;
    if (d1 < 4.0 * wdt || (!smooth0 && s0 < 4.0 * wdt)) {
        for (int k = 0; k < WG_DE; ++k) {
            const double delta = d1 + wdt * r.u[k], s = s0 + wdt * r.v[k];
            sum += r.w[k] * pow(wg_gdiff(delta, s, T, p, Tp), -alpha);
        }
        return wdt * sum;
    }
    if (d1 < 32.0 * wdt || (!smooth0 && s0 < 32.0 * wdt)) {
        for (int i = 0; i < WG_GL; ++i) {
            const double s = s0 + wdt * r.x[i], delta = d1 + wdt * (1.0 - r.x[i]);
            sum += r.gw[i] * pow(wg_gdiff(delta, s, T, p, Tp), -alpha);
        }
        return wdt * sum;
    }
    for (int i = 0; i < WG_GL8; ++i) {
        const double s = s0 + wdt * r.x8[i], delta = d1 + wdt * (1.0 - r.x8[i]);
        sum += r.gw8[i] * pow(wg_gdiff(delta, s, T, p, Tp), -alpha);
    }
    return wdt * sum;
}

// out[(n - n0) * ld + t] = kb_t(n) for t < n, kkk0(n) at t = n; rows n = n0 .. n0 + gridDim.y - 1.
__global__ void __launch_bounds__(256) k_weights_g(const double *__restrict__ time, int n0, double p, double alpha,
                                                   double *__restrict__ out, int64_t ld, const WeightRule rule)
{
    const int n = n0 + (int)blockIdx.y;
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t > n) return;
    const double T = time[n + 1];
    double v;
    if (alpha == 1.0) {                                  // kb :2169-2175
        v = t == n ? 1.0 : 0.0;
    } else {
        const bool smooth0 = p >= 1.0 && p == floor(p);
        v = wg_interval(rule, time[t], time[t + 1], T, p, alpha, pow(T, p), smooth0);
    }
    out[(int64_t)blockIdx.y * ld + t] = v;
}

// m-point Gauss-Legendre nodes and weights on (0, 1): Newton on P_m from the usual guesses.
static void gauss_legendre(int m, double *x01, double *w01)
{
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < m; ++i) {
        double x = std::cos(pi * (i + 0.75) / (m + 0.5)), dp = 1.0;
        auto legendre = [m](double z, double &d) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= m; ++k) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            d = m * (z * p1 - p0) / (z * z - 1.0);
            return p1;
        };
        for (int it = 0; it < 100; ++it) {
            const double dx = legendre(x, dp) / dp;
            x -= dx;
            if (std::fabs(dx) < 1e-17) break;
        }
        legendre(x, dp);
        x01[i] = 0.5 * (x + 1.0);
        w01[i] = 1.0 / ((1.0 - x * x) * dp * dp);
    }
}

static const WeightRule &weight_rule()
{
    static WeightRule r = [] {
        WeightRule q;
        const double pi = 3.14159265358979323846;
        for (int k = 0; k < WG_DE; ++k) {
            const double t = (k - 28) / 8.0, e = std::exp(pi * std::sinh(t));
            q.u[k] = e / (1.0 + e);
            q.v[k] = 1.0 / (1.0 + e);
            q.w[k] = (pi / 8.0) * std::cosh(t) * q.u[k] * q.v[k];
        }
        gauss_legendre(WG_GL, q.x, q.gw);
        gauss_legendre(WG_GL8, q.x8, q.gw8);
        return q;
    }();
    return r;
}

}  // namespace fpde

using namespace fpde;

extern "C" {

int fpde_weights_g(fpde_ctx *ctx, double p, double alpha, const double *time, int n0, int n1, double *out,
                   int64_t ld, int on_device)
{
    clear_error();
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    FPDE_CHECK_ARG(time && out, "null argument");
    FPDE_CHECK_ARG(std::isfinite(p) && p > 0.0, "g(t) = t^p needs p > 0");
    FPDE_CHECK_ARG(std::isfinite(alpha) && alpha >= 0.0 && alpha <= 1.0, "alpha must be in [0, 1]");
    FPDE_CHECK_ARG(n0 >= 0 && n1 >= n0 && ld >= (int64_t)n1 + 1, "rows n0..n1 need ld >= n1 + 1");
    FPDE_CHECK_ARG(on_device >= 0 && on_device <= 2, "on_device must be 0, 1 or 2");
    const int rows = n1 - n0 + 1;
    FPDE_CHECK_ARG(rows <= 65535, "at most 65,535 rows per call");
    cudaStream_t st = ctx->stream;
    const double *dtime = time;
    double *dout = out;
    void *mine[2] = {nullptr, nullptr};
    if (!on_device) {
        if ((rc = dev_alloc(&mine[0], (size_t)(n1 + 2) * sizeof(double)))) return rc;
        if ((rc = dev_alloc(&mine[1], (size_t)rows * ld * sizeof(double)))) { dev_free(mine[0]); return rc; }
        dtime = (const double *)mine[0];
        dout = (double *)mine[1];
        cudaMemcpyAsync(mine[0], time, (size_t)(n1 + 2) * sizeof(double), cudaMemcpyHostToDevice, st);
        // the caller's rows go up too, so that entries past t = n come back unchanged
        cudaMemcpyAsync(mine[1], out, (size_t)rows * ld * sizeof(double), cudaMemcpyHostToDevice, st);
    }
    const dim3 grid((unsigned)((n1 + 1 + 255) / 256), (unsigned)rows);
    k_weights_g<<<grid, 256, 0, st>>>(dtime, n0, p, alpha, dout, ld, weight_rule());
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) count_launches(1);
    if (!on_device) {
        cudaMemcpyAsync(out, dout, (size_t)rows * ld * sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        dev_free(mine[0]);
        dev_free(mine[1]);
    }
    if (e != cudaSuccess) return set_error(FPDE_ERR_CUDA, "weights launch: %s", cudaGetErrorString(e));
    if (on_device != 2) FPDE_CUDA(cudaStreamSynchronize(st));
    return FPDE_OK;
}

}  // extern "C"

// One time step of a 1D line with solution-dependent coefficients (the reference's Richards
// problem, analytic_test 0 of fpde_hpc_1d.cpp, on a column with the history):
//   k_rich_coefs : every node's A_/B/R (:3095-3142) from the closures KK / inv_dw_dh at the
//                  current values (suction P = -(U - Z), :2499-2500, :2529), the right-hand side
//                  Om = -(Da kkk0/tau) U + src + Da S (Om1 :4191, :4267) and the surface condition
//                  of al1 / bc0 (:4004-4012, :4493-4500) - a flat grid over all SMs (the closures
//                  are a dozen FP64 pows per node);
//   k_rich_thomas: the Thomas solve of al1 / bt1 / U1 on those coefficients in one CTA of 1,024
//                  threads, each owning a segment of the line. The alpha recurrence
//                  Al[i+1] = B/(R - A Al[i]) is a Moebius map (taken in 1 - Al, where its
//                  matrices are positive), so the segments' 2x2 matrix products are combined by a
//                  block scan and every segment starts from its Al; the beta recurrence and the back substitution are
//                  affine maps, combined the same way (the latter from the right end). Within a
//                  segment each recurrence runs in the reference's order and rounding.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.cuh"
#include "richards.cuh"

namespace fpde {

constexpr int RT = 1024;                  // threads of the solve

// A, B, R, Om at nodes 1..N-1; al[1], bt[1] from the surface condition.
__global__ void __launch_bounds__(256) k_rich_coefs(RichLineArgs p)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > p.N) return;
    auto suction = [&](int q) { return -__dadd_rn(p.U[q], -p.Z[q]); };
    if (i == 0) {
        const double kk1 = rich_KK(suction(1), p.kform, p.ksat);
        const double Uc = __ddiv_rn(__dmul_rn(p.dL[0], p.E - 0.0), kk1);
        if (rich_inv_dw_dh(suction(0)) != RICH_SATURATED) {
            p.al[1] = 1.0;
            p.bt[1] = -Uc;
        } else {
            p.al[1] = 0.0;
            p.bt[1] = __ddiv_rn(__dmul_rn(-Uc, kk1), p.dL[0]);
        }
        return;
    }
    if (i >= p.N) return;
    const double Pm = suction(i - 1), Pi = suction(i);
    const double kkm = rich_KK(Pm, p.kform, p.ksat), kk = rich_KK(Pi, p.kform, p.ksat), iw = rich_inv_dw_dh(Pi);
    const double dq = p.dL[i], dm = p.dL[i - 1];
    const double dqq = __dmul_rn(dq, dq), dqm = __dmul_rn(dq, dm);
    p.cA[i] = __ddiv_rn(__dmul_rn(kkm, iw), dqm);
    p.cB[i] = __ddiv_rn(__dmul_rn(kk, iw), dqq);
    p.cR[i] = __dadd_rn(__dmul_rn(iw, __dadd_rn(__ddiv_rn(kk, dqq), __ddiv_rn(kkm, dqm))), p.lamR);
    double sv = 0.0;
    for (int k = 0; k < p.KS; ++k) sv += __ldcg(p.part + (int64_t)k * p.pstride + i);
    const double om = __dadd_rn(-__dmul_rn(p.lam, p.U[i]), p.src ? p.src[i] : 0.0);
    p.cOm[i] = __dadd_rn(om, sv);
}

struct Mob { double a, b, c, d; };                 // 2x2 matrix [[a, b], [c, d]]
struct Aff { double a, c; };                       // x -> a x + c

__device__ __forceinline__ Mob mob_mul(const Mob &x, const Mob &y)   // x y
{
    return {x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d};
}
// Projective maps are unchanged by a common scale: keep the entries near 1 with an exact power of two.
__device__ __forceinline__ Mob mob_norm(Mob m)
{
    const double s = fmax(fmax(fabs(m.a), fabs(m.b)), fmax(fabs(m.c), fabs(m.d)));
    if (s > 0.0 && isfinite(s)) {
        const int e = ilogb(s);
        m.a = scalbn(m.a, -e); m.b = scalbn(m.b, -e); m.c = scalbn(m.c, -e); m.d = scalbn(m.d, -e);
    }
    return m;
}
__device__ __forceinline__ Aff aff_after(const Aff &later, const Aff &earlier)
{
    return {later.a * earlier.a, later.a * earlier.c + later.c};
}
__device__ __forceinline__ Mob shfl_up_mob(const Mob &m, int o)
{
    return {__shfl_up_sync(0xffffffffu, m.a, o), __shfl_up_sync(0xffffffffu, m.b, o),
            __shfl_up_sync(0xffffffffu, m.c, o), __shfl_up_sync(0xffffffffu, m.d, o)};
}
__device__ __forceinline__ Aff shfl_up_aff(const Aff &m, int o)
{
    return {__shfl_up_sync(0xffffffffu, m.a, o), __shfl_up_sync(0xffffffffu, m.c, o)};
}

// Inclusive scan over the CTA's threads in index order, combined as later * earlier.
__device__ Mob scan_mob(Mob v, Mob *warp_tot)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const Mob u = shfl_up_mob(v, o);
        if (lane >= o) v = mob_norm(mob_mul(v, u));
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
        Mob w = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const Mob u = shfl_up_mob(w, o);
            if (lane >= o) w = mob_norm(mob_mul(w, u));
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    if (warp > 0) v = mob_norm(mob_mul(v, warp_tot[warp - 1]));
    __syncthreads();
    return v;
}
__device__ Aff scan_aff(Aff v, Aff *warp_tot)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const Aff u = shfl_up_aff(v, o);
        if (lane >= o) v = aff_after(v, u);
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
        Aff w = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const Aff u = shfl_up_aff(w, o);
            if (lane >= o) w = aff_after(w, u);
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    if (warp > 0) v = aff_after(v, warp_tot[warp - 1]);
    __syncthreads();
    return v;
}

__global__ void __launch_bounds__(RT, 1) k_rich_thomas(RichLineArgs p)
{
    __shared__ Mob mtot[32];
    __shared__ Aff atot[32];
    // the matrix prefixes (phase 1) and the affine ones (phases 2 and 4) share one buffer: a
    // barrier separates the last read of the former from the first write of the latter
    __shared__ double pref[4 * RT];
    Mob *mincl = reinterpret_cast<Mob *>(pref);
    Aff *aincl = reinterpret_cast<Aff *>(pref);
    __shared__ double uN_s;
    const int t = threadIdx.x, N = p.N;
    const int seg = (N - 1 + RT - 1) / RT;
    const int i0 = 1 + t * seg, i1 = min(i0 + seg, N);          // nodes [i0, i1) of 1..N-1
    const double uold_last = p.U[N - 1];                         // before any write (U1 :4695-4718)
    const double al1 = p.al[1], bt1 = p.bt[1];
    // 1. alpha. In g = 1 - Al the recurrence reads g' = (A g + l) / (A g + B + l) with
    // l = R - A - B (the local term): a Moebius map with positive entries [[A, l], [A, B + l]], whose
    // products lose nothing to cancellation even where Al is close to 1 (the map in Al itself,
    // [[0, B], [-A, R]], cancels there). Segment products, a scan, then each segment in order.
    Mob m = {1.0, 0.0, 0.0, 1.0};
    for (int i = i0; i < i1; ++i) {
        const double A = p.cA[i], B = p.cB[i], l = (p.cR[i] - A) - B;
        m = mob_norm(mob_mul(Mob{A, l, A, B + l}, m));
    }
    mincl[t] = scan_mob(m, mtot);
    __syncthreads();
    double al = al1;
    if (t > 0) {
        const Mob e = mincl[t - 1];                              // segments 0 .. t-1
        const double g1 = 1.0 - al1;                             // exact: Al[1] is 0 or 1
        al = 1.0 - (e.a * g1 + e.b) / (e.c * g1 + e.d);
    }
    for (int i = i0; i < i1; ++i) {
        al = __ddiv_rn(p.cB[i], __dadd_rn(p.cR[i], -__dmul_rn(p.cA[i], al)));  // al1 :4026
        p.al[i + 1] = al;
    }
    __syncthreads();
    // 2. beta: Bt[i+1] = (Al[i+1]/B_i)(A_i Bt[i] - Om_i) (bt1 :4587-4589), affine in Bt[i]
    Aff f = {1.0, 0.0};
    for (int i = i0; i < i1; ++i) {
        const double g = p.al[i + 1] / p.cB[i];
        f = aff_after(Aff{g * p.cA[i], -g * p.cOm[i]}, f);
    }
    aincl[t] = scan_aff(f, atot);
    __syncthreads();
    double bt = bt1;
    if (t > 0) bt = aincl[t - 1].a * bt1 + aincl[t - 1].c;
    for (int i = i0; i < i1; ++i) {
        bt = __dmul_rn(__ddiv_rn(p.al[i + 1], p.cB[i]), __dadd_rn(__dmul_rn(p.cA[i], bt), -p.cOm[i]));
        p.bt[i + 1] = bt;
    }
    __syncthreads();
    // 3. right end (U1 :4685-4719)
    if (t == 0) {
        double uN;
        if (p.rkind == FPDE_BC_DIRICHLET) {
            uN = p.gN;
        } else {
            const double BtN = p.bt[N], AlN = p.al[N];
            if (fabs(BtN) > 1e-15)
                uN = (fabs(1.0 - AlN) > 1e-15) ? __ddiv_rn(__dadd_rn(BtN, __dmul_rn(p.gN, p.dLN)), 1.0 - AlN) : uold_last;
            else
                uN = (fabs(1.0 - AlN) > 1e-15) ? 0.0 : uold_last;
        }
        uN_s = uN;
    }
    __syncthreads();
    const double uN = uN_s;
    // 4. back substitution U_i = Al[i+1] U_{i+1} + Bt[i+1] from the right: segment t maps the
    // value at i1 to the one at i0; the scan runs over the segments in reverse order
    Aff h = {1.0, 0.0};
    for (int i = i1 - 1; i >= i0; --i) h = aff_after(Aff{p.al[i + 1], p.bt[i + 1]}, h);
    __syncthreads();
    aincl[RT - 1 - t] = h;                                       // reversed order
    __syncthreads();
    const Aff hr = aincl[t];
    __syncthreads();
    aincl[t] = scan_aff(hr, atot);
    __syncthreads();
    double u = uN;                                               // the value at node i1
    if (t < RT - 1) {
        const Aff e = aincl[RT - 2 - t];                         // segments t+1 .. last
        u = e.a * uN + e.c;
    }
    __syncthreads();
    if (t == 0) p.U[N] = uN;
    for (int i = i1 - 1; i >= i0; --i) {
        u = __dadd_rn(__dmul_rn(p.al[i + 1], u), p.bt[i + 1]);   // U1 :4723
        p.U[i] = u;
    }
    __syncthreads();
    if (t == 0) p.U[0] = __dadd_rn(__dmul_rn(al1, p.U[1]), bt1);
}

int launch_rich_line_step(cudaStream_t st, const RichLineArgs &a)
{
    if (a.N < 2) return set_error(FPDE_ERR_ARG, "richards line: N must be at least 2");
    k_rich_coefs<<<(unsigned)((a.N + 1 + 255) / 256), 256, 0, st>>>(a);
    FPDE_LAUNCHED(1);
    k_rich_thomas<<<1, RT, 0, st>>>(a);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

}  // namespace fpde

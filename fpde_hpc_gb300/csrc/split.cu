// Block preparation of the split-precision path (per block of 64 steps):
//   k_absmax  : largest |increment| of the finished block (for the fp16 scale)
//   k_convert : FP64 increments (time-major ring, 64 rows of P) -> 16-bit hi/lo pairs in the
//               node-major history used as the K-major A operand, scaled by 2^sexp
//   k_wgen    : Toeplitz weight tile W[j][t] = w[n0+j-t] * 2^(kexp - sexp(t)), split hi/lo,
//               and the output scale 2^-kexp of the contraction
// The power-of-two scales keep fp16 operands inside its normal range; they are exact, and
// A*W keeps its value up to the single global factor 2^kexp undone in the epilogue.
// bf16 has float's exponent range and runs unscaled (sexp = kexp = 0).
#include <algorithm>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"
#include "kernels.cuh"

namespace fpde {

__global__ void k_absmax(const double *__restrict__ x, int64_t n, unsigned long long *slot)
{
    double m = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(x[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0 && m > 0.0) atomicMax(slot, (unsigned long long)__double_as_longlong(m));
    }
}

__device__ __forceinline__ int scale_exp_from_max(unsigned long long bits)
{
    const double m = __longlong_as_double((long long)bits);
    if (!(m > 0.0)) return 0;
    const int e = ilogb(m) + 1;           // m < 2^e
    return 14 - e;                        // scaled max < 2^14
}

__device__ __forceinline__ void split16(double v, int bf16, uint16_t &h, uint16_t &l)
{
    if (bf16) {
        __nv_bfloat16 hb = __double2bfloat16(v);
        __nv_bfloat16 lb = __double2bfloat16(v - (double)__bfloat162float(hb));
        h = __bfloat16_as_ushort(hb);
        l = __bfloat16_as_ushort(lb);
    } else {
        __half hh = __double2half(v);
        __half lh = __double2half(v - (double)__half2float(hh));
        h = __half_as_ushort(hh);
        l = __half_as_ushort(lh);
    }
}

// One CTA per 64 nodes: transpose a 64 (rows of the ring) x 64 (nodes) FP64 tile through
// shared memory and write each node's 64 new history columns as 16-byte vectors.
__global__ void __launch_bounds__(256) k_convert(const double *__restrict__ ring, int64_t P, int64_t nvalid,
                                                 const unsigned long long *__restrict__ slot, int *__restrict__ exps,
                                                 int blk, uint16_t *__restrict__ hi, uint16_t *__restrict__ lo,
                                                 int64_t ld, int64_t col0, int bf16)
{
    __shared__ double tile[64][65];
    const int64_t node0 = (int64_t)blockIdx.x * 64;
    const int sexp = bf16 ? 0 : scale_exp_from_max(*slot);
    const double sc = ldexp(1.0, sexp);
    if (blockIdx.x == 0 && threadIdx.x == 0) exps[blk] = sexp;
    for (int e = threadIdx.x; e < 64 * 64; e += 256) {
        const int r = e >> 6, c = e & 63;
        const int64_t node = node0 + c;
        tile[c][r] = node < nvalid ? ring[(int64_t)r * P + node] * sc : 0.0;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 8; e += 256) {
        const int c = e >> 3, g = e & 7;                 // node c, columns 8g..8g+7
        const int64_t node = node0 + c;
        if (node >= nvalid) continue;
        uint16_t h[8], l[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) split16(tile[c][8 * g + k], bf16, h[k], l[k]);
        uint4 vh, vl;
        vh.x = h[0] | ((uint32_t)h[1] << 16); vh.y = h[2] | ((uint32_t)h[3] << 16);
        vh.z = h[4] | ((uint32_t)h[5] << 16); vh.w = h[6] | ((uint32_t)h[7] << 16);
        vl.x = l[0] | ((uint32_t)l[1] << 16); vl.y = l[2] | ((uint32_t)l[3] << 16);
        vl.z = l[4] | ((uint32_t)l[5] << 16); vl.w = l[6] | ((uint32_t)l[7] << 16);
        *(uint4 *)(hi + node * ld + col0 + 8 * g) = vh;
        *(uint4 *)(lo + node * ld + col0 + 8 * g) = vl;
    }
}

// grid = (ceil(n0/256), 64): row j of the weight tile, columns t < n0.
__global__ void __launch_bounds__(256) k_wgen(const double *__restrict__ wlag, int n0, const int *__restrict__ exps,
                                              uint16_t *__restrict__ whi, uint16_t *__restrict__ wlo, int64_t ldw,
                                              int bf16, double *__restrict__ out_scale)
{
    __shared__ int s_kexp;
    if (threadIdx.x < 32) {
        int kmax = -100000;
        if (!bf16) {
            for (int b = threadIdx.x; b < n0 / 64; b += 32) {
                const double wm = wlag[n0 - 64 * b - 63];            // largest weight of block b
                const int ew = (wm > 0.0) ? ilogb(wm) + 1 : -100000; // wm < 2^ew
                kmax = max(kmax, ew - exps[b]);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) kmax = max(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
        }
        if (threadIdx.x == 0) s_kexp = bf16 ? 0 : (kmax > -100000 ? 14 - kmax : 0);
    }
    __syncthreads();
    const int kexp = s_kexp;
    const int j = blockIdx.y;
    const int t = blockIdx.x * 256 + threadIdx.x;
    if (blockIdx.x == 0 && j == 0 && threadIdx.x == 0) *out_scale = ldexp(1.0, -kexp);
    if (t >= n0) return;
    const double v = wlag[n0 + j - t] * ldexp(1.0, kexp - (bf16 ? 0 : exps[t >> 6]));
    uint16_t h, l;
    split16(v, bf16, h, l);
    whi[(int64_t)j * ldw + t] = h;
    wlo[(int64_t)j * ldw + t] = l;
}

// ---- exact three-slice form (bf16): x 2^-pe = a0 + a1 2^-8 + a2 2^-16 (+ rounding at 2^-16),
// |x| < 2^(pe+8), with integer a0 (|a0| <= 256) and a1, a2 (|.| <= 128); the exponent pe is
// stored per (node, 64-column block) for the history and per (step j, k-tile) for the
// weights.
// Integer form of the slicing (no FP64 arithmetic; GB300's FP64 pipe is narrow):
// v = rint(x * 2^(16 - pe)) from the double's bits, |v| <= 2^24, then balanced base-256
// digits v = a0 2^16 + a1 2^8 + a2 with |a0| <= 256, |a1|, |a2| <= 128.
__device__ __forceinline__ long long fixed16(double x, int pe)
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (ex == 0) return 0;                               // zero / subnormal: below the 2^-16 grid
    const long long mant = (long long)((bits & 0xFFFFFFFFFFFFFull) | (1ull << 52));
    const int sh = (ex - 1075) + 16 - pe;                // value * 2^(16-pe) = mant * 2^sh
    long long v;
    if (sh >= 0) {
        v = sh > 10 ? (1ll << 62) : (mant << sh);        // out of range: caller's exponent prevents it
    } else if (sh < -62) {
        v = 0;
    } else {
        const int r = -sh;
        const long long q = mant >> r;
        const long long rem = mant & ((1ll << r) - 1);
        const long long half = 1ll << (r - 1);
        v = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);   // round half to even
    }
    return (bits >> 63) ? -v : v;
}
__device__ __forceinline__ void digits3(long long v, uint16_t &s0, uint16_t &s1, uint16_t &s2)
{
    const int iv = (int)v;                               // |v| <= 2^24
    const int a0 = (iv + 32768) >> 16;
    const int r1 = iv - a0 * 65536;                      // [-32768, 32767]
    const int a1 = (r1 + 128) >> 8;
    const int a2 = r1 - a1 * 256;                        // [-128, 127]
    s0 = __bfloat16_as_ushort(__float2bfloat16((float)a0));
    s1 = __bfloat16_as_ushort(__float2bfloat16((float)a1 * (1.0f / 256.0f)));
    s2 = __bfloat16_as_ushort(__float2bfloat16((float)a2 * (1.0f / 65536.0f)));
}
// Block exponent from the largest magnitude: |x| < 2^(pe + 8).
__device__ __forceinline__ int exp_of_maxbits(unsigned long long mbits)
{
    const int ex = (int)((mbits >> 52) & 0x7FF);
    if (ex == 0) return 0;
    const int p = (ex - 1023) + 1 - 8;
    return p < -127 ? -127 : (p > 127 ? 127 : p);
}

// Four adjacent lanes per node, each with 16 of the node's 64 increments of the finished block
// (time-major ring: for each row the lanes of a warp read eight consecutive nodes). The block
// exponent is the maximum over the four lanes (shuffles); each lane then writes its 16 columns of
// the three slices. Sixteen values per thread keep the registers low and many nodes' loads in
// flight (one thread per node with all 64 values had left the kernel latency-bound).
constexpr int CONV_LANES = 4, CONV_ROWS = 64 / CONV_LANES;
__global__ void __launch_bounds__(256) k_convert3(const double *__restrict__ ring, int64_t P, int64_t nvalid,
                                                  uint16_t *__restrict__ h0, uint16_t *__restrict__ h1,
                                                  uint16_t *__restrict__ h2, int64_t ld, int64_t col0,
                                                  int8_t *__restrict__ pA, int64_t ldp, int blk)
{
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t node = gt / CONV_LANES;
    const int part = (int)(gt % CONV_LANES);
    const bool live = node < nvalid;
    const int r0 = part * CONV_ROWS;
    unsigned long long v[CONV_ROWS];
    unsigned long long mb = 0;
    const unsigned long long *src = (const unsigned long long *)ring + (live ? node : 0);
#pragma unroll
    for (int r = 0; r < CONV_ROWS; ++r) {
        v[r] = live ? __ldcg(src + (int64_t)(r0 + r) * P) : 0ull;
        const unsigned long long m0 = v[r] & 0x7FFFFFFFFFFFFFFFull;
        mb = m0 > mb ? m0 : mb;
    }
#pragma unroll
    for (int o = 1; o < CONV_LANES; o <<= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, mb, o, CONV_LANES);
        mb = other > mb ? other : mb;
    }
    if (!live) return;
    const int pe = exp_of_maxbits(mb);
    if (part == 0) pA[node * ldp + blk] = (int8_t)pe;
#pragma unroll
    for (int g = 0; g < CONV_ROWS / 8; ++g) {
        uint16_t a[8], b[8], c[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            digits3(fixed16(__longlong_as_double((long long)v[8 * g + k]), pe), a[k], b[k], c[k]);
        uint4 va, vb, vc;
        va.x = a[0] | ((uint32_t)a[1] << 16); va.y = a[2] | ((uint32_t)a[3] << 16);
        va.z = a[4] | ((uint32_t)a[5] << 16); va.w = a[6] | ((uint32_t)a[7] << 16);
        vb.x = b[0] | ((uint32_t)b[1] << 16); vb.y = b[2] | ((uint32_t)b[3] << 16);
        vb.z = b[4] | ((uint32_t)b[5] << 16); vb.w = b[6] | ((uint32_t)b[7] << 16);
        vc.x = c[0] | ((uint32_t)c[1] << 16); vc.y = c[2] | ((uint32_t)c[3] << 16);
        vc.z = c[4] | ((uint32_t)c[5] << 16); vc.w = c[6] | ((uint32_t)c[7] << 16);
        const int64_t o = node * ld + col0 + r0 + 8 * g;
        *(uint4 *)(h0 + o) = va;
        *(uint4 *)(h1 + o) = vb;
        *(uint4 *)(h2 + o) = vc;
    }
}

// grid = (n0/64 + n_grp - 1 k-tiles, 64 n_grp steps r, columns), 64 threads:
// W[c*64*n_grp + r][t] = w_c[n0 + r - t] for the k-tile (one weight tile per column of an
// ensemble; one column for a line or a grid). Row r (of weight group r/64) gets the columns
// t < n0 + 64 (r/64): every lag n0 + r - t it holds is at least 1. With n_grp > 1 the groups past
// the first serve the steps of the later blocks of a super-block starting at n0, the columns
// past n0 their contraction over the super-block's own history.
__global__ void __launch_bounds__(64) k_wgen3(const double *__restrict__ wlag_all, int64_t wstride, int n0,
                                              uint16_t *__restrict__ w0, uint16_t *__restrict__ w1,
                                              uint16_t *__restrict__ w2, int64_t ld, float *__restrict__ pW,
                                              int64_t ldp, int n_grp, int kt_lim)
{
    __shared__ double red[2];
    const int kt = blockIdx.x, r = blockIdx.y;
    if (kt >= n0 / 64 + r / 64 || kt >= kt_lim) return;  // the whole CTA (uniform)
    const int j = r + 64 * n_grp * blockIdx.z;
    const double *wlag = wlag_all + (int64_t)blockIdx.z * wstride;
    const int t = kt * 64 + threadIdx.x;
    const double v = wlag[n0 + r - t];
    double m = fabs(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    m = fmax(red[0], red[1]);
    const int pe = exp_of_maxbits((unsigned long long)__double_as_longlong(m));
    if (threadIdx.x == 0)                                // the scale 2^pe, exact (pe in [-127, 127])
        pW[(int64_t)j * ldp + kt] = pe >= -126 ? __int_as_float((pe + 127) << 23) : __int_as_float(0x00400000);
    uint16_t a, b, c;
    digits3(fixed16(v, pe), a, b, c);
    w0[(int64_t)j * ld + t] = a;
    w1[(int64_t)j * ld + t] = b;
    w2[(int64_t)j * ld + t] = c;
}

int launch_block_prep3(cudaStream_t st, const SplitPrep3 &p, int64_t n0, bool weights)
{
    if (n0 >= 64) {
        const int blk = (int)(n0 / 64) - 1;
        const int64_t threads = p.nvalid * CONV_LANES;
        k_convert3<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(p.ring, p.P, p.nvalid, p.hist[0], p.hist[1],
                                                                      p.hist[2], p.ld, n0 - 64, p.pA, p.ldp, blk);
        FPDE_LAUNCHED(1);
    }
    if (weights && n0 / 64 + (p.n_grp > 0 ? p.n_grp : 1) - 1 > 0) {
        const int ng = p.n_grp > 0 ? p.n_grp : 1;
        dim3 g((unsigned)(n0 / 64 + ng - 1), 64 * ng, (unsigned)(p.ncols > 0 ? p.ncols : 1));
        // columns stop at the slices' pitch: a later block of the super-block exists only below the
        // step capacity, so its contraction never reaches past it
        const int kt_lim = (int)std::min<int64_t>(p.ld / 64, p.ldp);
        k_wgen3<<<g, 64, 0, st>>>(p.wlag, p.wstride, (int)n0, p.w[0], p.w[1], p.w[2], p.ld, p.pW, p.ldp, ng, kt_lim);
        FPDE_LAUNCHED(1);
    }
    return FPDE_OK;
}

int launch_block_prep(cudaStream_t st, const SplitPrep &p, int64_t n0)
{
    const int blk = (int)(n0 / 64) - 1;          // the block that has just finished
    if (!p.bf16) {
        FPDE_CUDA(cudaMemsetAsync(p.slots + blk, 0, sizeof(unsigned long long), st));
        k_absmax<<<512, 256, 0, st>>>(p.ring, 64 * p.P, p.slots + blk);
        FPDE_LAUNCHED(1);
    }
    k_convert<<<(unsigned)((p.nvalid + 63) / 64), 256, 0, st>>>(p.ring, p.P, p.nvalid, p.slots + blk, p.exps, blk,
                                                                p.hist_hi, p.hist_lo, p.ld, n0 - 64, p.bf16);
    FPDE_LAUNCHED(1);
    dim3 g((unsigned)((n0 + 255) / 256), 64);
    k_wgen<<<g, 256, 0, st>>>(p.wlag, (int)n0, p.exps, p.w_hi, p.w_lo, p.ld, p.bf16, p.out_scale);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

}  // namespace fpde

// Declarations shared between the translation units of libfpde_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fpde {

constexpr int KS_MAX = 64;   // maximum number of row splits of the FP64 history sum

double l1_interval_weight(double alpha, double a, double d);
double l1_lag(double alpha, int64_t j);

// part[ks][i] = sum over the rows of split ks of wt[t] * D[t][i] (P doubles per row, P even).
int launch_l1_partial(cudaStream_t st, const double *D, int64_t P, int n, const double *wt,
                      double *part, int KS);
int choose_splits(int n, int64_t P);
// row[i] = u[i] - last[i], last[i] = u[i] for i < nodes; row[i] = 0 up to P.
int launch_append(cudaStream_t st, const double *u, double *last, double *row, int64_t nodes, int64_t P);
// The same, also writing the increment row as float pairs (rowf, for the float-float near history).
int launch_append_ff(cudaStream_t st, const double *u, double *last, double *row, float2 *rowf, int64_t nodes,
                     int64_t P);

}  // namespace fpde

namespace fpde {

// Buffers of the split-precision path touched by the per-block preparation (split.cu).
struct SplitPrep {
    const double *ring = nullptr;        // [64][P] FP64 increments of the finished block (time-major)
    int64_t P = 0, nvalid = 0;           // row pitch of the ring, nodes with history
    unsigned long long *slots = nullptr; // per block: max |increment| (double bits)
    int *exps = nullptr;                 // per block: scale exponent sexp
    uint16_t *hist_hi = nullptr, *hist_lo = nullptr;   // [rows][ld] node-major history
    uint16_t *w_hi = nullptr, *w_lo = nullptr;         // [64][ld] weight tile
    int64_t ld = 0;
    const double *wlag = nullptr;        // w[lag], lag = 0 .. max_steps + 64
    double *out_scale = nullptr;         // 2^-kexp for the contraction
    int bf16 = 0;
};
// Convert the block ending at n0 (n0 % 64 == 0, n0 >= 64) and build the weights of the
// next contraction (K = n0).
int launch_block_prep(cudaStream_t st, const SplitPrep &p, int64_t n0);

// Exact three-slice form: history slices and per-(node, block) exponents, weight slices and
// per-(step, k-tile) exponents.
struct SplitPrep3 {
    const double *ring = nullptr;
    int64_t P = 0, nvalid = 0;
    uint16_t *hist[3] = {nullptr, nullptr, nullptr};
    uint16_t *w[3] = {nullptr, nullptr, nullptr};
    int64_t ld = 0;
    int8_t *pA = nullptr;                // per (node, k-tile) exponents
    float *pW = nullptr;                 // per (step, k-tile) scales 2^e of the weight tiles
    int64_t ldp = 0;
    const double *wlag = nullptr;        // w[lag] (per column: ncols rows of wstride)
    int ncols = 1;                       // weight tiles (columns of an ensemble)
    int64_t wstride = 0;
    int n_grp = 1;                       // weight groups of 64 steps per column (a super-block)
};
// Convert the block ending at n0 (n0 % 64 == 0; nothing to convert at n0 = 0); with `weights`,
// also build the weight slices for the n_grp * 64 steps from n0 (rows c*64*n_grp + r of column c).
int launch_block_prep3(cudaStream_t st, const SplitPrep3 &p, int64_t n0, bool weights = true);

// Near history of step j of a block for every node:
//   S[i] = sum_{q<KS} far_q[j][i] + sum_{r<j} w[j-r] D_r[i],
// far partials [KS][64][P] (float pairs when pairs != 0), in float-float arithmetic on the FP32
// pipe (GB300 issues 2 DFMA/clk/SM) from the float-pair ring (ringf [64][P]) and float-pair lag
// weights (wff, per column at wff + col * wstride when cta_col is given: each 512-node group's
// column); one FP64 add per node.
int launch_near_history_ff(cudaStream_t st, const float2 *ringf, int64_t P, int j, const float2 *wff,
                           const double *cfar, int KS, int pairs, double *S, const int *cta_col = nullptr,
                           int64_t wstride = 0, const float2 *pre = nullptr, int r0 = 0);
// Sub-blocks of the near history: the partial sums of NEAR_SUB steps from the rows before j0
// (pre: NEAR_SUB rows of P float pairs).
constexpr int NEAR_SUB = 8;
int launch_near_pre_ff(cudaStream_t st, const float2 *ringf, int64_t P, int j0, const float2 *wff, const double *cfar,
                       int KS, int pairs, float2 *pre, const int *cta_col = nullptr, int64_t wstride = 0);

}  // namespace fpde

namespace fpde {

// One step of a line with solution-dependent coefficients (the Richards problem, rich_line.cu).
struct RichLineArgs {
    double *U;                           // N+1 values, advanced in place
    const double *Z, *dL;                // node coordinates and steps (N+1)
    const double *part;                  // history partials (S = sum over KS rows of pstride), or KS = 0
    int KS = 0;
    int64_t pstride = 0;
    const double *src = nullptr;         // optional source row (N+1)
    double *cA, *cB, *cR, *cOm, *al, *bt;   // scratch, N+1 each (al/bt: Al[i], Bt[i])
    double lam = 0, lamR = 0, E = 0, ksat = 0;
    int kform = 1, N = 0, rkind = 0;
    double gN = 0, dLN = 0;              // right end: Dirichlet value, or the flux and last step
};
int launch_rich_line_step(cudaStream_t st, const RichLineArgs &a);

}  // namespace fpde

namespace fpde {

// One pass of the 3D LOD with the implicit space-fractional line solves (impl 2, spacefrac.cu):
// one CTA per line; coef holds per line 7 rows of Nl+1 values (A, B, Rlap, mc0, mc1, mc2, iw).
struct LodSfArgs {
    double *U;
    const double *coef, *Tm;             // Tm: Nl+1 values, entries 2..Nl-1 read
    const double *part = nullptr;        // history partials of the K pass, or KS = 0
    int KS = 0;
    int64_t pstride = 0;
    const double *rp = nullptr, *bc = nullptr;
    double lam = 0, lamR = 0, thr = 0, dLN = 0;
    int Nl = 0, lines = 0, n1 = 0, sd = 0, maxiter = 1, rkind = 0;
    int fast = 0;                        // tree dot products and fused multiply-adds (else bitwise)
    int64_t s1 = 0, s2 = 0, st = 0;
    unsigned long long *iters = nullptr; // total iterations (may be null)
    unsigned *flags = nullptr;
};
int launch_lod_pass_sf(cudaStream_t st, const LodSfArgs &a);
size_t sf_smem_bytes(int n);
int sf_prepare();

}  // namespace fpde

#include <vector>

namespace fpde {

// The fully implicit 3D space-fractional operator (implicit3d 1, spacefrac3d.cu) on the
// V = (sN+2)(M+2)(K+2) + 1 values of a grid (i fastest) and the one past it. Device pointers.
struct Sf3dSystem {
    int sN = 0, M = 0, K = 0, sd = 0;
    const double *mat = nullptr;         // 7 x V: Mat_3d[0..6]
    const double *mc = nullptr;          // 9 x V: Mcoefs_3d[c][d] at plane 3c+d (c = 0 sN, 1 _M, 2 K)
    const double *Tm[3] = {nullptr, nullptr, nullptr};   // axis c: len_c + 1 values
    const double *iw = nullptr;          // 3 x V, or null (1.0)
    const double *rs = nullptr;          // V row scales, or null
};
struct Sf3dWork;                         // the solve's device vectors
int sf3d_work_create(const Sf3dSystem &s, Sf3dWork **w);
void sf3d_work_destroy(Sf3dWork *w);
// r = A x (tc: 3V scratch for the axes' Toeplitz terms); two launches.
int sf3d_enqueue_matvec(cudaStream_t st, const Sf3dSystem &s, double *tc, const double *x, double *r);
// solve_mln<1> of A x = B from x (V values each), one cooperative launch; exact: the reference's
// sequential dot products. iters_total (device, may be null) += iterations; iters_out (device int,
// may be null) = iterations.
int sf3d_enqueue_solve(cudaStream_t st, const Sf3dSystem &s, Sf3dWork *w, const double *B, double *x, double thr,
                       int maxiter, bool exact, unsigned long long *iters_total, int *iters_out, unsigned *flags);

// Right-hand side of one implicit3d LOD step (and the grid copied into the solve's x).
struct Sf3dRhsArgs {
    int sN = 0, M = 0, K = 0;
    const double *U = nullptr;
    double *x = nullptr, *Om = nullptr;
    const double *rp = nullptr, *bc = nullptr;   // this step's rows (may be null)
    const double *part = nullptr;        // history partials of the K pass, or KS = 0
    int KS = 0;
    int64_t pstride = 0;
    double lam = 0;
    int rkind[3] = {0, 0, 0};
    double dLN[3] = {0, 0, 0};
};
int launch_sf3d_rhs(cudaStream_t st, const Sf3dRhsArgs &a);
// U[v] = x[v] for the G grid nodes.
int launch_sf3d_store(cudaStream_t st, const double *x, double *U, int64_t G);
// Mat_3d (7 x V), Mcoefs_3d (9 x V) and the inv_dw_dh planes (3 x V) of a LOD with implicit3d, from
// the per-pass coefficient grids (coefA/B/Rlap: 3 x G; mc[pass]: 3 x G; iw[pass]: G).
void sf3d_assemble_host(int sN, int M, int K, const double *coefA, const double *coefB, const double *coefRlap,
                        const double *const *mc, const double *const *iw, const int *rkind, double lamR,
                        std::vector<double> &mat, std::vector<double> &mc3, std::vector<double> &iw3);

}  // namespace fpde

// Drop-in for the reference's fully implicit 3D space-fractional solve through the C ABI.
//
// With implicit3d 1 and impl 2, calc_step (fpde_hpc_1d.cpp:5681-5716) assembles Mat_3d, Mcoefs_3d
// and Om and calls solve_mln<1>((double **)this, Om, Al, N, impl_err, impl_niter, vmul_T_3d, 0, N)
// with N = (sN+2)(_M+2)(K+2) + 1. This program is that call with the library in its place: it
// hands the reference's own arrays to fpde_sf3d_solve (exact dot products: the reference's
// iterates) and, for the product alone, to fpde_sf3d_matvec.
//
// Input (little-endian, written by tests/test_cpp_dropin.py from a recorded reference run):
// int64 sN, M, K, space_der, impl_niter; double impl_err; Mat_3d[7][V]; Mcoefs_3d[9][V] (plane
// 3c+d); Tm0[sN+1], Tm1[M+1], Tm2[K+1]; iw[3][V]; Om[V]; Al[V] (the initial guess); x[V] (a
// vector for the product).
// Output: the product r[V], the solution Al[V], int64 iterations.
//
//     dropin_sf3d IN OUT [device]
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fpde_gb300.h"

namespace {

bool read_all(FILE *f, void *p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: %s IN OUT [device]\n", argv[0]);
        return 2;
    }
    const int device = argc > 3 ? atoi(argv[3]) : 0;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t hdr[5];
    double thr = 0.0;
    if (!read_all(f, hdr, sizeof hdr) || !read_all(f, &thr, sizeof thr)) return 2;
    const int sN = (int)hdr[0], M = (int)hdr[1], K = (int)hdr[2], sd = (int)hdr[3], maxiter = (int)hdr[4];
    const size_t V = (size_t)(sN + 2) * (M + 2) * (K + 2) + 1;
    std::vector<double> mat(7 * V), mc(9 * V), Tm0(sN + 1), Tm1(M + 1), Tm2(K + 1), iw(3 * V), Om(V), Al(V), x(V);
    bool ok = read_all(f, mat.data(), mat.size() * 8) && read_all(f, mc.data(), mc.size() * 8) &&
              read_all(f, Tm0.data(), Tm0.size() * 8) && read_all(f, Tm1.data(), Tm1.size() * 8) &&
              read_all(f, Tm2.data(), Tm2.size() * 8) && read_all(f, iw.data(), iw.size() * 8) &&
              read_all(f, Om.data(), V * 8) && read_all(f, Al.data(), V * 8) && read_all(f, x.data(), V * 8);
    fclose(f);
    if (!ok) return 2;

    fpde_ctx *ctx = nullptr;
    if (fpde_ctx_create(device, &ctx)) {
        fprintf(stderr, "GB300: %s\n", fpde_last_error_string());
        return 1;
    }
    fpde_sf3d_system sys = {sN, M, K, sd, mat.data(), mc.data(), {Tm0.data(), Tm1.data(), Tm2.data()}, iw.data(),
                            nullptr};
    std::vector<double> r(V);
    int iters = 0;
    if (fpde_sf3d_matvec(ctx, &sys, x.data(), r.data(), /*on_device=*/0) ||
        fpde_sf3d_solve(ctx, &sys, Om.data(), Al.data(), thr, maxiter, /*exact=*/1, &iters, /*on_device=*/0)) {
        fprintf(stderr, "GB300: %s\n", fpde_last_error_string());
        fpde_ctx_destroy(ctx);
        return 1;
    }
    fpde_ctx_destroy(ctx);
    FILE *o = fopen(argv[2], "wb");
    if (!o) return 2;
    const int64_t it64 = iters;
    fwrite(r.data(), 8, V, o);
    fwrite(Al.data(), 8, V, o);
    fwrite(&it64, 8, 1, o);
    fclose(o);
    printf("vmul_T_3d and solve_mln<1> through the C ABI: V = %zu, %d iterations\n", V, iters);
    return 0;
}

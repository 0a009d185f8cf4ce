// A whole H_solver column advanced on the device from C++ through the C ABI, three ways:
//   whole  - one fpde_line_solve_host call (upload, all steps, download), the end-to-end call;
//   blocks - fpde_step_block until the history is full: the blocked schedule one 64-step block
//            per call (append -> far history -> near history -> RHS -> solve), which replaces the
//            reference's per-step calc_step -> fr_ocl_call_sum -> time_summing sequence
//            (fpde_hpc_1d.cpp:5156-5157, :1835-1880, :4100-4104);
//   steps  - fpde_line_run(line, 1) once per time step, as the reference's time loop (solve,
//            :8932-9547) calls calc_step.
// The line's coefficients come from fpde_line_coefs (A_ / B / R, :3095-3142) and its weights are
// the library's closed form (precalc_kb_3, :4069-4085).
//
// Input (little-endian, from tests/test_cpp_dropin.py): int64 N, int64 steps, int64 precision,
// double alpha, tau, Da; k[N+1] (conductivity at the nodes), u0[N+1].
// Output: the final state (N+1 doubles) of each way, in the order above.
//
//     dropin_line IN OUT [device]
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fpde_gb300.h"

#define CHECK(call)                                                                      \
    do {                                                                                 \
        if ((call) != FPDE_OK) {                                                         \
            fprintf(stderr, "%s failed: %s\n", #call, fpde_last_error_string());        \
            return 1;                                                                    \
        }                                                                                \
    } while (0)

static bool read_all(FILE *f, void *p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: %s IN OUT [device]\n", argv[0]);
        return 2;
    }
    FILE *in = fopen(argv[1], "rb");
    if (!in) return 2;
    int64_t N = 0, steps = 0, precision = 0;
    double alpha = 0, tau = 0, Da = 0;
    if (!read_all(in, &N, 8) || !read_all(in, &steps, 8) || !read_all(in, &precision, 8) ||
        !read_all(in, &alpha, 8) || !read_all(in, &tau, 8) || !read_all(in, &Da, 8) || N < 2 || steps < 1)
        return 2;
    std::vector<double> k(N + 1), u0(N + 1);
    if (!read_all(in, k.data(), 8 * (N + 1)) || !read_all(in, u0.data(), 8 * (N + 1))) return 2;
    fclose(in);

    std::vector<double> dL(N + 1, 1.0 / (double)N), A(N + 1), B(N + 1), R(N + 1);
    CHECK(fpde_line_coefs(N, k.data(), nullptr, dL.data(), A.data(), B.data(), R.data()));
    fpde_line_desc d = {};
    d.N = N;
    d.alpha = alpha;
    d.tau = tau;
    d.Da = Da;
    d.left_kind = FPDE_BC_DIRICHLET;
    d.right_kind = FPDE_BC_DIRICHLET;
    d.dLN = 1.0 / (double)N;
    d.precision = (int)precision;
    d.max_steps = (int)steps;

    fpde_ctx *ctx = nullptr;
    CHECK(fpde_ctx_create(argc > 3 ? atoi(argv[3]) : 0, &ctx));
    FILE *out = fopen(argv[2], "wb");
    if (!out) return 2;
    std::vector<double> u(N + 1);
    for (int way = 0; way < 3; ++way) {
        fpde_line *line = nullptr;
        CHECK(fpde_line_create(ctx, &d, A.data(), B.data(), R.data(), u0.data(), &line));
        if (way == 0) {
            CHECK(fpde_line_solve_host(line, u0.data(), (int)steps, u.data()));
        } else {
            int64_t done = 0;
            while (done < steps) {
                if (way == 1) {
                    int ran = 0;
                    CHECK(fpde_step_block(line, &ran));
                    if (ran == 0) break;
                } else {
                    CHECK(fpde_line_run(line, 1));
                }
                CHECK(fpde_line_steps_done(line, &done));
            }
            CHECK(fpde_line_get_state(line, u.data(), 0));
        }
        int cached = -1;
        int64_t made = -1;
        CHECK(fpde_line_graph_stats(line, &cached, &made));
        fprintf(stderr, "way %d: %lld steps, graphs cached %d, instantiated %lld\n", way, (long long)steps, cached,
                (long long)made);
        CHECK(fpde_line_destroy(line));
        if (fwrite(u.data(), 8, N + 1, out) != (size_t)(N + 1)) return 1;
    }
    fclose(out);
    CHECK(fpde_ctx_destroy(ctx));
    return 0;
}

// Drop-in replay of the reference's GPU history-sum call sequence through the C ABI.
//
// fpde_hpc_1d.cpp keeps one snapshot per step in `oldH` (calc_step :5729-5745), builds the
// step's weights kb_3_cache with precalc_kb_3 (:4069-4085) and, before the K pass of every step,
// calls fr_ocl_call_sum (:1819-1883, from calc_step :5155-5158), whose results time_summing
// returns (:4100-4104). This program is that caller with fr_ocl_call_sum replaced by the
// gb300_call_sum adapter (fpde_history_append of each new snapshot, then fpde_l1_sum with the
// step's kb_3_cache): a C++ host program linked against libfpde_gb300.so, no Python in between.
//
// Input (little-endian, written by tests/test_cpp_dropin.py from the reference's recorded column
// run): int64 nodes, int64 steps; U0[nodes]; U[steps][nodes] (the grid after each step);
// tau[steps]; int64 kb_off[steps + 1]; kb_flat[kb_off[steps]] (step n's kb_3_cache is
// kb_flat[kb_off[n] .. kb_off[n + 1])).
// Output: for n = 1 .. steps - 1, the Sums of step n (nodes doubles each).
//
//     dropin_sum IN OUT [device]
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fpde_gb300.h"

namespace {

// The parts of H_solver's state the adapter touches.
struct Column {
    int device = 0;
    int64_t nodes = 0;
    std::vector<double *> oldH;          // snapshots, oldest first (the reference's oldH)
    std::vector<double> kb_3_cache, tau; // precalc_kb_3's output for the current step
    // gb300_call_sum state: the library context and the device snapshot history
    fpde_ctx *gb_ctx = nullptr;
    fpde_hist *gb_hist = nullptr;
    double *Sums = nullptr;

    int gb300_call_sum()                 // drop-in for fr_ocl_call_sum()
    {
        if (!gb_ctx) {
            if (fpde_ctx_create(device, &gb_ctx) ||
                fpde_history_create(gb_ctx, nodes, /*max_steps=*/1 << 16, FPDE_PREC_FP64, &gb_hist)) {
                fprintf(stderr, "GB300: %s\n", fpde_last_error_string());
                return 1;
            }
            Sums = new double[nodes];
            for (size_t t = 0; t < oldH.size(); t++)            // snapshots taken so far
                if (fpde_history_append(gb_hist, oldH[t], /*on_device=*/0)) return 1;
        } else if (fpde_history_append(gb_hist, oldH.back(), 0)) {   // newest snapshot -> increment
            fprintf(stderr, "GB300: %s\n", fpde_last_error_string());
            return 1;
        }
        if (fpde_l1_sum(gb_hist, kb_3_cache.data(), tau.data(), /*scale=*/1.0, Sums, 0)) {
            fprintf(stderr, "GB300: %s\n", fpde_last_error_string());
            return 1;
        }
        return 0;
    }

    ~Column()
    {
        delete[] Sums;
        if (gb_ctx) fpde_ctx_destroy(gb_ctx);
    }
};

bool read_all(FILE *f, void *p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: %s IN OUT [device]\n", argv[0]);
        return 2;
    }
    FILE *in = fopen(argv[1], "rb");
    if (!in) return 2;
    int64_t nodes = 0, steps = 0;
    if (!read_all(in, &nodes, 8) || !read_all(in, &steps, 8) || nodes <= 0 || steps < 2) return 2;
    std::vector<double> U0(nodes), U((size_t)steps * nodes), tau_all(steps);
    std::vector<int64_t> kb_off(steps + 1);
    bool ok = read_all(in, U0.data(), 8 * nodes) && read_all(in, U.data(), 8 * U.size()) &&
              read_all(in, tau_all.data(), 8 * steps) && read_all(in, kb_off.data(), 8 * (steps + 1));
    std::vector<double> kb_flat(ok ? kb_off[steps] : 0);
    ok = ok && read_all(in, kb_flat.data(), 8 * kb_flat.size());
    fclose(in);
    if (!ok) return 2;

    Column col;
    col.device = argc > 3 ? atoi(argv[3]) : 0;
    col.nodes = nodes;
    FILE *out = fopen(argv[2], "wb");
    if (!out) return 2;
    col.oldH.push_back(U0.data());                          // the initial snapshot
    for (int64_t n = 1; n < steps; ++n) {
        // calc_step of step n: the snapshots so far are U0 and the grids after steps 0 .. n-1
        col.oldH.push_back(U.data() + (size_t)(n - 1) * nodes);
        col.kb_3_cache.assign(kb_flat.begin() + kb_off[n], kb_flat.begin() + kb_off[n + 1]);
        col.tau.assign(tau_all.begin(), tau_all.begin() + n);
        if (col.gb300_call_sum()) return 1;
        if (fwrite(col.Sums, 8, nodes, out) != (size_t)nodes) return 1;
    }
    fclose(out);
    return 0;
}

// Shared host/device plumbing of libfpde_gb300: error reporting, the context object,
// device allocation tracking and a bounded grid-wide barrier for cooperative kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdarg.h>
#include <stdio.h>

#include <string>
#include <vector>
#include <set>

#include "fpde_gb300.h"

namespace fpde {

// ---------------------------------------------------------------- errors

int set_error(int code, const char *fmt, ...);
void clear_error();
void count_launches(int64_t n);

#define FPDE_CUDA(call)                                                                    \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return ::fpde::set_error(FPDE_ERR_CUDA, "%s failed: %s (%s:%d)", #call,        \
                                     cudaGetErrorString(e_), __FILE__, __LINE__);          \
    } while (0)

#define FPDE_CHECK_ARG(cond, msg)                                                          \
    do {                                                                                   \
        if (!(cond)) return ::fpde::set_error(FPDE_ERR_ARG, "%s", msg);                    \
    } while (0)

// Launch-error check after a <<<>>> launch.
#define FPDE_LAUNCHED(n)                                                                   \
    do {                                                                                   \
        cudaError_t e_ = cudaGetLastError();                                               \
        if (e_ != cudaSuccess)                                                             \
            return ::fpde::set_error(FPDE_ERR_CUDA, "kernel launch failed: %s (%s:%d)",    \
                                     cudaGetErrorString(e_), __FILE__, __LINE__);          \
        ::fpde::count_launches(n);                                                         \
    } while (0)

// Device error flags (bit set by kernels, read by the host).
enum : unsigned {
    DEVERR_BARRIER_TIMEOUT = 1u,
    DEVERR_MBAR_TIMEOUT = 2u,
    DEVERR_BAD_SHAPE = 4u,
    DEVERR_SOLVER = 8u,           // an iterative solve broke down repeatedly or ran past its time limit
};

}  // namespace fpde

// ---------------------------------------------------------------- context

struct fpde_ctx {
    int device = 0;
    int sm_count = 0;
    int cc_major = 0, cc_minor = 0;
    size_t smem_optin = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    unsigned *d_flags = nullptr;       // device error flags
    unsigned *d_barrier = nullptr;     // grid barrier state (count, generation) x 64 slots
    int *d_scratch = nullptr;          // 16 ints of per-call device scratch (one call at a time)
    std::set<fpde_hist *> hists;
    std::set<fpde_line *> lines;
    std::set<void *> extra;            // other objects registered by modules (freed by them)
};

namespace fpde {

// Make ctx's device current for the calling thread.
int ctx_enter(fpde_ctx *ctx);
// Streaming multiprocessors of the current device (queried once per device).
int device_sm_count();
// Opt kernel `fn` in to `bytes` of dynamic shared memory on the current device (the attribute is
// per device: done once per (device, kernel) and remembered).
cudaError_t smem_opt_in(const void *fn, int bytes);
// Allocate/free device memory (returns FPDE_ERR_NOMEM on failure).
int dev_alloc(void **p, size_t bytes);
void dev_free(void *p);
// Read and clear the device error flags (synchronises the context stream).
int ctx_check_flags(fpde_ctx *ctx, const char *where);

// ---------------------------------------------------------- device helpers

// Grid-wide barrier for a cooperative launch (all CTAs co-resident). state[0] is the
// arrival count, state[1] the generation. The wait is bounded: after ~2^24 polls
// (about a second) it sets DEVERR_BARRIER_TIMEOUT in *flags and returns false, and the
// caller must return without touching shared results.
__device__ __forceinline__ bool grid_barrier(unsigned *state, unsigned nblocks, unsigned *flags)
{
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = state + 1;
        unsigned gen = *vgen;
        __threadfence();
        unsigned arrived = atomicAdd(state, 1u);
        int ok = 1;
        if (arrived == nblocks - 1) {
            atomicExch(state, 0u);
            __threadfence();
            atomicAdd(state + 1, 1u);
        } else {
            unsigned polls = 0;
            while (*vgen == gen) {
                if (++polls > (1u << 24)) { atomicOr(flags, DEVERR_BARRIER_TIMEOUT); ok = 0; break; }
                if (polls > 64) __nanosleep(32);
            }
        }
        __threadfence();
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

}  // namespace fpde

// History sum that allocates nothing: fpde_l1_sum_noalloc.
//
// Some callers cannot call cudaMalloc while they run: a host framework that owns all device
// memory through its own pool and forbids plugins from allocating, a process working under a
// fixed device-memory budget agreed at start-up, or a time-step loop that must not hit the
// implicit device synchronisation of cudaMalloc/cudaFree. For them this entry point computes
// the same sum as fpde_l1_sum, but from caller-owned device buffers (increments, weights,
// result) and with its split-K partial sums in a fixed array compiled into this library.
//
// The array below is the only scratch. It lives in device global memory of every GPU that
// loads the library, until the process exits. Every call shares it and it keeps the last
// call's contents; nothing in it needs to start at zero (each call writes every partial it
// later reads). Calls whose work overlaps on the GPU (on different streams, or from
// different host threads) race on it and must be serialised by the caller.
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

namespace fpde {

// Maximum scratch: 2^20 doubles (8 MiB) of partial sums, KS splits x P row pitch.
constexpr int64_t NOALLOC_SCRATCH_DOUBLES = (int64_t)1 << 20;
static __device__ __align__(256) double g_noalloc_partials[NOALLOC_SCRATCH_DOUBLES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static double *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};
static std::mutex g_noalloc_mu;

// Device address of the scratch on the current device (resolved once per device; the host
// symbol g_noalloc_partials is not a device address and is never passed to a kernel).
static int noalloc_scratch(double **out)
{
    int dev = -1;
    FPDE_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return set_error(FPDE_ERR_UNSUPPORTED, "device index %d beyond %d", dev, NOALLOC_MAX_DEVICES);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess || !p)
            return set_error(FPDE_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed on device %d: %s", dev,
                             cudaGetErrorString(e));
        g_noalloc_ptr[dev] = (double *)p;
    }
    *out = g_noalloc_ptr[dev];
    return FPDE_OK;
}

__global__ void k_noalloc_reduce(const double *__restrict__ part, int KS, int64_t P, int64_t nodes,
                                 double *__restrict__ S)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nodes) return;
    double s = 0.0;
    for (int k = 0; k < KS; ++k) s += part[(int64_t)k * P + i];
    S[i] = s;
}

}  // namespace fpde

using namespace fpde;

extern "C" int fpde_l1_sum_noalloc(const double *D, int n, int64_t P, int64_t nodes, const double *w,
                                   double *S, void *stream)
{
    clear_error();
    FPDE_CHECK_ARG(S && nodes > 0 && n >= 0, "bad arguments");
    FPDE_CHECK_ARG(n == 0 || (D && w), "D and w are required when n > 0");
    FPDE_CHECK_ARG(P >= nodes && P % 2 == 0, "row pitch P must be even and >= nodes");
    FPDE_CHECK_ARG(((uintptr_t)D % 16) == 0, "D must be 16-byte aligned");
    if (P > NOALLOC_SCRATCH_DOUBLES)
        return set_error(FPDE_ERR_CAPACITY,
                         "fpde_l1_sum_noalloc: row pitch %lld exceeds the fixed scratch of %lld doubles "
                         "(at most %lld nodes); use fpde_l1_sum", (long long)P,
                         (long long)NOALLOC_SCRATCH_DOUBLES, (long long)NOALLOC_SCRATCH_DOUBLES);
    double *part = nullptr;
    int rc = noalloc_scratch(&part);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (n == 0) {
        FPDE_CUDA(cudaMemsetAsync(S, 0, nodes * sizeof(double), st));
        return FPDE_OK;
    }
    int KS = choose_splits(n, P);
    const int64_t fit = NOALLOC_SCRATCH_DOUBLES / P;     // splits that fit the scratch
    if (KS > fit) KS = (int)fit;
    if ((rc = launch_l1_partial(st, D, P, n, w, part, KS))) return rc;
    k_noalloc_reduce<<<(unsigned)((nodes + 255) / 256), 256, 0, st>>>(part, KS, P, nodes, S);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

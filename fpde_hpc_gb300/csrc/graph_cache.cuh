// Replay of step runs from CUDA graphs (line.cu, lod3d.cu, batch.cu).
//
// The captured work names absolute step positions (weight offsets, history rows, far-contraction
// ranges), so a graph serves one (first step, steps) run. Runs of at least GRAPH_MIN_STEPS steps
// are captured once and replayed; the instantiated graphs live in a bounded cache that evicts the
// least recently used one. Shorter runs are enqueued directly on the stream: a caller that
// advances step by step or block by block (the reference's own time loop through the drop-in
// adapter, fpde_step_block) instantiates no graph at all.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace fpde {

constexpr int GRAPH_MIN_STEPS = 128;     // shortest run replayed from a graph
constexpr size_t GRAPH_CACHE_MAX = 8;    // instantiated graphs kept per object

template <class Aux>
struct GraphCache {
    struct Entry {
        int64_t n0 = 0;
        int steps = 0;
        cudaGraphExec_t exec = nullptr;
        int64_t launches = 0;            // kernels one replay launches
        Aux aux{};                       // per-graph data of the owner (e.g. probe records)
        uint64_t stamp = 0;
    };
    std::vector<Entry> entries;
    uint64_t clock = 0;
    int64_t instantiated = 0;            // graphs instantiated over the owner's life

    void clear()
    {
        for (auto &e : entries)
            if (e.exec) cudaGraphExecDestroy(e.exec);
        entries.clear();
    }

    Entry *find(int64_t n0, int steps)
    {
        for (auto &e : entries)
            if (e.n0 == n0 && e.steps == steps) {
                e.stamp = ++clock;
                return &e;
            }
        return nullptr;
    }

    // Capture enqueue(stream, &kernels, &aux) -> status on a private stream, instantiate it and
    // keep it (evicting the least recently used graph when the cache is full).
    template <class F>
    int capture(int64_t n0, int steps, F &&enqueue, Entry **out)
    {
        cudaStream_t cs;
        FPDE_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaStreamDestroy(cs);
            return set_error(FPDE_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        }
        Entry ent;
        ent.n0 = n0;
        ent.steps = steps;
        const int64_t before = fpde_kernel_launch_count();
        const int rc = enqueue(cs, &ent.launches, &ent.aux);
        e = cudaStreamEndCapture(cs, &graph);
        count_launches(-(fpde_kernel_launch_count() - before));   // counted at each replay
        cudaStreamDestroy(cs);
        if (rc || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            if (rc) return rc;
            return set_error(FPDE_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        }
        e = cudaGraphInstantiate(&ent.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return set_error(FPDE_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
        ++instantiated;
        if (entries.size() >= GRAPH_CACHE_MAX) {
            size_t lru = 0;
            for (size_t i = 1; i < entries.size(); ++i)
                if (entries[i].stamp < entries[lru].stamp) lru = i;
            cudaGraphExecDestroy(entries[lru].exec);
            entries.erase(entries.begin() + (long)lru);
        }
        ent.stamp = ++clock;
        entries.push_back(ent);
        *out = &entries.back();
        return FPDE_OK;
    }
};

// Event record inside or outside a stream capture (inside it becomes an external event node).
inline cudaError_t record_probe_event(cudaEvent_t ev, cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    return cudaEventRecordWithFlags(ev, st, cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal
                                                                               : cudaEventRecordDefault);
}

}  // namespace fpde

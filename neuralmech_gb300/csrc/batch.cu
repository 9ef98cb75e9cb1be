// Uneven multi-model batches as one CUDA graph (wfd_batch_plan / _run / _free).
//
// A batch is a list of independent misfit gradients (wfd_misfit_gradient
// calls), each with its own problem (grid, step count, shots, tiles),
// inputs, outputs and workspace: the many-surveys-at-once FWI workload. The
// plan gives every item a stream of its own, forked from and joined to one
// capture stream, so that the models' step kernels overlap on the GPU, and
// records the whole batch as one CUDA graph; a run is one graph launch. This
// is the native form of the reference's graph replay of its step loop
// (projects/18_simple_wave_fd/2D_wave_cuda_graph.py:73-95, a captured
// sequence of padded_step launches replayed per block of steps), for whole
// gradients of several models.
#include <cstdint>
#include <cstdio>
#include <new>
#include <vector>

#include "../../include/wavefd.h"
#include "internal.h"

struct wfd_batch {
    std::vector<wfd_batch_item> items;
    std::vector<wfd_problem> problems;  // the items' problems, copied
    std::vector<cudaStream_t> streams;  // one per item
    std::vector<cudaEvent_t> joins;     // one per item
    cudaStream_t cap = nullptr;         // the capture's origin stream
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t launches = 0;  // kernels one replay launches
};

namespace {

void destroy(wfd_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (cudaEvent_t e : b->joins)
        if (e) cudaEventDestroy(e);
    for (cudaStream_t s : b->streams)
        if (s) cudaStreamDestroy(s);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->cap) cudaStreamDestroy(b->cap);
    delete b;
}

int cuda_fail(cudaError_t e, const char* what) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s failed: %s", what, cudaGetErrorString(e));
    return wfd::set_error(WFD_ERR_CUDA, buf);
}

// Every item's gradient on its own stream, forked from `origin` and joined
// back to it: eagerly, or recorded when `origin` is capturing.
int enqueue(wfd_batch* b, cudaStream_t origin) {
    cudaError_t e = cudaEventRecord(b->fork, origin);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventRecord (fork)");
    for (size_t i = 0; i < b->items.size(); ++i) {
        const wfd_batch_item& t = b->items[i];
        if ((e = cudaStreamWaitEvent(b->streams[i], b->fork, 0)) != cudaSuccess)
            return cuda_fail(e, "cudaStreamWaitEvent (fork)");
        const int rc = wfd_misfit_gradient(t.problem, t.vel, t.sponge_z, t.sponge_y, t.sponge_x, t.wavelet, t.src,
                                           t.rec, t.observed, t.traces, t.grad_vel, t.grad_wavelet, t.misfit,
                                           t.workspace, t.workspace_bytes, b->streams[i]);
        if (rc) return rc;
        if ((e = cudaEventRecord(b->joins[i], b->streams[i])) != cudaSuccess)
            return cuda_fail(e, "cudaEventRecord (join)");
        if ((e = cudaStreamWaitEvent(origin, b->joins[i], 0)) != cudaSuccess)
            return cuda_fail(e, "cudaStreamWaitEvent (join)");
    }
    return WFD_OK;
}

}  // namespace

int wfd_batch_plan(const wfd_batch_item* items, int count, void* stream, wfd_batch** out) {
    if (!out) return wfd::set_error(WFD_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!items || count < 1) return wfd::set_error(WFD_ERR_INVALID, "a batch needs at least one item");
    for (int i = 0; i < count; ++i)
        if (!items[i].problem) return wfd::set_error(WFD_ERR_INVALID, "a batch item has no problem");
    wfd_batch* b = new (std::nothrow) wfd_batch();
    if (!b) return wfd::set_error(WFD_ERR_INVALID, "out of host memory");
    b->items.assign(items, items + count);
    b->problems.resize(count);
    for (int i = 0; i < count; ++i) {
        b->problems[i] = *items[i].problem;
        b->items[i].problem = &b->problems[i];
    }
    b->streams.assign(count, nullptr);
    b->joins.assign(count, nullptr);
    cudaError_t e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int i = 0; i < count && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&b->streams[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        const int rc = cuda_fail(e, "stream / event creation");
        destroy(b);
        return rc;
    }
    // eager run on `stream` (argument checks, kernel attributes), then the capture
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = enqueue(b, s);
    if (!rc && (e = cudaStreamSynchronize(s)) != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize");
    if (rc) {
        destroy(b);
        return rc;
    }
    const uint64_t n0 = wfd_kernel_launches();
    if ((e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
        rc = cuda_fail(e, "cudaStreamBeginCapture");
        destroy(b);
        return rc;
    }
    rc = enqueue(b, b->cap);
    e = cudaStreamEndCapture(b->cap, &b->graph);  // (ends the capture whatever happened in it)
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "cudaStreamEndCapture");
    if (!rc && (e = cudaGraphInstantiate(&b->exec, b->graph, 0)) != cudaSuccess)
        rc = cuda_fail(e, "cudaGraphInstantiate");
    if (rc) {
        destroy(b);
        return rc;
    }
    b->launches = wfd_kernel_launches() - n0;
    *out = b;
    return WFD_OK;
}

int wfd_batch_run(wfd_batch* batch, void* stream) {
    if (!batch || !batch->exec) return wfd::set_error(WFD_ERR_INVALID, "batch is NULL");
    const cudaError_t e = cudaGraphLaunch(batch->exec, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
    wfd::count_launch(int(batch->launches));
    return WFD_OK;
}

uint64_t wfd_batch_launches(const wfd_batch* batch) { return batch ? batch->launches : 0; }

int wfd_batch_free(wfd_batch* batch) {
    destroy(batch);
    return WFD_OK;
}

// Host-side runtime of the C ABI: the handle (one device, one stream, owned
// device buffers), CUDA error capture and launch accounting.  The reference's
// counterpart is its RAII wrapper algcuda::device::Memory<T> plus
// throw_if_cuda_error (algcuda/cuda-cpp-wrapper/include/algcuda/memory.hpp:
// 39-110, error.hpp:84-98); here errors become status codes.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/circlecover_gb300.h"

struct cc_handle {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    uint64_t launches = 0;
    std::atomic<int> interrupt{0};

    // growable device scratch buffers, keyed by purpose
    struct Buf {
        void* ptr = nullptr;
        size_t bytes = 0;
    };
    Buf bufs[48];
    // pinned host staging for the host-memory entry points
    void* pinned = nullptr;
    size_t pinned_bytes = 0;
    // evaluation passes' register budget and grid (blocks per SM), set by cc_autotune_eval
    // (the certification and repair passes, 4 and 5, keep the defaults)
    int tune_minb[CC_EVAL_STAGES] = {1, 1, 1, 1, 1, 1};
    int tune_grid[CC_EVAL_STAGES] = {8, 8, 8, 8, 8, 8};
    // FP64 certification of the evaluation's FP32 decisions (cc_set_eval_certify)
    bool eval_certify = true;
    // how cc_tight_refine decides a level's boxes (cc_set_refine_order)
    int refine_order = CC_REFINE_MASKS;
    // where the tight proof writes its state after each generation (empty: off)
    std::string checkpoint_path;
    // sample of r3 cells logged by the last tight proof (CC_PROVE_LOG_CELLS)
    std::vector<cc_tight_box> cell_log;
    int cell_log_splits = 0;
    // learned-ordering network (cc_mlp_*), owned by the handle
    void* mlp = nullptr;
    void (*mlp_free)(cc_handle*) = nullptr;
    // per-stage events of the evaluation (cc_set_stage_timing)
    bool timing = false;
    cudaEvent_t stage_ev[CC_EVAL_STAGES + 1] = {};
    int stages_recorded = 0;
    // queue counters of the last evaluation batch (device memory)
    unsigned long long* eval_counts = nullptr;
    // kernels may read and write ordinary (pageable) host memory
    // (cudaDevAttrPageableMemoryAccess, e.g. over NVLink-C2C with the host's
    // page tables); CC_HOST_STAGING=1 in the environment turns this off
    bool pageable_access = false;
    // second stream for transfers that overlap evaluation (created on first use)
    cudaStream_t stream2 = nullptr;
    // CUDA graph of the evaluation's launch sequence (cc_set_eval_graph):
    // replayed while its key (every pointer, size and setting the launches
    // take) repeats, re-captured into the same executable graph otherwise
    bool eval_graph = true;
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<uintptr_t> graph_key;
    uint64_t graph_launches = 0;  // kernels in the captured sequence
    uint64_t graph_captures = 0, graph_replays = 0;
};

namespace ccrt {

inline int fail(cc_handle* h, int status, const char* what, cudaError_t e = cudaSuccess) {
    if (h) {
        h->last_error = what;
        if (e != cudaSuccess) {
            h->last_error += ": ";
            h->last_error += cudaGetErrorString(e);
        }
    }
    return status;
}

#define CC_CUDA(h, call)                                                              \
    do {                                                                              \
        cudaError_t cc_e_ = (call);                                                   \
        if (cc_e_ != cudaSuccess) return ccrt::fail((h), CC_ERR_CUDA, #call, cc_e_); \
    } while (0)

#define CC_LAUNCHED(h)                                                                  \
    do {                                                                                \
        cudaError_t cc_e_ = cudaGetLastError();                                         \
        if (cc_e_ != cudaSuccess) return ccrt::fail((h), CC_ERR_CUDA, "launch", cc_e_); \
        (h)->launches += 1;                                                             \
    } while (0)

// two CUDA events, destroyed on every return path
struct EventPair {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    EventPair() = default;
    EventPair(const EventPair&) = delete;
    EventPair& operator=(const EventPair&) = delete;
    ~EventPair() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    }
};

// grow-only device buffer; contents are not preserved
inline int ensure(cc_handle* h, int slot, size_t bytes, void** out) {
    cc_handle::Buf& b = h->bufs[slot];
    if (b.bytes < bytes) {
        if (b.ptr) {
            cudaFree(b.ptr);
            b.ptr = nullptr;
            b.bytes = 0;
        }
        size_t want = bytes + bytes / 4 + 4096;
        cudaError_t e = cudaMalloc(&b.ptr, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(h, CC_ERR_OOM, "cudaMalloc", e);
        }
        b.bytes = want;
    }
    *out = b.ptr;
    return CC_OK;
}

inline int ensure_pinned(cc_handle* h, size_t bytes) {
    if (h->pinned_bytes < bytes) {
        if (h->pinned) cudaFreeHost(h->pinned);
        h->pinned = nullptr;
        h->pinned_bytes = 0;
        cudaError_t e = cudaMallocHost(&h->pinned, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(h, CC_ERR_OOM, "cudaMallocHost", e);
        }
        h->pinned_bytes = bytes;
    }
    return CC_OK;
}

// Host-side parallel loop over [0, n) in contiguous blocks, for the staging
// copies of the host-memory entry points (one thread streams memory at a
// fraction of what the host's memory system delivers).  Small ranges run on
// the calling thread.
template <class F>
inline void parallel_blocks(size_t n, F f) {
    unsigned t = std::thread::hardware_concurrency();
    t = t < 1 ? 1 : (t > 16 ? 16 : t);
    if (n < ((size_t)1 << 16) || t == 1) {
        f((size_t)0, n);
        return;
    }
    std::vector<std::thread> pool;
    const size_t per = (n + t - 1) / t;
    for (unsigned k = 1; k < t; ++k) {
        size_t lo = k * per, hi = lo + per < n ? lo + per : n;
        if (lo < hi) pool.emplace_back(f, lo, hi);
    }
    f((size_t)0, per < n ? per : n);
    for (auto& th : pool) th.join();
}

}  // namespace ccrt

// Size-bound criteria on the GPU (sm_103a): per-box verdict masks
// (cc_sb_eval, cc_sb_eval_device).
//
// Per-box cost differs by three orders of magnitude between the criteria
// (the seven-disk strategies alone reach 10^6 directed-rounding operations on
// some boxes), so instead of one kernel running the whole cascade per thread
// every criterion is its own grid-stride kernel over all boxes: a warp then
// runs one criterion on 32 boxes and only diverges inside it.  The masks are
// OR-ed in place; the launches are stream-ordered.
#include <cuda_runtime.h>

#include <cstring>

#include "cc_runtime.cuh"
#include "cc_sb_eval.cuh"

using cc::Iv;
namespace sb = cc::sb;

namespace {

enum class Layout { AoS, SoA };

template <Layout L>
__device__ __forceinline__ sb::Box6 load_box6(const double* __restrict__ in, size_t n, size_t i) {
    double v[14];
    if (L == Layout::SoA) {
#pragma unroll
        for (int k = 0; k < 14; ++k) v[k] = __ldg(in + (size_t)k * n + i);
    } else {
        const double2* p = reinterpret_cast<const double2*>(in + i * 14);
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            double2 t = __ldg(p + k);
            v[2 * k] = t.x;
            v[2 * k + 1] = t.y;
        }
    }
    sb::Box6 b;
    b.la = Iv{v[0], v[1]};
#pragma unroll
    for (int k = 0; k < 6; ++k) b.r[k] = Iv{v[2 + 2 * k], v[3 + 2 * k]};
    return b;
}

// shortcuts (bits 15..19) and the empty flag (bit 14); writes the mask
template <Layout L>
__global__ void __launch_bounds__(128) k_sb_prefix(const double* __restrict__ in, size_t n, uint32_t* __restrict__ masks) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const sb::Box6 raw = load_box6<L>(in, n, i);
        uint32_t m = 0;
        bool any_trap = false;
        for (int k = 15; k <= 19; ++k) {
            cc::trap_clear();
            if (sb::trap_free(sb::sb_shortcut(k, raw.la, raw.r[0], raw.r[1], raw.r[2]), any_trap)) m |= 1u << k;
        }
        const sb::Box6 b = sb::tightened(raw);
        if (sb::box_empty(b) || cc::empty(sb::remaining_weight(b))) m |= 1u << 14;
        if (any_trap) m |= 1u << 31;
        masks[i] = m;
    }
}

// criterion K on every box; ORs bit K (and the trap bit) into the mask
template <Layout L, int K>
__global__ void __launch_bounds__(128) k_sb_criterion(const double* __restrict__ in, size_t n, uint32_t* __restrict__ masks) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const sb::Box6 b = sb::tightened(load_box6<L>(in, n, i));
        sb::Vals v;
        v.R = sb::remaining_weight(b);
        cc::trap_clear();
        bool any_trap = false;
        bool ok = sb::trap_free(sb::sb_criterion(K, b, v), any_trap);
        uint32_t m = (ok ? (1u << K) : 0u) | (any_trap ? (1u << 31) : 0u);
        if (m) masks[i] |= m;
    }
}

template <Layout L, int K>
int launch_criteria(cc_handle* h, const double* in, size_t n, uint32_t* masks, cudaStream_t s, int g) {
    if constexpr (K < sb::SB_NUM_CRITERIA) {
        k_sb_criterion<L, K><<<g, 128, 0, s>>>(in, n, masks);
        CC_LAUNCHED(h);
        return launch_criteria<L, K + 1>(h, in, n, masks, s, g);
    }
    return CC_OK;
}

template <Layout L>
int sb_eval_batch(cc_handle* h, const double* in, size_t n, uint32_t* masks, cudaStream_t s) {
    size_t want = (n + 127) / 128;
    size_t cap = (size_t)h->sm_count * 8;
    const int g = (int)(want < cap ? (want ? want : 1) : cap);
    k_sb_prefix<L><<<g, 128, 0, s>>>(in, n, masks);
    CC_LAUNCHED(h);
    return launch_criteria<L, 0>(h, in, n, masks, s, g);
}

}  // namespace

extern "C" int cc_sb_eval_device(cc_handle* h, const double* soa, size_t n, uint32_t* masks, void* stream) {
    if (!h || (n && (!soa || !masks))) return CC_ERR_PARAM;
    h->launches = 0;
    if (n == 0) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    return sb_eval_batch<Layout::SoA>(h, soa, n, masks, stream ? (cudaStream_t)stream : h->stream);
}

extern "C" int cc_sb_eval(cc_handle* h, const cc_sb_box* boxes, size_t n, uint32_t* masks) {
    if (!h || (n && (!boxes || !masks))) return CC_ERR_PARAM;
    h->launches = 0;
    if (n == 0) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    const size_t chunk = n < ((size_t)1 << 20) ? n : ((size_t)1 << 20);
    void *d_in, *d_out;
    int st = ccrt::ensure(h, 21, chunk * sizeof(cc_sb_box), &d_in);
    if (!st) st = ccrt::ensure(h, 22, chunk * sizeof(uint32_t), &d_out);
    if (st) return st;
    for (size_t off = 0; off < n; off += chunk) {
        size_t cnt = n - off < chunk ? n - off : chunk;
        CC_CUDA(h, cudaMemcpyAsync(d_in, boxes + off, cnt * sizeof(cc_sb_box), cudaMemcpyHostToDevice, h->stream));
        st = sb_eval_batch<Layout::AoS>(h, (const double*)d_in, cnt, (uint32_t*)d_out, h->stream);
        if (st) return st;
        CC_CUDA(h, cudaMemcpyAsync(masks + off, d_out, cnt * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
        CC_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    return CC_OK;
}

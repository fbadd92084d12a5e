// Learned strategy ordering for the tight criteria: a 10 -> 64 -> 64 -> 7
// multilayer perceptron that predicts, per box, which of the six exported
// tight criteria will certify it (six logits) and whether none will (the
// "split" logit: the box is critical and must be bisected).
//
// * Training runs on the GPU with the kernels below (no library): a fused
//   forward/backward kernel per block of 128 samples writes per-block
//   gradient partials, a second kernel reduces them and applies an Adam
//   step.  FP32 master weights.  The records are (box, criterion, verdict)
//   triples from the plain evaluation (cc_tight_eval).
// * Inference runs the network with BF16 weights and activations and FP32
//   accumulation on the tensor cores (warp-level mma.sync m16n8k16: the
//   layers are 16..64 columns wide, so one warp owns a 16-box tile through
//   all three layers and the accumulators of one layer become the next
//   layer's operands without leaving registers).
// * Use: cc_tight_first evaluates boxes until the first criterion certifies
//   them ("first success", the proof's question), either in the plain order
//   (the reference's nesting: r1, r1+r2, r1+r2+r3, R empty, 2x2, r1+r2+r3
//   leaf, gaps) or with the network's most likely criterion tried first and
//   the plain order as the fallback.  Every certification is the FP64
//   criterion itself; the order changes which criteria run, never whether a
//   box counts as certified (criticals are the boxes no criterion
//   certifies, in either order).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "cc_mlp.cuh"
#include "cc_runtime.cuh"
#include "cc_tight.cuh"

using cc::Iv;
namespace ct = cc::tight;

namespace {

constexpr int kF = 10, kH = 64, kO = 7;
constexpr int P_W1 = 0, P_B1 = P_W1 + kF * kH, P_W2 = P_B1 + kH, P_B2 = P_W2 + kH * kH, P_W3 = P_B2 + kH,
              P_B3 = P_W3 + kH * kO, P_N = P_B3 + kO;
static_assert(P_N == CC_MLP_PARAMS, "parameter count");
constexpr int kTrainBlock = 128;   // samples per block of the gradient kernel
constexpr int kPartBlocks = 512;   // blocks per gradient launch at most
constexpr int kStride = kH + 1;    // padded activation rows (no shared-memory bank conflicts)
// fragments of the BF16 weights for mma.m16n8k16: layer 1 (1 k-step x 8
// n-tiles), layer 2 (4 x 8), layer 3 (4 x 1), 32 lanes each
constexpr int FR_L1 = 0, FR_L2 = FR_L1 + 1 * 8 * 32, FR_L3 = FR_L2 + 4 * 8 * 32, FR_N = FR_L3 + 4 * 1 * 32;

struct MlpState {
    float* w = nullptr;     // master weights
    float* m = nullptr;     // Adam first moments
    float* v = nullptr;     // Adam second moments
    float* part = nullptr;  // kPartBlocks x P_N gradient partials
    float* loss = nullptr;  // kPartBlocks loss partials
    float* grad = nullptr;  // reduced gradient (for inspection)
    uint2* frag = nullptr;  // BF16 weight fragments
    float* bias = nullptr;  // biases padded: b1[64], b2[64], b3[8]
    int steps = 0;
    bool packed = false;
};

void mlp_free(cc_handle* h) {
    MlpState* s = static_cast<MlpState*>(h->mlp);
    if (!s) return;
    for (void* p : {(void*)s->w, (void*)s->m, (void*)s->v, (void*)s->part, (void*)s->loss, (void*)s->grad,
                    (void*)s->frag, (void*)s->bias})
        if (p) cudaFree(p);
    delete s;
    h->mlp = nullptr;
}

int mlp_state(cc_handle* h, MlpState** out) {
    if (h->mlp) {
        *out = static_cast<MlpState*>(h->mlp);
        return CC_OK;
    }
    MlpState* s = new MlpState();
    cudaError_t e = cudaSuccess;
    e = e ? e : cudaMalloc(&s->w, P_N * sizeof(float));
    e = e ? e : cudaMalloc(&s->m, P_N * sizeof(float));
    e = e ? e : cudaMalloc(&s->v, P_N * sizeof(float));
    e = e ? e : cudaMalloc(&s->grad, P_N * sizeof(float));
    e = e ? e : cudaMalloc(&s->part, (size_t)kPartBlocks * P_N * sizeof(float));
    e = e ? e : cudaMalloc(&s->loss, kPartBlocks * sizeof(float));
    e = e ? e : cudaMalloc(&s->frag, FR_N * sizeof(uint2));
    e = e ? e : cudaMalloc(&s->bias, (kH + kH + 8) * sizeof(float));
    h->mlp = s;
    h->mlp_free = mlp_free;
    if (e != cudaSuccess) {
        cudaGetLastError();
        mlp_free(h);
        return ccrt::fail(h, CC_ERR_OOM, "cc_mlp: cudaMalloc", e);
    }
    *out = s;
    return CC_OK;
}

// ---------------------------------------------------------------- features
__device__ void box_features(const double* __restrict__ soa, size_t n, size_t i, float depth, float* f) {
    double v[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) v[k] = soa[(size_t)k * n + i];
    cc::mlp::features(v, ct::required_weight_for(Iv{v[0], v[1]}), depth, f);
}

__global__ void k_mlp_features(const double* __restrict__ soa, size_t n, float depth, float* __restrict__ feat) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float f[kF];
        box_features(soa, n, i, depth, f);
#pragma unroll
        for (int k = 0; k < kF; ++k) feat[i * kF + k] = f[k];
    }
}

// ---------------------------------------------------------------- training
// One block = 128 samples, one thread per sample for the forward pass and
// the per-sample backward quantities; the weight gradients are sums over
// the block's samples, one thread per weight.  Loss: mean over samples of
// the summed binary cross-entropies of the 7 outputs.
__global__ void __launch_bounds__(kTrainBlock) k_mlp_grad(const float* __restrict__ w, const float* __restrict__ feat,
                                                         const uint32_t* __restrict__ labels, size_t n, size_t off,
                                                         float inv_total, float* __restrict__ part,
                                                         float* __restrict__ loss_part) {
    extern __shared__ float sm[];
    float* sw = sm;                                // P_N
    float* sx = sw + ((P_N + 3) & ~3);             // 128 x kF
    float* sh1 = sx + kTrainBlock * kF;            // 128 x kStride: h1, later dh1
    float* sh2 = sh1 + kTrainBlock * kStride;      // 128 x kStride: h2, later dh2
    float* sdz = sh2 + kTrainBlock * kStride;      // 128 x 8
    float* sred = sdz + kTrainBlock * 8;           // 128 (loss reduction)
    const int t = threadIdx.x;
    for (int i = t; i < P_N; i += kTrainBlock) sw[i] = w[i];
    const size_t s_idx = off + (size_t)blockIdx.x * kTrainBlock + t;
    const bool valid = s_idx < n;
    for (int f = 0; f < kF; ++f) sx[t * kF + f] = valid ? feat[s_idx * kF + f] : 0.0f;
    __syncthreads();
    float* h1 = sh1 + t * kStride;
    float* h2 = sh2 + t * kStride;
    for (int j = 0; j < kH; ++j) {
        float a = sw[P_B1 + j];
        for (int f = 0; f < kF; ++f) a = fmaf(sx[t * kF + f], sw[P_W1 + f * kH + j], a);
        h1[j] = a > 0.0f ? a : 0.0f;
    }
    for (int j = 0; j < kH; ++j) {
        float a = sw[P_B2 + j];
        for (int i = 0; i < kH; ++i) a = fmaf(h1[i], sw[P_W2 + i * kH + j], a);
        h2[j] = a > 0.0f ? a : 0.0f;
    }
    const uint32_t y = valid ? labels[s_idx] : 0u;
    float loss = 0.0f;
    for (int k = 0; k < kO; ++k) {
        float z = sw[P_B3 + k];
        for (int j = 0; j < kH; ++j) z = fmaf(h2[j], sw[P_W3 + j * kO + k], z);
        const float yk = (float)((y >> k) & 1u);
        const float p = 1.0f / (1.0f + expf(-z));
        if (valid) loss += fmaxf(z, 0.0f) - z * yk + log1pf(expf(-fabsf(z)));
        sdz[t * 8 + k] = valid ? (p - yk) * inv_total : 0.0f;
    }
    sred[t] = loss;
    __syncthreads();
    float* g = part + (size_t)blockIdx.x * P_N;
    // layer 3
    for (int e = t; e < kH * kO; e += kTrainBlock) {
        const int j = e / kO, k = e % kO;
        float a = 0.0f;
        for (int s = 0; s < kTrainBlock; ++s) a = fmaf(sh2[s * kStride + j], sdz[s * 8 + k], a);
        g[P_W3 + e] = a;
    }
    if (t < kO) {
        float a = 0.0f;
        for (int s = 0; s < kTrainBlock; ++s) a += sdz[s * 8 + t];
        g[P_B3 + t] = a;
    }
    if (t == 0) {
        float a = 0.0f;
        for (int s = 0; s < kTrainBlock; ++s) a += sred[s];
        loss_part[blockIdx.x] = a;
    }
    __syncthreads();
    // dh2 = dz W3^T masked by relu (in place)
    for (int j = 0; j < kH; ++j) {
        float d = 0.0f;
        for (int k = 0; k < kO; ++k) d = fmaf(sdz[t * 8 + k], sw[P_W3 + j * kO + k], d);
        h2[j] = h2[j] > 0.0f ? d : 0.0f;
    }
    __syncthreads();
    // layer 2
    for (int e = t; e < kH * kH; e += kTrainBlock) {
        const int i = e / kH, j = e % kH;
        float a = 0.0f;
        for (int s = 0; s < kTrainBlock; ++s) a = fmaf(sh1[s * kStride + i], sh2[s * kStride + j], a);
        g[P_W2 + e] = a;
    }
    if (t < kH) {
        float a = 0.0f;
        for (int s = 0; s < kTrainBlock; ++s) a += sh2[s * kStride + t];
        g[P_B2 + t] = a;
    }
    __syncthreads();
    // dh1 = dh2 W2^T masked by relu (in place)
    for (int i = 0; i < kH; ++i) {
        float d = 0.0f;
        for (int j = 0; j < kH; ++j) d = fmaf(h2[j], sw[P_W2 + i * kH + j], d);
        h1[i] = h1[i] > 0.0f ? d : 0.0f;
    }
    __syncthreads();
    // layer 1
    for (int e = t; e < kF * kH; e += kTrainBlock) {
        const int f = e / kH, i = e % kH;
        float a = 0.0f;
        for (int s = 0; s < kTrainBlock; ++s) a = fmaf(sx[s * kF + f], sh1[s * kStride + i], a);
        g[P_W1 + e] = a;
    }
    if (t < kH) {
        float a = 0.0f;
        for (int s = 0; s < kTrainBlock; ++s) a += sh1[s * kStride + t];
        g[P_B1 + t] = a;
    }
}

constexpr size_t kGradSmem = (size_t)(((P_N + 3) & ~3) + kTrainBlock * kF + 2 * kTrainBlock * kStride +
                                      kTrainBlock * 8 + kTrainBlock) * sizeof(float);

// sum of the partials (fixed order: deterministic), then optionally one Adam step
__global__ void k_mlp_reduce_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                                  const float* __restrict__ part, int blocks, float* __restrict__ grad, float lr,
                                  float b1t, float b2t, int update) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P_N) return;
    float gsum = 0.0f;
    for (int b = 0; b < blocks; ++b) gsum += part[(size_t)b * P_N + p];
    grad[p] = gsum;
    if (!update) return;
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    const float mm = beta1 * m[p] + (1.0f - beta1) * gsum;
    const float vv = beta2 * v[p] + (1.0f - beta2) * gsum * gsum;
    m[p] = mm;
    v[p] = vv;
    w[p] -= lr * (mm / (1.0f - b1t)) / (sqrtf(vv / (1.0f - b2t)) + eps);
}

// ---------------------------------------------------------------- inference
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const uint32_t a = __bfloat16_as_ushort(__float2bfloat16_rn(lo));
    const uint32_t b = __bfloat16_as_ushort(__float2bfloat16_rn(hi));
    return a | (b << 16);
}

// B fragments of a K x N weight matrix (row k = input, column n = output)
// for mma.m16n8k16 .bf16: lane (g, q) = (lane / 4, lane % 4) holds
// {W[16s+2q][8t+g], W[16s+2q+1][8t+g]} and {W[16s+2q+8][8t+g], W[16s+2q+9][8t+g]}
__device__ float wat(const float* w, int off, int K, int N, int k, int n) {
    return (k < K && n < N) ? w[off + k * N + n] : 0.0f;
}

__global__ void k_mlp_pack(const float* __restrict__ w, uint2* __restrict__ frag, float* __restrict__ bias) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < FR_N) {
        int layer, rel, K, N, NT, off;
        if (idx < FR_L2) layer = 1, rel = idx - FR_L1, K = kF, N = kH, NT = 8, off = P_W1;
        else if (idx < FR_L3) layer = 2, rel = idx - FR_L2, K = kH, N = kH, NT = 8, off = P_W2;
        else layer = 3, rel = idx - FR_L3, K = kH, N = kO, NT = 1, off = P_W3;
        (void)layer;
        const int lane = rel % 32, tile = rel / 32, s = tile / NT, t = tile % NT;
        const int g = lane >> 2, q = lane & 3, k = 16 * s + 2 * q, nn = 8 * t + g;
        frag[idx] = make_uint2(pack_bf16(wat(w, off, K, N, k, nn), wat(w, off, K, N, k + 1, nn)),
                               pack_bf16(wat(w, off, K, N, k + 8, nn), wat(w, off, K, N, k + 9, nn)));
    }
    if (idx < kH) {
        bias[idx] = w[P_B1 + idx];
        bias[kH + idx] = w[P_B2 + idx];
    }
    if (idx < 8) bias[2 * kH + idx] = idx < kO ? w[P_B3 + idx] : 0.0f;
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint2 b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

__device__ __forceinline__ float relu(float x) { return x > 0.0f ? x : 0.0f; }

// one warp per 16-box tile: features (16 x 16, 10 used) -> 64 -> 64 -> 8 logits
// (7 used); logits[i * 8 + k]
__global__ void __launch_bounds__(128) k_mlp_infer(const uint2* __restrict__ frag, const float* __restrict__ bias,
                                                   const float* __restrict__ feat, size_t n_arg,
                                                   const unsigned long long* n_dev, float* __restrict__ logits) {
    const size_t n = n_dev ? (*n_dev < n_arg ? *n_dev : n_arg) : n_arg;
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const size_t warps = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t tile = warp; tile * 16 < n; tile += warps) {
        const size_t r0 = tile * 16 + g, r1 = r0 + 8;
        auto x = [&](size_t r, int c) { return (r < n && c < kF) ? feat[r * kF + c] : 0.0f; };
        uint32_t a[4] = {pack_bf16(x(r0, 2 * q), x(r0, 2 * q + 1)), pack_bf16(x(r1, 2 * q), x(r1, 2 * q + 1)),
                         pack_bf16(x(r0, 2 * q + 8), x(r0, 2 * q + 9)), pack_bf16(x(r1, 2 * q + 8), x(r1, 2 * q + 9))};
        float c1[8][4];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            c1[t][0] = c1[t][2] = bias[8 * t + 2 * q];
            c1[t][1] = c1[t][3] = bias[8 * t + 2 * q + 1];
            mma_bf16(c1[t], a, frag[FR_L1 + t * 32 + lane]);
        }
        float c2[8][4];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            c2[t][0] = c2[t][2] = bias[kH + 8 * t + 2 * q];
            c2[t][1] = c2[t][3] = bias[kH + 8 * t + 2 * q + 1];
        }
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const uint32_t a2[4] = {pack_bf16(relu(c1[2 * s][0]), relu(c1[2 * s][1])),
                                    pack_bf16(relu(c1[2 * s][2]), relu(c1[2 * s][3])),
                                    pack_bf16(relu(c1[2 * s + 1][0]), relu(c1[2 * s + 1][1])),
                                    pack_bf16(relu(c1[2 * s + 1][2]), relu(c1[2 * s + 1][3]))};
#pragma unroll
            for (int t = 0; t < 8; ++t) mma_bf16(c2[t], a2, frag[FR_L2 + (s * 8 + t) * 32 + lane]);
        }
        float c3[4];
        c3[0] = c3[2] = bias[2 * kH + 2 * q];
        c3[1] = c3[3] = bias[2 * kH + 2 * q + 1];
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const uint32_t a3[4] = {pack_bf16(relu(c2[2 * s][0]), relu(c2[2 * s][1])),
                                    pack_bf16(relu(c2[2 * s][2]), relu(c2[2 * s][3])),
                                    pack_bf16(relu(c2[2 * s + 1][0]), relu(c2[2 * s + 1][1])),
                                    pack_bf16(relu(c2[2 * s + 1][2]), relu(c2[2 * s + 1][3]))};
            mma_bf16(c3, a3, frag[FR_L3 + s * 32 + lane]);
        }
        if (r0 < n) {
            logits[r0 * 8 + 2 * q] = c3[0];
            logits[r0 * 8 + 2 * q + 1] = c3[1];
        }
        if (r1 < n) {
            logits[r1 * 8 + 2 * q] = c3[2];
            logits[r1 * 8 + 2 * q + 1] = c3[3];
        }
    }
}

// ---------------------------------------------------------------- first success
struct LeafArgs {
    Iv la, weight;
    Iv r[4];
    ct::Box v;
    Iv R, R4;
};

__device__ LeafArgs leaf_args(const double* __restrict__ soa, size_t n, size_t i) {
    LeafArgs a;
    a.la = Iv{soa[i], soa[n + i]};
#pragma unroll
    for (int k = 0; k < 4; ++k) a.r[k] = Iv{soa[(2 + 2 * k) * n + i], soa[(3 + 2 * k) * n + i]};
    a.weight = ct::required_weight_for(a.la);
    // the leaf's quantities as the reference computes them (tight_rectangle.cu:223-238)
    a.R4 = a.weight - a.r[0] - a.r[1] - a.r[2];
    cc::tighten_lb(a.R4, 0.0);
    a.v = ct::Box{a.la, {a.r[0], a.r[1], a.r[2], a.r[3]}};
    cc::tighten_lb(a.v.r[2], a.v.r[3].lo);
    cc::tighten_lb(a.v.r[1], a.v.r[2].lo);
    cc::tighten_lb(a.v.r[0], a.v.r[1].lo);
    a.R = a.weight - a.v.r[0] - a.v.r[1] - a.v.r[2] - a.v.r[3];
    cc::tighten_lb(a.R, 0.0);
    return a;
}

// criterion k (CC_TV_* bit order) at the leaf arguments; 6 = R or R4 empty
// (one out-of-line copy: called from a loop whose order varies per box)
__device__ __noinline__ bool tight_criterion(int k, const LeafArgs& a) {
    switch (k) {
        case 0: return ct::r1_strategies(a.la, a.weight, a.r[0], a.r[1].hi);
        case 1: return ct::r1_r2_strategies(a.la, a.weight, a.r[0], a.r[1], a.r[2].hi);
        case 2: return ct::r1_r2_r3_strategies(a.la, a.weight, a.r[0], a.r[1], a.r[2], a.r[3].hi);
        case 3: return ct::two_by_two_strategies(a.v, a.R);
        case 4: return ct::r1_r2_r3_strategies(a.v, a.R4);
        case 5: return ct::r1_r2_large_r3_r4_gaps_strategy(a.v, a.R);
        case 6: return cc::empty(a.R4) || cc::empty(a.R);
    }
    return false;
}

// the reference's nesting: r1 cell, r2 cell, r3 cell, R4/R empty, leaf criteria
__constant__ int kPlainOrder[7] = {0, 1, 2, 6, 3, 4, 5};

// outcome: the step that decided (0..5 a criterion, 6 R empty, 7 none: the
// box is critical), | 0x80 if a trap site was reached on the way; evals =
// how many steps ran
__global__ void __launch_bounds__(128) k_tight_first(const double* __restrict__ soa, size_t n,
                                                     const float* __restrict__ logits, uint8_t* __restrict__ outcome,
                                                     uint8_t* __restrict__ evals) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const LeafArgs a = leaf_args(soa, n, i);
        int first = -1;
        if (logits) {  // the network's most likely criterion first
            float best = -INFINITY;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const float z = logits[i * 8 + k];
                if (z > best) best = z, first = k;
            }
        }
        cc::trap_clear();
        int decided = 7, ran = 0;
        if (first >= 0) {
            ++ran;
            if (tight_criterion(first, a)) decided = first;
        }
#pragma unroll 1
        for (int s = 0; s < 7 && decided == 7; ++s) {
            const int k = kPlainOrder[s];
            if (k == first) continue;
            ++ran;
            if (tight_criterion(k, a)) decided = k;
        }
        const bool trapped = cc::trap_status() != cc::TRAP_NONE;
        cc::trap_clear();
        outcome[i] = (uint8_t)(decided | (trapped ? 0x80 : 0));
        if (evals) evals[i] = (uint8_t)ran;
    }
}

int grid_for(cc_handle* h, size_t n, int threads) {
    size_t want = (n + threads - 1) / threads, cap = (size_t)h->sm_count * 16;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace

// ---------------------------------------------------------------- C ABI
extern "C" int cc_mlp_init(cc_handle* h, uint64_t seed) {
    if (!h) return CC_ERR_PARAM;
    CC_CUDA(h, cudaSetDevice(h->device));
    MlpState* s;
    int st = mlp_state(h, &s);
    if (st) return st;
    // He initialisation from a counter-based generator (splitmix64 + Box-Muller)
    std::vector<float> w(P_N, 0.0f);
    auto mix = [](uint64_t x) {
        x += 0x9e3779b97f4a7c15ULL;
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
        return x ^ (x >> 31);
    };
    auto normal = [&](uint64_t k) {
        const double u1 = ((mix(seed * 0x100000001b3ULL + 2 * k) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        const double u2 = ((mix(seed * 0x100000001b3ULL + 2 * k + 1) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    };
    for (int i = 0; i < kF * kH; ++i) w[P_W1 + i] = (float)(normal(i) * std::sqrt(2.0 / kF));
    for (int i = 0; i < kH * kH; ++i) w[P_W2 + i] = (float)(normal(10000 + i) * std::sqrt(2.0 / kH));
    for (int i = 0; i < kH * kO; ++i) w[P_W3 + i] = (float)(normal(20000 + i) * std::sqrt(1.0 / kH));
    CC_CUDA(h, cudaMemcpyAsync(s->w, w.data(), P_N * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CC_CUDA(h, cudaMemsetAsync(s->m, 0, P_N * sizeof(float), h->stream));
    CC_CUDA(h, cudaMemsetAsync(s->v, 0, P_N * sizeof(float), h->stream));
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    s->steps = 0;
    s->packed = false;
    return CC_OK;
}

extern "C" int cc_mlp_set_weights(cc_handle* h, const float* w) {
    if (!h || !w) return CC_ERR_PARAM;
    CC_CUDA(h, cudaSetDevice(h->device));
    MlpState* s;
    int st = mlp_state(h, &s);
    if (st) return st;
    CC_CUDA(h, cudaMemcpyAsync(s->w, w, P_N * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    s->packed = false;
    return CC_OK;
}

extern "C" int cc_mlp_get_weights(cc_handle* h, float* w) {
    if (!h || !w || !h->mlp) return ccrt::fail(h, CC_ERR_PARAM, "cc_mlp_get_weights: no network");
    CC_CUDA(h, cudaSetDevice(h->device));
    MlpState* s = static_cast<MlpState*>(h->mlp);
    CC_CUDA(h, cudaMemcpyAsync(w, s->w, P_N * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

extern "C" int cc_mlp_features(cc_handle* h, const double* soa, size_t n, float depth, float* feat) {
    if (!h || (n && (!soa || !feat))) return CC_ERR_PARAM;
    if (!n) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    k_mlp_features<<<grid_for(h, n, 128), 128, 0, h->stream>>>(soa, n, depth, feat);
    CC_LAUNCHED(h);
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

// gradient of the mean loss over the batch (and, if lr > 0, one Adam step)
static int mlp_grad_step(cc_handle* h, const float* feat, const uint32_t* labels, size_t n, float lr, float* loss,
                         float* grad_host) {
    if (!h || !n || !feat || !labels) return CC_ERR_PARAM;
    CC_CUDA(h, cudaSetDevice(h->device));
    if (!h->mlp) return ccrt::fail(h, CC_ERR_PARAM, "cc_mlp: call cc_mlp_init first");
    MlpState* s = static_cast<MlpState*>(h->mlp);
    CC_CUDA(h, cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem));
    const size_t blocks_total = (n + kTrainBlock - 1) / kTrainBlock;
    if (blocks_total > kPartBlocks) return ccrt::fail(h, CC_ERR_TOO_LARGE, "cc_mlp: batch above 65536 samples");
    float* dloss = s->loss;  // per-block loss partials
    k_mlp_grad<<<(int)blocks_total, kTrainBlock, kGradSmem, h->stream>>>(s->w, feat, labels, n, 0,
                                                                        1.0f / (float)n, s->part, dloss);
    CC_LAUNCHED(h);
    s->steps += lr > 0.0f ? 1 : 0;
    const float b1t = powf(0.9f, (float)(s->steps ? s->steps : 1)), b2t = powf(0.999f, (float)(s->steps ? s->steps : 1));
    k_mlp_reduce_adam<<<(P_N + 255) / 256, 256, 0, h->stream>>>(s->w, s->m, s->v, s->part, (int)blocks_total, s->grad,
                                                               lr, b1t, b2t, lr > 0.0f ? 1 : 0);
    CC_LAUNCHED(h);
    if (loss) {
        std::vector<float> lp(blocks_total);
        CC_CUDA(h, cudaMemcpyAsync(lp.data(), dloss, blocks_total * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
        CC_CUDA(h, cudaStreamSynchronize(h->stream));
        double a = 0.0;
        for (float x : lp) a += x;
        *loss = (float)(a / (double)n);
    }
    if (grad_host) {
        CC_CUDA(h, cudaMemcpyAsync(grad_host, s->grad, P_N * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    }
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    s->packed = false;
    return CC_OK;
}

extern "C" int cc_mlp_gradients(cc_handle* h, const float* feat, const uint32_t* labels, size_t n, float* grad,
                                float* loss) {
    if (!grad) return CC_ERR_PARAM;
    return mlp_grad_step(h, feat, labels, n, 0.0f, loss, grad);
}

extern "C" int cc_mlp_train_step(cc_handle* h, const float* feat, const uint32_t* labels, size_t n, float lr,
                                 float* loss) {
    if (!(lr > 0.0f)) return CC_ERR_PARAM;
    return mlp_grad_step(h, feat, labels, n, lr, loss, nullptr);
}

static int mlp_pack(cc_handle* h, MlpState* s) {
    if (s->packed) return CC_OK;
    k_mlp_pack<<<(FR_N + 127) / 128, 128, 0, h->stream>>>(s->w, s->frag, s->bias);
    CC_LAUNCHED(h);
    s->packed = true;
    return CC_OK;
}

extern "C" int cc_mlp_infer(cc_handle* h, const float* feat, size_t n, float* logits) {
    if (!h || (n && (!feat || !logits))) return CC_ERR_PARAM;
    if (!h->mlp) return ccrt::fail(h, CC_ERR_PARAM, "cc_mlp: call cc_mlp_init first");
    if (!n) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    MlpState* s = static_cast<MlpState*>(h->mlp);
    int st = mlp_pack(h, s);
    if (st) return st;
    k_mlp_infer<<<grid_for(h, (n + 15) / 16 * 32, 128), 128, 0, h->stream>>>(s->frag, s->bias, feat, n, nullptr,
                                                                            logits);
    CC_LAUNCHED(h);
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

int cc_mlp_infer_async(cc_handle* h, const float* feat, const unsigned long long* n_dev, unsigned long long cap,
                       float* logits, cudaStream_t st) {
    if (!h->mlp) return ccrt::fail(h, CC_ERR_PARAM, "learned order: call cc_mlp_init and train first");
    MlpState* s = static_cast<MlpState*>(h->mlp);
    int rc = mlp_pack(h, s);
    if (rc) return rc;
    k_mlp_infer<<<h->sm_count * 16, 128, 0, st>>>(s->frag, s->bias, feat, (size_t)cap, n_dev, logits);
    CC_LAUNCHED(h);
    return CC_OK;
}

int cc_first_success_async(cc_handle* h, const double* soa, size_t n, float depth, float* scratch, uint8_t* outcome,
                           uint8_t* evals, cudaStream_t st) {
    static_assert(kFirstScratchFloats == kF + 8, "scratch layout: features, then 8 logits per box");
    if (!n) return CC_OK;
    float* logits = nullptr;
    if (scratch) {
        if (!h->mlp) return ccrt::fail(h, CC_ERR_PARAM, "learned order: no trained network (cc_mlp_init)");
        MlpState* s = static_cast<MlpState*>(h->mlp);
        int rc = mlp_pack(h, s);
        if (rc) return rc;
        float* feat = scratch;
        logits = feat + n * kF;
        k_mlp_features<<<grid_for(h, n, 128), 128, 0, st>>>(soa, n, depth, feat);
        CC_LAUNCHED(h);
        k_mlp_infer<<<grid_for(h, (n + 15) / 16 * 32, 128), 128, 0, st>>>(s->frag, s->bias, feat, n, nullptr, logits);
        CC_LAUNCHED(h);
    }
    k_tight_first<<<grid_for(h, n, 128), 128, 0, st>>>(soa, n, logits, outcome, evals);
    CC_LAUNCHED(h);
    return CC_OK;
}

extern "C" int cc_tight_first(cc_handle* h, const double* soa, size_t n, int learned, uint8_t* outcome,
                              uint8_t* evals) {
    if (!h || (n && (!soa || !outcome))) return CC_ERR_PARAM;
    h->launches = 0;
    if (!n) return CC_OK;
    CC_CUDA(h, cudaSetDevice(h->device));
    float* scratch = nullptr;
    if (learned) {
        if (!h->mlp) return ccrt::fail(h, CC_ERR_PARAM, "cc_tight_first: no trained network (cc_mlp_init)");
        void* p;
        int st = ccrt::ensure(h, 23, n * kFirstScratchFloats * sizeof(float), &p);
        if (st) return st;
        scratch = (float*)p;
    }
    int rc = cc_first_success_async(h, soa, n, 0.0f, scratch, outcome, evals, h->stream);
    if (rc) return rc;
    CC_CUDA(h, cudaStreamSynchronize(h->stream));
    return CC_OK;
}

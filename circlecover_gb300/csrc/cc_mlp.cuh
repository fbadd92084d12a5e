// Pieces of the learned strategy ordering shared by the library's
// translation units: the network's input features and an asynchronous
// inference launch whose row count lives in device memory (a queue counter).
#pragma once

#include <cuda_runtime.h>

#include "cc_iv.cuh"
#include "cc_runtime.cuh"

namespace cc {
namespace mlp {

constexpr int kFeatures = CC_MLP_FEATURES;

// Ten FP32 inputs (they steer the order only, never a verdict) from a box
// (v: la, r1^2..r4^2 as lower/upper pairs) and the weight W its criteria
// require: lambda bounds minus 1, midpoints of r1^2..r3^2, log2 widths of
// r1^2..r3^2 over 16, the signed area slack log10(|sum of midpoints / W - 1|)
// over 8, and the refinement depth.
__device__ inline void features(const double v[10], Iv W, float depth, float* f) {
    f[0] = (float)(v[0] - 1.0);
    f[1] = (float)(v[1] - 1.0);
    double total = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) total += 0.5 * (v[2 + 2 * k] + v[3 + 2 * k]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f[2 + k] = (float)(0.5 * (v[2 + 2 * k] + v[3 + 2 * k]));
        f[5 + k] = log2f(fmaxf((float)(v[3 + 2 * k] - v[2 + 2 * k]), 1e-30f)) * (1.0f / 16.0f);
    }
    const double w = 0.5 * (W.lo + W.hi);
    const float slack = (float)(total / w - 1.0);
    f[8] = log10f(fmaxf(fabsf(slack), 1e-9f)) * (1.0f / 8.0f) * (slack < 0.0f ? -1.0f : 1.0f);
    f[9] = depth;
}

}  // namespace mlp
}  // namespace cc

// logits[i * 8 + k] for rows i < min(*n_dev, cap) of feat, on stream s
// (no synchronisation); the network must have been initialised
int cc_mlp_infer_async(cc_handle* h, const float* feat, const unsigned long long* n_dev, unsigned long long cap,
                       float* logits, cudaStream_t s);

// First-success outcomes (as cc_tight_first) of n boxes in SoA device memory
// on stream s, no synchronisation.  With scratch != nullptr the network's
// most likely criterion runs first: scratch holds n * kFirstScratchFloats
// floats (features at `depth`, then logits).  evals may be nullptr.
constexpr int kFirstScratchFloats = CC_MLP_FEATURES + 8;
int cc_first_success_async(cc_handle* h, const double* soa, size_t n, float depth, float* scratch, uint8_t* outcome,
                           uint8_t* evals, cudaStream_t s);

// Platform layer of the prover: function qualifiers, the FP64 directed-
// rounding primitives and the per-box trap status.
//
// The criteria headers are compiled two ways:
//   * by nvcc for sm_103a (the product): primitives are the CUDA intrinsics
//     __dadd_rd ... __drcp_ru, exactly what the reference's interval type uses
//     (reference: algcuda/cuda-utils/cuh/include/algcuda/interval.cuh:30-355);
//   * by a host C++ compiler with CC_HOST_PORT defined (the oracle's CPU port
//     and the CPU baseline): primitives come from a host rounding layer that
//     the including translation unit provides as cc_sw_* functions.
#pragma once

#include <stdint.h>
#include <math.h>

#include <atomic>

#if defined(__CUDACC__) && !defined(CC_HOST_PORT)
#define CC_DEVICE_BUILD 1
#define CC_FN __device__ __forceinline__
#define CC_FN_NOINLINE static __device__ __noinline__
#define CC_FN_INL __device__ inline
#define CC_METHOD __device__ __forceinline__
#else
#define CC_FN static inline
#define CC_FN_NOINLINE static
#define CC_FN_INL static inline
#define CC_METHOD inline
#endif

namespace cc {

// ------------------------------------------------------------------ rounding
#if CC_DEVICE_BUILD
CC_FN double add_dn(double a, double b) { return __dadd_rd(a, b); }
CC_FN double add_up(double a, double b) { return __dadd_ru(a, b); }
CC_FN double mul_dn(double a, double b) { return __dmul_rd(a, b); }
CC_FN double mul_up(double a, double b) { return __dmul_ru(a, b); }
CC_FN double div_dn(double a, double b) { return __ddiv_rd(a, b); }
CC_FN double div_up(double a, double b) { return __ddiv_ru(a, b); }
CC_FN double sqrt_dn(double a) { return __dsqrt_rd(a); }
CC_FN double sqrt_up(double a) { return __dsqrt_ru(a); }
CC_FN double rcp_dn(double a) { return __drcp_rd(a); }
CC_FN double rcp_up(double a) { return __drcp_ru(a); }
#else
CC_FN double add_dn(double a, double b) { CC_PORT_TICK(); return cc_sw_add_rd(a, b); }
CC_FN double add_up(double a, double b) { CC_PORT_TICK(); return cc_sw_add_ru(a, b); }
CC_FN double mul_dn(double a, double b) { CC_PORT_TICK(); return cc_sw_mul_rd(a, b); }
CC_FN double mul_up(double a, double b) { CC_PORT_TICK(); return cc_sw_mul_ru(a, b); }
CC_FN double div_dn(double a, double b) { CC_PORT_TICK(); return cc_sw_div_rd(a, b); }
CC_FN double div_up(double a, double b) { CC_PORT_TICK(); return cc_sw_div_ru(a, b); }
CC_FN double sqrt_dn(double a) { CC_PORT_TICK(); return cc_sw_sqrt_rd(a); }
CC_FN double sqrt_up(double a) { CC_PORT_TICK(); return cc_sw_sqrt_ru(a); }
CC_FN double rcp_dn(double a) { CC_PORT_TICK(); return cc_sw_rcp_rd(a); }
CC_FN double rcp_up(double a) { CC_PORT_TICK(); return cc_sw_rcp_ru(a); }
#endif

// "+infinity", which the reference spells DBL_MAX*DBL_MAX (interval.cuh:
// 227-240).
#define CC_INF ((double)INFINITY)
#define CC_DBL_MAX 1.7976931348623157e308

// ------------------------------------------------------------ trap status
// The reference calls algcuda::trap() (a PTX `trap`, which kills the CUDA
// context and every other box of the launch) on interval-domain errors and
// on geometric situations its proofs exclude.  Here a trap only marks the box
// that hit it: the evaluation keeps going with NaN-valued intervals (all
// loops are iteration-bounded), and the caller reads and clears the status,
// reports the box as "trapped" and never as certified.
enum TrapSite : uint32_t {
    TRAP_NONE = 0,
    TRAP_SQRT_NEGATIVE = 1,    // Interval::sqrt with lb < 0 (interval.cuh:339-346)
    TRAP_BISECTION_CAP = 2,    // a bisection did not reach its fixpoint (NaN bounds)
    TRAP_FIVE_DISK = 3,        // rectangle_size_bound/five_disk_full_cover.cu:140
    TRAP_SIX_DISK = 4,         // rectangle_size_bound/six_disk_full_cover.cu:69
    TRAP_SEVEN_DISK_A = 5,     // rectangle_size_bound/seven_disk_strategies.cu:267
    TRAP_SEVEN_DISK_B = 6,     // rectangle_size_bound/seven_disk_strategies.cu:409
    TRAP_SEVEN_DISK_C = 7,     // rectangle_size_bound/seven_disk_strategies.cu:456
    TRAP_SEVEN_DISK_D = 8,     // rectangle_size_bound/seven_disk_strategies.cu:971
    TRAP_F32_UNDECIDED = 9,    // not a reference trap: an FP32 enclosure could not decide (cc_f32.cuh)
};

// A bisection on doubles halves its bracket every step; from any finite
// bracket it reaches the FP64 fixpoint in fewer than 2100 steps.  Hitting
// this cap means the bracket held a NaN: the reference would spin forever.
#define CC_BISECTION_CAP 2200

#if CC_DEVICE_BUILD
// one status byte per thread, kept in shared memory so that any device
// function can set it without threading a context argument through every
// criterion; 1024 threads per block at most.
// Bits 5, 6 and 7 of the byte are mode bits (cc_tight.cuh): bit 7 makes the
// FP32 can_recurse record its arguments instead of evaluating, bit 6 makes
// the FP64 can_recurse evaluate only one chosen call of a certification run
// (cc_cert_state) and answer "false" to the others, and bit 5 (with bit 6)
// makes that chosen call store its arguments (cc_cert_out) and answer "true"
// instead of evaluating.  trap_clear() clears them, trap() keeps them.
static __shared__ uint8_t cc_trap_words[1024];
static constexpr uint8_t kTrapModeBit = 0x80;
static constexpr uint8_t kCertModeBit = 0x40;
static constexpr uint8_t kCertRecordBit = 0x20;
static constexpr uint8_t kTrapModeBits = kTrapModeBit | kCertModeBit | kCertRecordBit;
CC_FN void trap(uint32_t site) {
    cc_trap_words[threadIdx.x] = (uint8_t)((cc_trap_words[threadIdx.x] & kTrapModeBits) | site);
}
CC_FN uint32_t trap_status() { return cc_trap_words[threadIdx.x] & (uint8_t)~kTrapModeBits; }
CC_FN void trap_clear() { cc_trap_words[threadIdx.x] = TRAP_NONE; }
// Per-thread call bookkeeping of the certification runs: the low byte counts
// can_recurse calls, the high byte is the number (1-based) of the one call a
// certification run evaluates (0: none).
static __shared__ uint16_t cc_cert_state[1024];
// The arguments of a certification run's chosen call (record form, bit 5):
// ub_w, ub_h, ub_largest, lb_weight.  cc_cert_out points to one per thread
// of the block, in the shared memory of the kernel that sets bit 5.
struct CertCall {
    double w, h, largest, lb;
};
static __shared__ CertCall* cc_cert_out;
// FP64 certifications that failed in this translation unit's kernels since
// the library was loaded: an FP32 decision the FP64 check did not confirm
// (the FP64 result is used instead).  Expected to stay 0; the host reads it
// with cudaMemcpyFromSymbol.
static __device__ unsigned long long cc_cert_fail_count;
CC_FN void cert_failed() { atomicAdd(&cc_cert_fail_count, 1ULL); }
// failures the host learnt of from a certification pass's counters
static std::atomic<unsigned long long> cert_failures_host{0};
#else
// host build: per-thread status (initial-exec TLS: a plain load per access)
#ifndef CC_HOST_TLS
#define CC_HOST_TLS thread_local __attribute__((tls_model("initial-exec")))
#endif
extern CC_HOST_TLS uint32_t cc_port_trap_word;
CC_FN void trap(uint32_t site) { cc_port_trap_word = site; }
CC_FN uint32_t trap_status() { return cc_port_trap_word; }
CC_FN void trap_clear() { cc_port_trap_word = TRAP_NONE; }
#endif

}  // namespace cc

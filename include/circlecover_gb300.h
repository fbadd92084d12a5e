/*
 * circlecover_gb300 — C ABI of the GB300 (sm_103a) prover for the
 * rectangle-covering-by-disks proofs of phillip-keldenich/circlecover.
 *
 * The reference has no plugin or FFI layer; its boundary is a set of C++
 * declarations.  Each entry point below names the reference interface it
 * replaces (paths relative to the reference's Prover/ directory):
 *
 *   cc_tight_eval / cc_tight_eval_device
 *       the six exported tight-rectangle criteria, evaluated per box
 *       (tight_rectangle/strategies.cuh:54-87: r1_strategies,
 *       r1_r2_strategies, both r1_r2_r3_strategies overloads,
 *       two_by_two_strategies, r1_r2_large_r3_r4_gaps_strategy) at the
 *       arguments the reference's leaf passes them
 *       (tight_rectangle/tight_rectangle.cu:229-248)
 *   cc_tight_prove
 *       circlecover::tight_rectangle::find_critical_intervals()
 *       (tight_rectangle/tight_rectangle.cu:458-537; called by prover.cpp:34),
 *       with the split counts as parameters instead of compile-time constants
 *       (tight_rectangle.cu:44-68)
 *   cc_tight_summary
 *       kernel_compute_distance_from_theoretical_worst_cases
 *       (tight_rectangle.cu:322-456)
 *   cc_sb_eval / cc_sb_eval_device
 *       the size-bound criteria and shortcuts, evaluated per box
 *       (rectangle_size_bound/strategies.cuh:32-147, in the cascade of
 *       rectangle_size_bound.cu:161-231)
 *   cc_sb_prove
 *       circlecover::rectangle_size_bound::find_critical_intervals()
 *       (rectangle_size_bound/rectangle_size_bound.cu:312-382; called by
 *       prover.cpp:35), split counts as parameters (:36-62)
 *
 * Conventions: plain C types, caller-owned buffers unless stated, status
 * codes instead of exceptions (the reference throws std::system_error or
 * std::logic_error, or kills the CUDA context with a device trap).  A handle
 * owns one CUDA stream and its device buffers; calls on one handle must not
 * overlap (not thread-safe per handle).
 */
#ifndef CIRCLECOVER_GB300_H
#define CIRCLECOVER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* == algcuda::Interval<double> (interval.hpp:84-242): {lb, ub} */
typedef struct cc_iv {
    double lb, ub;
} cc_iv;

/* == circlecover::tight_rectangle::Variables (tight_rectangle/strategies.cuh:33-35) */
typedef struct cc_tight_box {
    cc_iv la;
    cc_iv r[4]; /* squared radii r1^2 >= r2^2 >= r3^2 >= r4^2 */
} cc_tight_box;

/* == circlecover::rectangle_size_bound::Variables (rectangle_size_bound/variables.hpp:33-35) */
typedef struct cc_sb_box {
    cc_iv la;
    cc_iv r[6];
} cc_sb_box;

enum cc_status {
    CC_OK = 0,
    CC_ERR_CUDA = 1,           /* a CUDA runtime call failed */
    CC_ERR_PARAM = 2,          /* invalid argument */
    CC_ERR_QUEUE_OVERFLOW = 3, /* a device work queue exceeded its capacity */
    CC_ERR_TIMEOUT = 4,        /* a bounded device wait ran out */
    CC_ERR_INTERRUPTED = 5,    /* cc_interrupt() was called during a proof */
    CC_ERR_NO_DEVICE = 6,      /* no CUDA device / not built for this device */
    CC_ERR_OOM = 7,            /* device or host allocation failed */
    CC_ERR_TOO_LARGE = 8       /* batch larger than a fixed-capacity entry point accepts */
};

/* ---- per-box verdict mask of cc_tight_eval ------------------------------- */
#define CC_TV_R1 (1u << 0)          /* r1_strategies(la, r1, r2.ub) */
#define CC_TV_R1R2 (1u << 1)        /* r1_r2_strategies(la, r1, r2, r3.ub) */
#define CC_TV_R1R2R3 (1u << 2)      /* r1_r2_r3_strategies(la, r1, r2, r3, r4.ub) */
#define CC_TV_TWO_BY_TWO (1u << 3)  /* two_by_two_strategies(tightened box, R) */
#define CC_TV_R1R2R3_LEAF (1u << 4) /* r1_r2_r3_strategies(tightened box, R4) */
#define CC_TV_GAPS (1u << 5)        /* r1_r2_large_r3_r4_gaps_strategy(tightened box, R) */
#define CC_TV_R_EMPTY (1u << 6)     /* R or R4 is empty: the reference's leaf skips the box */
#define CC_TV_TRAPPED (1u << 31)    /* a criterion hit a reference trap site */

/* ---- per-box verdict mask of cc_sb_eval ---------------------------------- */
/* bit k (0..13) = the k-th criterion of the size-bound cascade certified the
 * tightened box (rectangle_size_bound/rectangle_size_bound.cu:201-229, in
 * that order: even split, uneven split, multi-disk strip, wall building, r1
 * in corner (explicit), r1/r2 opposite corners, r1/r2 vertical strip, 2x2
 * cover (with strip and recursion), L-shaped, r1 in corner (wall building),
 * advanced multi-disk strip, five-disk cover, six-disk cover, seven-disk
 * strategies); bit 14 = box or R empty (the reference's leaf skips it);
 * bits 15..19 = the kernel's shortcuts on the untightened box
 * (rectangle_size_bound.cu:162-177): even split (la,r1,r2), uneven split
 * (la,r1,r2), uneven split (la,r1,r2,r3), opposite corners, vertical strip;
 * bit 31 = a criterion reached a trap site. */
#define CC_SV_CRITERIA_MASK 0x3fffu
#define CC_SV_EMPTY (1u << 14)
#define CC_SV_SHORTCUTS_MASK (0x1fu << 15)
#define CC_SV_TRAPPED (1u << 31)

/* ---- outcome codes of the proof trace (one per grid cell visited) -------- */
enum cc_trace_outcome {
    /* level 0: r1 cells */
    CC_T_L1_EMPTY = 0, CC_T_L1_R1 = 1, CC_T_L1_SPLIT = 2,
    /* level 1: r2 cells */
    CC_T_L2_R1 = 0, CC_T_L2_EMPTY = 1, CC_T_L2_R12 = 2, CC_T_L2_SPLIT = 3,
    /* level 2: r3 cells */
    CC_T_L3_R12 = 0, CC_T_L3_EMPTY = 1, CC_T_L3_R123 = 2, CC_T_L3_R4EMPTY = 3, CC_T_L3_SPLIT = 4,
    /* level 3: r4 cells (leaves) */
    CC_T_L4_R123 = 0, CC_T_L4_REMPTY = 1, CC_T_L4_2X2 = 2, CC_T_L4_R123LEAF = 3, CC_T_L4_GAPS = 4,
    CC_T_L4_CRITICAL = 5, CC_T_L4_TRAPPED = 6
};

#define CC_MAX_GENERATIONS 32

/* Split counts of the tight proof.  The reference's values
 * (tight_rectangle.cu:44-58) are la_splits_init 256, r_splits_init
 * {128,128,128,128}, num_generations 11, la_splits_gen
 * {1,2,2,2,2,1,2,1,2,1,2}, r_splits_gen {128,128,128,64}. */
typedef struct cc_tight_grid {
    int la_splits_init;
    int r_splits_init[4];
    int num_generations;
    int la_splits_gen[CC_MAX_GENERATIONS];
    int r_splits_gen[4];
} cc_tight_grid;

typedef struct cc_prove_stats {
    uint64_t counts[4][8];     /* grid cells visited, by level and outcome */
    uint64_t digest;           /* sum of mix64(cell key) over all cells */
    uint64_t leaf_evals;       /* r4 cells evaluated */
    uint64_t trapped_leaves;   /* leaves kept as critical because of a trap */
    uint64_t gen_sizes[CC_MAX_GENERATIONS + 1]; /* criticals after init, gen 1, ... */
    int32_t generations_run;
    int32_t reserved;
    double seconds;            /* wall time of the call */
    uint64_t kernel_launches;  /* kernels launched by the call */
    /* Leaf criteria evaluated FP32-first (the prepared form's 2x2 and leaf
     * r1_r2_r3 criteria), by outcome: [0] FP32 undecided, evaluated in FP64;
     * [1] FP32 "false"; [2] FP32 "true", certified in FP64 (the criterion's
     * FP64 code with only the settling can_recurse call evaluated); [3]
     * certification failed, the FP64 result used.  Generations run by this
     * call only (a resumed proof counts from the checkpoint on). */
    uint64_t fp32_first[4];
    /* FP64 certifications that failed during the call (leaf criteria and the
     * bisections' results; expected 0): the FP64 result was used instead.
     * Counted per device for the library's tight kernels, so calls running
     * at the same time on other handles of the device add theirs. */
    uint64_t cert_failures;
} cc_prove_stats;

/* ---- size-bound proof ------------------------------------------------------
 * Trace outcomes by level: 0 = task (one lambda x r1 x r2 piece of a parent
 * box), 1 = r3 cell of a task, 2 = leaf (an r4 x r5 x r6 cell). */
enum cc_sb_trace_outcome {
    CC_SBT_TASK_EMPTY = 0, CC_SBT_TASK_EVEN = 1, CC_SBT_TASK_UNEVEN = 2, CC_SBT_TASK_SPLIT = 3,
    CC_SBT_CELL_UNEVEN = 0, CC_SBT_CELL_OPPOSITE = 1, CC_SBT_CELL_VSTRIP = 2, CC_SBT_CELL_SPLIT = 3,
    /* leaves: 0..13 = the criterion (CC_SV_* bit order) that certified it */
    CC_SBT_LEAF_EMPTY = 14, CC_SBT_LEAF_CRITICAL = 15, CC_SBT_LEAF_TRAPPED = 16
};
#define CC_SBT_LEAF_OUTCOMES 17

/* Split counts of the size-bound proof.  The reference's values
 * (rectangle_size_bound.cu:36-62): la_splits_init 256, r_splits_init
 * {128,128,64,64,64,64}, la_splits_gen 64, r_splits_gen {32,32,16,16,16,32},
 * num_generations 1.  Every count in [1, 2047]. */
typedef struct cc_sb_grid {
    int la_splits_init;
    int r_splits_init[6];
    int la_splits_gen;
    int r_splits_gen[6];
    int num_generations;
} cc_sb_grid;

typedef struct cc_sb_prove_stats {
    uint64_t task_counts[4];                  /* by CC_SBT_TASK_* */
    uint64_t cell_counts[4];                  /* by CC_SBT_CELL_* */
    uint64_t leaf_counts[CC_SBT_LEAF_OUTCOMES];
    uint64_t digest;                          /* sum of the mixed trace keys */
    uint64_t leaf_evals;                      /* leaves visited */
    uint64_t trapped_leaves;                  /* leaves kept because of a trap */
    uint64_t trapped_shortcuts;               /* shortcuts not taken because of a trap */
    uint64_t gen_sizes[CC_MAX_GENERATIONS + 1]; /* criticals after init (merged), gen 1, ... */
    int32_t generations_run;
    int32_t reserved;
    double seconds;
    uint64_t kernel_launches;
    /* FP32 pre-filter: leaves it proved empty (no FP64 work for them), and
     * over the other leaves with an FP64 R of nonzero width the mean and the
     * largest ratio of the FP32 bounds' width to the FP64 width of R */
    uint64_t fp32_decided;
    uint64_t widening_samples;
    double widening_mean;
    double widening_max;
    /* FP64 certification of the FP32 decisions: leaf verdicts the FP32-first
     * passes (uneven split, multi-disk strip) decided "true", certified by
     * the FP64 criterion from that placement on; anchors of the pre-filter's
     * empty leaves certified by the FP64 emptiness test (one anchor certifies
     * the run of empty leaves after it in its (r3, r4, r5) row: the test is
     * monotone in the r6 piece); certifications that failed during the call
     * (the FP64 verdict was used, a slice with a failed anchor was redone
     * without the pre-filter; expected 0, counted per device).  The FP32
     * "true" of the even split and of the r1-in-corner backtracking are
     * decided by their FP64 form, whose verdict is the one used. */
    uint64_t fp32_certified;
    uint64_t empty_anchors;
    uint64_t cert_failures;
} cc_sb_prove_stats;

/* summary of the final criticals vs the theoretical worst cases;
 * == Max_distances (tight_rectangle.cu:322-341) */
typedef struct cc_tight_summary_t {
    int32_t have_range_2d, have_range_3d;
    cc_iv la_range_2d, la_range_3d;
    cc_iv dist_r1_2d;
    cc_tight_box dist_r1_2d_criticals[2];
    cc_iv dist_r2_2d;
    cc_tight_box dist_r2_2d_criticals[2];
    double lb_h1_2d;
    double ub_la_by_S1;
    double ub_R3_2d;
    cc_iv dist_r1_3d;
    cc_tight_box dist_r1_3d_criticals[2];
    cc_iv dist_r2_3d;
    cc_tight_box dist_r2_3d_criticals[2];
    cc_iv dist_r3_3d;
    cc_tight_box dist_r3_3d_criticals[2];
    double ub_R4_3d;
    cc_iv S1, h2, S3;
    double pocket_width_3d;
} cc_tight_summary_t;

typedef struct cc_handle cc_handle;

/* Open a handle on CUDA device `device` (creates one stream). */
int cc_create(cc_handle** out, int device);
int cc_destroy(cc_handle* h);
const char* cc_status_str(int status);
/* text of the last error on this handle (CUDA error string etc.) */
const char* cc_last_error(cc_handle* h);

/* Evaluate the six tight criteria on n boxes given in HOST memory (AoS);
 * verdict masks (CC_TV_*) are written to host memory.  Includes the
 * host<->device transfers: the boxes move in chunks (4M boxes; above 2^20
 * boxes the first chunk is a quarter of that) by the copy engine on a
 * second stream, which also transposes each chunk to SoA, while the
 * previous chunk is evaluated; straight from the caller's array when it is
 * page-locked or the device can access pageable host memory
 * (cudaDevAttrPageableMemoryAccess, e.g. GB300 with its host over
 * NVLink-C2C), otherwise through pinned buffers that host threads fill.  The
 * masks return in one copy at the end.  Environment: CC_HOST_STAGING=1,
 * read when the handle is created, forces the staging path;
 * CC_EVAL_CHUNK_LOG2 (16..26, read once) sets the chunk size (same
 * results). */
int cc_tight_eval(cc_handle* h, const cc_tight_box* boxes, size_t n, uint32_t* masks);

/* Same on DEVICE memory: `soa` holds 10 arrays of n doubles each, in the order
 * la.lb, la.ub, r1.lb, r1.ub, ..., r4.ub (structure of arrays, element i of
 * array k at soa[k*n + i]); masks is a device array of n uint32.  Launches on
 * `stream` (a cudaStream_t; NULL = the handle's stream) and does not
 * synchronise. */
int cc_tight_eval_device(cc_handle* h, const double* soa, size_t n, uint32_t* masks, void* stream);

/* Allocation-free variant of cc_tight_eval_device.  It has no counterpart in
 * the reference.  It is for callers that cannot allocate device memory while
 * they run -- a host framework that owns every device allocation, a
 * latency-critical loop in which cudaMalloc's implicit synchronisation is not
 * acceptable, a process that reserves all memory at start-up -- and so cannot
 * create a handle either.  Same inputs, outputs and results as
 * cc_tight_eval_device (FP64 certification included); it works on the
 * calling thread's current device and launches on `stream` (a cudaStream_t;
 * NULL = the legacy default stream) without synchronising.
 *   - Its scratch is a fixed array inside the library image,
 *     CC_STATIC_EVAL_SCRATCH_BYTES per GPU (about 2.3 MiB: the queues of the
 *     evaluation passes, 37 bytes per box), held until the process exits;
 *     batches of more than CC_STATIC_EVAL_MAX_BOXES boxes are rejected with
 *     CC_ERR_TOO_LARGE (split larger batches into several calls).
 *   - Set-up: the first call on a device looks up that array's device
 *     address, and the first launch of each of its kernels may make the CUDA
 *     driver load the library's module (lazy module loading), which can
 *     allocate and synchronise.  Make one warm-up call (n = 1 will do) on
 *     each device at start-up, before any stream capture and before the part
 *     of the program that must not allocate; later calls then allocate
 *     nothing.
 *   - All calls on a device share the array, which keeps the last call's
 *     queues (each call clears the counters it needs): calls that can
 *     overlap on the GPU (different streams, or other threads) race and give
 *     wrong masks; serialise them (one stream, or events).
 *   - It calls no cudaMalloc, cudaFree or allocating library routine.
 *   - A CUDA error already pending when it is called is left as it is and
 *     reported as CC_ERR_CUDA without launching anything. */
#define CC_STATIC_EVAL_MAX_BOXES 65536
#define CC_STATIC_EVAL_SCRATCH_BYTES (256 + 65536 * 37) /* 2,425,088 bytes */
int cc_tight_eval_device_static(const double* soa, size_t n, uint32_t* masks, void* stream);

/* Evaluate the size-bound criteria on n boxes in HOST memory (AoS, 112-byte
 * boxes); verdict masks (CC_SV_*) to host memory.  Replaces the criteria of
 * rectangle_size_bound/strategies.cuh:32-147 as the reference's leaf calls
 * them (rectangle_size_bound/rectangle_size_bound.cu:189-231). */
int cc_sb_eval(cc_handle* h, const cc_sb_box* boxes, size_t n, uint32_t* masks);
/* Same on DEVICE memory: 14 arrays of n doubles (la.lb, la.ub, r1.lb, ...,
 * r6.ub); asynchronous on `stream` (NULL = the handle's stream). */
int cc_sb_eval_device(cc_handle* h, const double* soa, size_t n, uint32_t* masks, void* stream);

/* Number of kernels the last call on this handle launched. */
uint64_t cc_last_launch_count(cc_handle* h);

/* Autotuner (no reference counterpart).  Times each of the four
 * evaluation passes of cc_tight_eval_device with every register budget
 * (minimum resident blocks 1, 4, 8: at most 255, 128, 64 registers per
 * thread) and grid size (2, 4, 8, 16 blocks of 128 threads per SM) on the
 * caller's sample (device SoA boxes and a masks array), and keeps the
 * fastest per pass in the handle for later evaluation calls.  The defaults
 * are 1 and 8. */
typedef struct cc_tune_result {
    int min_blocks[4];     /* chosen register budget of the FP32, FP64, strip-width and gap-width pass */
    int blocks_per_sm[4];  /* chosen grid */
    float ms[4];           /* time of each pass with the chosen setting */
    float ms_default[4];   /* time with the defaults */
} cc_tune_result;
int cc_autotune_eval(cc_handle* h, const double* soa, size_t n, uint32_t* masks, cc_tune_result* out);

/* Per-stage device timing (no reference counterpart; a measurement aid).
 * While enabled, cc_tight_eval_device records a CUDA event around each of
 * its six passes on the stream it launches on:
 *   stage 0 = k_eval_f32   (all criteria on FP32 enclosures of the FP64
 *                           values, one kernel per criterion group, and
 *                           k_eval_collect, which queues the boxes they could
 *                           not decide, the bisection jobs and the FP32
 *                           verdicts to certify),
 *   stage 1 = k_eval_main  (the FP64 criteria on the queued boxes),
 *   stage 2 = k_eval_cover (strip-width bisection of the compacted queue,
 *                           with the FP64 certificate of a true result),
 *   stage 3 = k_eval_gaps  (gap-width bisection of the compacted queue,
 *                           with the FP64 certificate of a true result),
 *   stage 4 = k_eval_cert  (FP64 certification of every verdict bit the FP32
 *                           pass decided "true", one kernel per criterion
 *                           group on its compacted queue),
 *   stage 5 = k_eval_repair (the boxes whose certification failed, evaluated
 *                           again in FP64 alone; expected to be none).
 * cc_last_stage_times waits for the last recorded event and writes the
 * elapsed milliseconds of each stage of the most recent call (at most
 * max_stages values; *n_stages = how many were written). */
#define CC_EVAL_STAGES 6
/* the first four stages are the ones cc_autotune_eval tunes */
#define CC_EVAL_TUNED_STAGES 4
int cc_set_stage_timing(cc_handle* h, int enable);
/* CUDA graph of the evaluation's launch sequence (on by default; no
 * reference counterpart): cc_tight_eval_device captures its launches once
 * into a CUDA graph and replays it with one cudaGraphLaunch while the same
 * arguments (input, count, masks, stream, tuning) repeat, and re-captures it
 * into the same executable graph when they change.  Off while stage timing
 * is on, and on a stream the caller is capturing (the launches then join
 * the caller's graph); cc_tight_eval launches its chunks directly.
 * cc_eval_graph_stats: how many captures and replays this handle made. */
int cc_set_eval_graph(cc_handle* h, int enable);
int cc_eval_graph_stats(cc_handle* h, unsigned long long* captures, unsigned long long* replays);
int cc_last_stage_times(cc_handle* h, float* ms, int max_stages, int* n_stages);
/* Queue sizes of the most recent evaluation batch (waits for the device):
 * counts[0] boxes the FP32 pass left to the FP64 pass, counts[1] boxes that
 * needed the strip-width bisection, counts[2] the gap-width bisection,
 * counts[3] nonzero if a queue overflowed (cannot happen: each queue holds
 * the whole batch). */
int cc_last_eval_counts(cc_handle* h, unsigned long long* counts);

/* FP64 certification of the evaluation (no reference counterpart).  The FP32
 * pass decides most verdict bits on outward-rounded FP32 enclosures of the
 * FP64 values.  With certification on (the default), every bit it decides
 * "true" -- a criterion certifies the box, or R / R4 is empty -- is checked
 * again in FP64 directed rounding before it is reported: the criterion's
 * FP64 code runs with only the can_recurse call that settled the FP32 run
 * evaluated (every other call answers "false", which can only make the
 * criterion false), the three-strips placement and the emptiness test run
 * in full, and a bisection's result is checked as the reference's own
 * argument (the width used is realizable in FP64 and the rest of the
 * rectangle recursively coverable in FP64).  A bit whose certification fails
 * sends its box through the FP64 evaluation alone, whose mask is reported.
 * Bits decided "false" are not re-checked: a false bit can only keep a box,
 * never discard one.  cc_set_eval_certify(h, 0) is the uncertified FP32
 * form (opt-in, for measurement). */
int cc_set_eval_certify(cc_handle* h, int enable);
/* Certification counts of the most recent evaluation batch (waits for the
 * device), CC_EVAL_CERT_COUNTS values: [0..4] FP32 "true" verdicts certified
 * per criterion group (r1 bit 0, r1_r2 bit 1, 2x2 bit 3, leaf r1_r2_r3 bit 4,
 * and boxes with the three-strips bit 2 or the emptiness bit 6), [5] boxes
 * whose certification failed and were evaluated in FP64 alone, [6] true
 * strip-width results certified, [7] true gap-width results certified. */
#define CC_EVAL_CERT_COUNTS 8
int cc_last_eval_cert(cc_handle* h, unsigned long long* counts);

/* Run the tight proof from `root` with split counts `grid`.  On success
 * *criticals points to *n_crit boxes (release with cc_free), in the order the
 * reference's driver produces them; stats may be NULL. */
int cc_tight_prove(cc_handle* h, const cc_tight_box* root, const cc_tight_grid* grid, cc_tight_box** criticals,
                   size_t* n_crit, cc_prove_stats* stats);

/* cc_tight_prove with options.  CC_PROVE_PLAIN evaluates every criterion in
 * every grid cell as the reference does; the default (0) prepares the parts
 * of a criterion that do not depend on the child cell's bound once per parent
 * cell.  Both give identical criticals and traces. */
#define CC_PROVE_PLAIN 1
/* Learned leaf order (prepared form only): per r3 cell the network
 * (cc_mlp_*) predicts whether the leaf criterion r1_r2_r3_strategies(box,
 * R4) certifies the cell's leaves; where it does, that criterion is tried
 * before the 2x2 criterion.  The criticals are the same as without it (a box
 * is critical when no criterion certifies it, in any order; only a leaf that
 * reaches a trap site in one order and is certified earlier in the other
 * could differ); the trace then records the criterion that certified in the
 * order used. */
#define CC_PROVE_LEARNED 4
/* Log a sample (1 in 64, at most 2^20) of the r3 cells the proof splits,
 * as boxes with r4 = the cell's r4 range, for training records
 * (cc_tight_cell_log). */
#define CC_PROVE_LOG_CELLS 8
int cc_tight_prove_ex(cc_handle* h, const cc_tight_box* root, const cc_tight_grid* grid, int flags,
                      cc_tight_box** criticals, size_t* n_crit, cc_prove_stats* stats);

/* Checkpoints of the tight proof (no reference counterpart; the reference
 * can only be interrupted).  With a path set, cc_tight_prove_ex writes the
 * state after every completed generation (grid, next generation, trace
 * totals, generation sizes, the criticals so far) to `path` (atomically:
 * written to path.tmp, then renamed).  cc_tight_resume continues from such a
 * file with `grid` (NULL: the saved one), which must extend the saved
 * schedule; the result and stats equal those of an uninterrupted run.
 * cc_set_checkpoint(h, NULL) turns checkpoints off. */
int cc_set_checkpoint(cc_handle* h, const char* path);
int cc_tight_resume(cc_handle* h, const char* path, const cc_tight_grid* grid, int flags, cc_tight_box** criticals,
                    size_t* n_crit, cc_prove_stats* stats);

/* One generation of the tight proof restricted to the tasks [task_lo,
 * task_hi) of that generation (task = parent index * la_splits + lambda
 * piece; tasks outside the range contribute nothing).  Criticals are
 * returned in task order, merged per task as the reference does; the
 * concatenation over consecutive ranges equals the whole generation's
 * output, and the stats (counts, digest, leaves) add up.  This is the unit a
 * process group shards (one range per rank, the criticals all-gathered in
 * rank order as the next generation's parents).  flags as cc_tight_prove_ex. */
int cc_tight_generation(cc_handle* h, const cc_tight_box* parents, size_t n_parents, int la_splits,
                        const int r_splits[4], uint64_t task_lo, uint64_t task_hi, int flags,
                        cc_tight_box** criticals, size_t* n_crit, cc_prove_stats* stats);

/* The cells logged by the last cc_tight_prove_ex with CC_PROVE_LOG_CELLS:
 * *n = how many (at most cap copied into out), *r4_splits = the r4 split
 * count of their leaves (may be NULL). */
int cc_tight_cell_log(cc_handle* h, cc_tight_box* out, size_t cap, size_t* n, int* r4_splits);

/* Summary of a critical set vs the 2- and 3-disk worst cases
 * (kernel_compute_distance_from_theoretical_worst_cases). */
int cc_tight_summary(cc_handle* h, const cc_tight_box* criticals, size_t n, cc_tight_summary_t* out);

/* Run the size-bound proof from `root` (replaces the driver and kernel of
 * rectangle_size_bound/rectangle_size_bound.cu:132-382: the (lambda, r1, r2)
 * host loops of find_critical_intervals_in, one kernel launch per task
 * there, the r3..r6 grid of kernel_find_critical_intervals_in with its
 * shortcuts and cascade, and the generation loop with
 * merge_critical_intervals<N>).  On success *criticals points to *n_crit
 * boxes (release with cc_free) in the reference's final order (sorted and
 * merged), each with a flag in *flags (NULL allowed; cc_free it): bit 0 =
 * kept because a criterion reached a trap site.  stats may be NULL.
 * Work units: tasks are processed in chunks of 2^18 and undecided leaves in
 * queues of 2^24 (about 9 GB of device memory in all); the environment
 * variables CC_SB_TASK_CHUNK_LOG2 (0..18) and
 * CC_SB_SLICE_LOG2 (5..26) change them (same results, other launches). */
int cc_sb_prove(cc_handle* h, const cc_sb_box* root, const cc_sb_grid* grid, cc_sb_box** criticals, size_t* n_crit,
                uint32_t** flags, cc_sb_prove_stats* stats);

/* One generation of the size-bound proof restricted to the tasks [task_lo,
 * task_hi) of that generation (task = parent * (la_splits * r1 splits * r2
 * splits) + lambda piece * (r1 * r2 splits) + r1 piece * r2 splits + r2
 * piece, the order of the reference's host loops,
 * rectangle_size_bound/rectangle_size_bound.cu:276-310); generation `gen`
 * (0 = the initial pass) selects the trace keys and the merge of the found
 * leaves (merge_critical_intervals<N> with N = 0 for gen 0, else 2, 1, 3 by
 * gen mod 3; :351-362).  The unit the sampled parity tests of the full runs
 * check against the reference's criteria; stats as cc_sb_prove (gen_sizes[0]
 * = the criticals returned).  options as cc_sb_prove_ex. */
int cc_sb_generation(cc_handle* h, const cc_sb_box* parents, size_t n_parents, int gen, int la_splits,
                     const int r_splits[6], uint64_t task_lo, uint64_t task_hi, int options, cc_sb_box** criticals,
                     size_t* n_crit, uint32_t** flags, cc_sb_prove_stats* stats);

/* cc_sb_prove with options: CC_PROVE_PLAIN runs the plain form (one thread
 * per leaf runs the whole cascade, as the reference's kernel does; no
 * pre-filter); CC_SB_NO_FP32_PREFILTER keeps the batched passes but decides
 * every leaf's emptiness in FP64 only.  All forms give identical criticals,
 * flags and traces (the pre-filter skips FP64 work only where its FP32
 * bounds prove the FP64 test's answer). */
#define CC_SB_NO_FP32_PREFILTER 2
int cc_sb_prove_ex(cc_handle* h, const cc_sb_box* root, const cc_sb_grid* grid, int options, cc_sb_box** criticals,
                   size_t* n_crit, uint32_t** flags, cc_sb_prove_stats* stats);

/* ---- learned strategy ordering (no reference counterpart) ------------------
 * A 10 -> 64 -> 64 -> 7 perceptron per handle: 6 logits, "criterion k
 * certifies the box" (CC_TV_* order), and 1 logit, "no criterion certifies
 * it" (the box must be split).  Parameters, FP32, in this order: W1[10][64],
 * b1[64], W2[64][64], b2[64], W3[64][7], b3[7].  Trained on the GPU by the
 * library's own kernels (Adam on the mean summed binary cross-entropy);
 * inference with BF16 weights and activations, FP32 accumulation, tensor
 * cores.  All array arguments except the weights are DEVICE pointers. */
#define CC_MLP_FEATURES 10
#define CC_MLP_OUTPUTS 7
#define CC_MLP_PARAMS 5319
int cc_mlp_init(cc_handle* h, uint64_t seed);            /* He initialisation, Adam state cleared */
int cc_mlp_set_weights(cc_handle* h, const float* w);    /* host array of CC_MLP_PARAMS */
int cc_mlp_get_weights(cc_handle* h, float* w);          /* host array of CC_MLP_PARAMS */
/* features of n tight boxes (SoA, 10 x n doubles) -> feat[n][10] */
int cc_mlp_features(cc_handle* h, const double* soa, size_t n, float depth, float* feat);
/* gradient of the mean loss over n <= 65536 samples (labels: bit k = target
 * of output k) into grad (host, CC_MLP_PARAMS floats); *loss = the mean loss */
int cc_mlp_gradients(cc_handle* h, const float* feat, const uint32_t* labels, size_t n, float* grad, float* loss);
/* one Adam step (learning rate lr) on the mean loss over n <= 65536 samples */
int cc_mlp_train_step(cc_handle* h, const float* feat, const uint32_t* labels, size_t n, float lr, float* loss);
/* logits[n][8] (column 7 unused) */
int cc_mlp_infer(cc_handle* h, const float* feat, size_t n, float* logits);
/* First-success evaluation of n tight boxes (SoA on the device): the steps
 * of the reference's nesting (r1, r1+r2, r1+r2+r3 criteria, R4/R empty,
 * 2x2, r1+r2+r3 leaf, gaps) until one decides; with learned != 0 the
 * network's most likely criterion runs first and the plain order follows.
 * outcome[i] = deciding step (0..5 criterion, 6 R empty, 7 none: critical)
 * | 0x80 if a trap site was reached; evals[i] (may be NULL) = steps run. */
int cc_tight_first(cc_handle* h, const double* soa, size_t n, int learned, uint8_t* outcome, uint8_t* evals);

/* ---- adaptive refinement (no reference counterpart) ----------------------
 * The near-critical stress workload: n tight boxes (host memory) refined by
 * bisection up to max_depth levels.  Each level runs the certified
 * evaluation of cc_tight_eval on all its boxes (device batches of up to 2^24
 * boxes); a box that a criterion certifies, or whose R or R4 is empty, is
 * done; a box that reached a trap site is kept as critical (flag 1); any
 * other box is bisected at mid = 0.5 lo + 0.5 hi (rounded to nearest; the
 * halves' union is the box) along lambda, r1, r2, r3, r4 in turn by depth
 * (depth mod 5), and both halves go to the next level.  Boxes still
 * undecided at the last level are kept as criticals (flag 2).  A level holds
 * at most max_live boxes (0: 2^26): of the boxes to bisect, the first
 * max_live / 2 in level order go on, the others are kept as criticals
 * (flag 3), which stats->cut and stats->stopped_at_cap report.  The next
 * level lists the halves (lower, upper) in the order of their boxes, and
 * *criticals / *flags (cc_free) come in level order and, within a level, in
 * box order, so a refinement is deterministic.  cc_interrupt stops after the
 * current level.
 *
 * cc_set_refine_order chooses how a level decides its boxes:
 *   CC_REFINE_MASKS        the certified evaluation of all six criteria and
 *                          the emptiness bits (the default);
 *   CC_REFINE_FIRST_PLAIN  first-success evaluation in FP64 (cc_tight_first):
 *                          the criteria in the reference's order until one
 *                          certifies the box;
 *   CC_REFINE_FIRST_LEARNED  the same with the network's most likely criterion
 *                          first (features at the level's depth; needs a
 *                          trained network, cc_mlp_init).
 * A box is decided in every order exactly when some criterion certifies it or
 * R / R4 is empty; only the trap flag can differ (a first-success run stops
 * before a later criterion's trap site). */
#define CC_REFINE_MAX_DEPTH 48
#define CC_REFINE_MASKS 0
#define CC_REFINE_FIRST_PLAIN 1
#define CC_REFINE_FIRST_LEARNED 2
int cc_set_refine_order(cc_handle* h, int order);
typedef struct cc_refine_stats {
    uint64_t live[CC_REFINE_MAX_DEPTH + 1];    /* boxes evaluated at each depth */
    uint64_t decided[CC_REFINE_MAX_DEPTH + 1]; /* of which certified or empty */
    float ms[CC_REFINE_MAX_DEPTH + 1];         /* device time of each depth (CUDA events) */
    int32_t depths_run;
    int32_t stopped_at_cap;                    /* some level cut boxes (flag 3) */
    double seconds;                            /* wall time of the call */
    uint64_t kernel_launches;
    /* queue occupancy per depth (CC_REFINE_MASKS): boxes the FP32 pass left
     * to the FP64 pass, strip-width and gap-width bisection jobs, and FP32
     * "true" verdicts sent to FP64 certification */
    uint64_t fp64_boxes[CC_REFINE_MAX_DEPTH + 1];
    uint64_t cover_jobs[CC_REFINE_MAX_DEPTH + 1];
    uint64_t gaps_jobs[CC_REFINE_MAX_DEPTH + 1];
    uint64_t cert_jobs[CC_REFINE_MAX_DEPTH + 1];
    /* criterion steps run per depth (first-success orders), and the sum over
     * groups of 32 consecutive boxes (one warp of the first-success kernel)
     * of their largest step count: steps / (32 * warp_max_steps) is the
     * share of lanes that work while the warp runs criteria */
    uint64_t steps[CC_REFINE_MAX_DEPTH + 1];
    uint64_t warp_max_steps[CC_REFINE_MAX_DEPTH + 1];
    uint64_t cut[CC_REFINE_MAX_DEPTH + 1];     /* boxes kept as criticals by the population cap */
    int32_t order;
    int32_t pad;
} cc_refine_stats;
int cc_tight_refine(cc_handle* h, const cc_tight_box* boxes, size_t n, int max_depth, size_t max_live,
                    cc_tight_box** criticals, uint32_t** flags, size_t* n_crit, cc_refine_stats* stats);

/* Ask a running proof on this handle to stop (the reference's Ctrl-C
 * behaviour, interrupt.cpp:30-46).  cc_tight_prove stops after the current
 * generation; cc_sb_prove stops inside the current refinement generation and
 * keeps the previous one's result (its initial pass is not interruptible,
 * rectangle_size_bound.cu:325, 341).  Either returns CC_ERR_INTERRUPTED with
 * *criticals and *n_crit set to the result so far. */
void cc_interrupt(cc_handle* h);

void cc_free(void* p);

/* ---- diagnostics (no reference counterpart) ------------------------------ */
/* The device's FP64 directed-rounding primitives on host arrays, for the
 * bit-equality check against a host implementation (op: 0 add, 1 mul, 2 div,
 * 3 sqrt, 4 reciprocal; up: round toward +inf, else toward -inf; b unused for
 * ops 3 and 4). */
int cc_selftest_round(cc_handle* h, int op, int up, const double* a, const double* b, double* out, size_t n);
/* The FP32 enclosures' rounding of doubles to floats (integer operations on
 * the bits) next to the directed conversion instructions: out gets 4 floats
 * per value (rounded down, rounded up, __double2float_rd, __double2float_ru). */
int cc_selftest_round_to_floats(cc_handle* h, const double* x, size_t n, float* out);
/* Equal splits computed with the prover's explicit FMA (out_a) and with the
 * reference's plain expression under nvcc's default contraction (out_b),
 * 2n doubles each (reference: subintervals.hpp:33-43). */
int cc_selftest_subinterval(cc_handle* h, const double* lo, const double* hi, const int* idx, const int* cnt, size_t n,
                            double* out_a, double* out_b);
/* One step of the cover-strip (which = 0) or gaps (which = 1) bisection
 * decided by the FP32 enclosure that runs before the FP64 predicate and by
 * the FP64 predicate itself, for checking that every decided FP32 outcome
 * equals the FP64 one.  args: n rows of 8 doubles, (r1, r2, r3, -, -, -, lo,
 * hi) for strip_width_realizable (r1_r2_r3_strategies.cu:49-67) and (r1, r2,
 * w1, w2, r4, -, lo, hi) for the gap width check
 * (r1_r2_large_r3_r4_gaps_strategy.cu:29-59).  f32_out: the FP32 decision
 * for every width in [lo, hi] at once (-1 undecided, 0 false, 1 true);
 * f64_out: the FP64 predicate at the width lo (0 / 1, plus 2 if it reached a
 * trap site). */
int cc_selftest_bisection_f32(cc_handle* h, int which, const double* args, size_t n, int8_t* f32_out,
                              int8_t* f64_out);
/* The whole cover-strip (which = 0) or gaps (which = 1) bisection of each
 * row, FP32 shortcuts included: rows of 8 doubles as for
 * cc_selftest_bisection_f32, with la_hi in column 6 for the cover strip
 * (r1_r2_r3_strategies.cu:69-94) and (r1, r2, w1, w2, r4) for the gaps
 * (r1_r2_large_r3_r4_gaps_strategy.cu:61-98).  out: the widths; trapped: 1
 * where the bisection reached its iteration cap. */
int cc_selftest_bisection_width(cc_handle* h, int which, const double* args, size_t n, double* out,
                                int8_t* trapped);
/* The FP64 certification run of a tight criterion group (0 r1_strategies,
 * 1 r1_r2_strategies, 2 two_by_two_strategies, 3 the leaf form of
 * r1_r2_r3_strategies) on n boxes in host memory, at the arguments of
 * cc_tight_eval, each with its own call number call[i]: 1-based number of
 * the one can_recurse call evaluated (every other call answers "false"), 0
 * for none, -1 for all (the plain FP64 criterion).  out[i] bit 0 = the
 * criterion holds without reaching a trap site; bit 1 = the same run in the
 * record form the evaluation uses (the chosen call stores its arguments and
 * answers "true", then can_recurse is evaluated on them) certifies it. */
int cc_selftest_certify(cc_handle* h, int group, const cc_tight_box* boxes, const int* call, size_t n,
                        uint8_t* out);
/* Measured FP64 instruction throughput of the device (ops/s; one FP64
 * instruction = one op): chains of directed-rounding add/mul, or of FMA. */
int cc_selftest_fp64_peak(cc_handle* h, int use_fma, double* ops_per_s);
/* Measured instruction throughput of the device in thread instructions per
 * second, the roofline denominators of the evaluation's passes: kind 0 FP64
 * directed add/mul, 1 FP64 FMA, 2 FP32 directed add/mul, 3 FP32 FMA (an FP32
 * FMA warp instruction issues every cycle on each SM sub-partition, so kind
 * 3 / 32 is the warp-instruction issue rate).  Independent chains, 8 per
 * thread, 8 blocks of 256 threads per SM; best of three timed launches. */
int cc_selftest_peak(cc_handle* h, int kind, double* ops_per_s);

#ifdef __cplusplus
}
#endif

#endif

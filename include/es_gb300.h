/*
 * es_gb300.h -- C ABI of the GB300 (sm_103a) Erdős–Selfridge CRT-wheel sieve engine.
 *
 * The library (libes_gb300.so) replaces the device half of the reference engine's
 * GpuSieve object (sieve/gpu_sieve_v9.py:425-568, sieve/gpu_sieve_v11.py, and the word-mask
 * variant sieve/es_word_masks.py:95-162).  The Python host (es_gb300.py) keeps the
 * reference's Plan/GpuSieve surface and binds these entry points with ctypes.
 *
 * Conventions
 *   - Every call returns int: ES_OK (0) or a negative ES_ERR_* code; es_last_error() gives a
 *     one-line message for the calling thread.  Nothing throws across the ABI.
 *   - Buffers passed in are caller-owned and copied before the call returns; contexts and
 *     batches own all of their device memory.
 *   - Launch calls are asynchronous on the context's own CUDA stream; the calls that return
 *     results synchronise that stream first.  One host thread per context.
 *   - Positions are block-relative indices idx = oidx * r0 + d0 in the ORIGINAL inner-ring
 *     order (the reference's out[] contents, sieve/gpu_sieve_v9.py:325,
 *     sieve/es_word_masks.py:44,88).  An "outer index" oidx covers one whole inner ring.
 */
#ifndef ES_GB300_H
#define ES_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ES_ABI_VERSION 1

#define ES_OK 0
#define ES_ERR_ARG (-1)       /* bad argument or descriptor */
#define ES_ERR_CUDA (-2)      /* CUDA runtime error (message in es_last_error) */
#define ES_ERR_OVERFLOW (-3)  /* survivor buffer overflow: count exceeded capacity */
#define ES_ERR_RANGE (-4)     /* outer range outside [0, R/r0) or size limit exceeded */
#define ES_ERR_NOMEM (-5)     /* device or host allocation failed */
#define ES_ERR_STATE (-6)     /* call out of order (e.g. results before a launch) */
#define ES_ERR_NODEV (-7)     /* no CUDA device / device is not sm_103 */

#define ES_LAYOUT_WORDMASK 0  /* phase word-mask tables: 32 candidates per load */
#define ES_LAYOUT_SCALAR 1    /* per-candidate incremental residue + bit-table test */
#define ES_LAYOUT_PAIR 2      /* word-mask tables with each phase's wrapped row beside it: one
                                 load per filter and word (inner rings of <= 64 slots; wider
                                 rings use ES_LAYOUT_WORDMASK) */
#define ES_LAYOUT_SMEM 3      /* word-mask tables of the inner-stage filters copied into shared
                                 memory by every CTA at launch (inner rings of <= 64 slots whose
                                 tables fit beside the scan's own shared memory; otherwise the
                                 launch uses ES_LAYOUT_WORDMASK) */
#define ES_LAYOUT_SMEM_PAIR 4 /* the pair tables of the inner-stage filters copied into shared
                                 memory the same way (one 8- or 16-byte load per filter and word;
                                 otherwise the launch uses ES_LAYOUT_PAIR) */
#define ES_LAYOUT_AUTO 5      /* chosen per launch from the inner-stage tables' bytes: staged word
                                 masks where they fit, else word masks through L1 when they fit
                                 L1 and pair tables would not, else pair tables (rings of three
                                 or more words: word masks); a batch decides per width class */

#define ES_MAX_MASK_FILTERS 8 /* filters evaluated in the inner-ring stage */
#define ES_MAX_Q (1u << 20)   /* filter moduli q = p^t_p must be below 2^20 (k <= 1024) */

typedef struct es_ctx es_ctx;
typedef struct es_batch es_batch;

/* One wheel plan (the reference's Plan, sieve/gpu_sieve_v9.py:344-383), flattened.
 * Rings are in the plan's ring order (ring 0 = inner ring swept per outer index, ring 1 the
 * next-fastest digit, ...); the terms of ring j are (residue * basis_j) mod M for every
 * admissible residue of the ring, in the ring's sorted residue order -- exactly the
 * reference's term_lo/term_hi arrays (sieve/gpu_sieve_v9.py:433-437).  Filters are the
 * residual primes in cascade order with their full-power modulus q = p^t_p and a packed
 * bit table of admissible residues, ceil(q/32) little-endian words each, concatenated
 * (sieve/gpu_sieve_v11.py bit-packed tables). */
typedef struct es_plan_desc {
    uint32_t k;
    uint32_t n_rings;          /* may be 0 (no wheel: M = 1) */
    uint32_t n_filters;
    uint32_t flags;            /* reserved, must be 0 */
    uint64_t M_lo, M_hi;       /* wheel modulus, 1 <= M < 2^126 */
    const uint32_t* radix;     /* [n_rings] admissible residues per ring */
    const uint64_t* term_lo;   /* [sum radix] low 64 bits of the ring terms */
    const uint64_t* term_hi;   /* [sum radix] high 64 bits */
    const uint32_t* filter_q;  /* [n_filters] moduli, each < ES_MAX_Q */
    const uint32_t* allowed;   /* [sum ceil(q/32)] packed admissible-residue bits */
} es_plan_desc;

/* Launch shape and table layout; chosen by the autotuner (es_autotune.py).  None of these
 * changes which candidates pass. */
typedef struct es_tune {
    uint32_t layout;        /* ES_LAYOUT_WORDMASK, _SCALAR, _PAIR, _SMEM, _SMEM_PAIR or _AUTO */
    uint32_t mask_filters;  /* filters in the inner-ring stage, 1..ES_MAX_MASK_FILTERS */
    uint32_t threads;       /* CTA size, multiple of 32 in [64, 512] */
    uint32_t strip;         /* at most this many ring-1 cycles per thread per work unit: the
                               lanes of a warp take 32 consecutive ring-2 rows over one of
                               ceil(r2 / strip) balanced windows of ring-2 digits; lists and
                               plans without a ring 2 take `strip` consecutive entries */
    uint32_t smem_kb;       /* accepted, no effect (the staged layouts size their own shared
                               memory) */
    uint32_t ctas_per_sm;   /* persistent grid = SM count * ctas_per_sm */
    uint32_t count_stages;  /* 1: accumulate per-filter-stage pass counts */
    uint32_t reserved;
} es_tune;

/* One survivor of the full cascade (kernel emit, sieve/gpu_sieve_v9.py:323-326). */
typedef struct es_survivor {
    uint64_t idx;       /* block-relative position index, original inner order */
    uint64_t s_lo;      /* n mod M, low 64 bits */
    uint64_t s_hi;      /* n mod M, high 64 bits */
    uint64_t t;         /* block: n = t*M + s */
    uint32_t item;      /* batch item that produced it (0 for es_launch) */
    uint32_t good;      /* 1 iff n > k + 1 */
} es_survivor;

/* One work item of a persistent batch launch: a block t of one plan and an outer-index range.
 * Items sharing a group form one block-ordered search: a good survivor in block t lets the
 * kernel skip the group's later blocks (t' > t), never blocks <= t. */
typedef struct es_batch_item {
    uint32_t ctx_index;   /* index into the ctx array given to es_batch_create */
    uint32_t group;       /* search group id, < n_items */
    uint64_t t;           /* block index */
    uint64_t o_begin;     /* outer-index range [o_begin, o_end) within [0, R/r0) */
    uint64_t o_end;
} es_batch_item;

/* ---- library ------------------------------------------------------------------------- */
const char* es_last_error(void);
int es_abi_version(void);
/* Device facts for the tuner: SM count, compute capability, opt-in shared memory per CTA. */
int es_device_info(int* sm_count, int* cc_major, int* cc_minor, uint64_t* smem_optin_bytes);
/* The current device's name (NUL-terminated, truncated to cap bytes): part of the tuner's cache key. */
int es_device_name(char* out, uint32_t cap);

/* ---- context: one plan on the device ---------------------------------------------------- */
/* Replaces GpuSieve.__init__ (sieve/gpu_sieve_v9.py:426-498): copies term tables, filter bit
 * tables, and builds every derived table (sorted inner ring, carry-split keys, ring-1/ring-2
 * residue tables, word-mask phase tables) on the host in C++, then uploads them once. */
int es_ctx_create(const es_plan_desc* desc, const es_tune* tune, es_ctx** out);
/* Releases the context's device memory (the reference relied on CuPy garbage collection). */
int es_ctx_destroy(es_ctx* ctx);
int es_ctx_set_tune(es_ctx* ctx, const es_tune* tune);
int es_ctx_get_tune(const es_ctx* ctx, es_tune* tune);
/* Geometry: R/r0 outer indices, inner radix r0, filter count, bytes of derived tables. */
int es_ctx_info(const es_ctx* ctx, uint64_t* n_outer, uint32_t* r0, uint32_t* n_filters,
                uint64_t* table_bytes);
/* Survivor capacity (reference TUNABLES max_survivors, sieve/gpu_sieve_v9.py:107). */
int es_set_capacity(es_ctx* ctx, uint64_t cap);

/* Per-block constants tconst[j] = (t mod q_j)(M mod q_j) mod q_j for every filter; replaces
 * sieve.tconst.set(tconst_h) (harness/run_k.py:102-104, sieve/gpu_sieve_v9.py:512-514). */
int es_set_block(es_ctx* ctx, const uint32_t* tconst, uint32_t n_filters, uint64_t t);
/* Replaces out_n.fill(0) (harness/run_k.py:118, sieve/gpu_sieve_v9.py:515). */
int es_reset_survivors(es_ctx* ctx);
/* Replaces GpuSieve._launch(ostart, ocount) (sieve/gpu_sieve_v9.py:500-506): scans outer
 * indices [ostart, ostart+ocount) of the current block; asynchronous; survivors accumulate
 * until es_reset_survivors. */
int es_launch(es_ctx* ctx, uint64_t ostart, uint64_t ocount);
/* Same scan over an explicit list of outer indices (seeded sub-samples). */
int es_launch_list(es_ctx* ctx, const uint64_t* outer, uint64_t n);
int es_sync(es_ctx* ctx);
/* Replaces int(out_n.get()[0]) (harness/run_k.py:120): synchronises, returns the count of
 * survivors since the last reset (may exceed capacity: then ES_ERR_OVERFLOW on read). */
int es_survivor_count(es_ctx* ctx, uint64_t* n);
/* Replaces out[:n].get() (harness/run_k.py:124): block-relative indices, device order. */
int es_read_survivors(es_ctx* ctx, uint64_t* idx_out, uint64_t cap, uint64_t* n);
int es_read_survivor_records(es_ctx* ctx, es_survivor* out, uint64_t cap, uint64_t* n);
/* Per-filter-stage pass counts since the last es_reset_counts: counts[j] = positions whose
 * n passed filters 0..j of the cascade (order-dependent).  No reference counterpart beyond
 * the docstring estimates (sieve/gpu_sieve_v9.py:1-27); needs tune.count_stages = 1. */
int es_stage_counts(es_ctx* ctx, uint64_t* counts, uint32_t n_filters);
int es_reset_counts(es_ctx* ctx);
/* Block-ordered minimum over the survivors since the last reset: the least n = t*M + s with
 * n > k+1 (replaces the host sort + first good in GpuSieve.search, gpu_sieve_v9.py:551-563;
 * the host still re-verifies it). found = 0 when there is none.  ES_ERR_OVERFLOW when the
 * survivor count exceeded the capacity (dropped records could hold the minimum). */
int es_min_survivor(es_ctx* ctx, int* found, uint64_t* t, uint64_t* s_lo, uint64_t* s_hi);
/* Launch + CUDA-event time of the scan kernel alone (milliseconds), synchronising. */
int es_launch_timed(es_ctx* ctx, uint64_t ostart, uint64_t ocount, float* ms);

/* ---- persistent batch: many (plan, block, range) scans in one work-stealing launch ------- */
int es_batch_create(es_ctx* const* ctxs, uint32_t n_ctx, const es_batch_item* items,
                    uint32_t n_items, const es_tune* tune, es_batch** out);
/* Resets counters and survivors, then runs the persistent scan kernel and the block-ordered
 * min-reduction; use_graph = 1 replays a captured CUDA graph of that sequence. */
int es_batch_run(es_batch* b, int use_graph);
/* Synchronises; ms = device time of the last run (CUDA events around the whole sequence). */
int es_batch_sync(es_batch* b, float* ms);
/* Least good survivor of one search group.  ES_ERR_OVERFLOW when the batch's survivor count
 * exceeded its buffer: *found = 2 and *t = the least block of the group that holds a good
 * survivor (exact, from the scan's own per-group record; UINT64_MAX when none), *s_lo = *s_hi = 0;
 * rescan that group's blocks one at a time to get the survivor itself. */
int es_batch_group_min(es_batch* b, uint32_t group, int* found, uint64_t* t, uint64_t* s_lo,
                       uint64_t* s_hi);
int es_batch_item_counts(es_batch* b, uint32_t item, uint64_t* counts, uint32_t n_filters);
int es_batch_survivors(es_batch* b, es_survivor* out, uint64_t cap, uint64_t* n);
int es_batch_destroy(es_batch* b);

/* ---- no-allocation search ---------------------------------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc (code whose device
 * memory is owned by another framework or a fixed-budget pool, or that must not allocate after
 * start-up): blocks t0 .. t0+n_blocks-1 of an existing context scanned as one block-ordered
 * search in one persistent launch on `stream`, allocating nothing.  The caller passes the outputs:
 * d_out (out_cap survivor records), d_count (1 word, zeroed by the call) and d_min (4 words:
 * found, t, s_lo, s_hi of the least n = t*M + s > k+1).  found = 2 means the survivor count
 * (*d_count) exceeded out_cap and records were dropped: the minimum is then unknown, d_min[1]
 * is the least block holding a good survivor (exact; UINT64_MAX when none) and the caller
 * retries with fewer blocks or a larger buffer.  Scratch lives in a file-scope device
 * array sized for ES_STATIC_MAX_BLOCKS blocks (about 57 KB, held by every GPU that loads the
 * library until exit); larger n_blocks is rejected with ES_ERR_RANGE.  Stage counts are not
 * accumulated.  The first call on a device looks up the scratch array's device address.  The
 * call must not be made while `stream` is capturing (it returns ES_ERR_STATE): its small
 * descriptor copies come from host staging arrays that the next call reuses.  Every call shares
 * the one scratch array, so calls that overlap on the GPU race.  Asynchronous: synchronise
 * `stream` before reading the outputs. */
#define ES_STATIC_MAX_BLOCKS 64
int es_search_blocks_static(const es_ctx* ctx, uint64_t t0, uint32_t n_blocks, es_survivor* d_out,
                            uint64_t out_cap, unsigned long long* d_count, unsigned long long* d_min,
                            void* stream);

/* ---- meet-in-the-middle search ------------------------------------------------------------
 * Replaces the CuPy kernel and driver of sieve/gpu_mitm.py:33-219 (the derivation is
 * harness/mitm_search.py:1-25).  Wheel residues n = (s1 + s2) mod M: s1 sums one term per ring of
 * the large half (decoded from its index in the kernel), s2 one per ring of the small half (held
 * sorted on the device with a directory over its top bits).  A scan tests every n < B of the s1
 * indices given against the residual filters in order and keeps the survivors. */
typedef struct es_mitm es_mitm;
typedef struct es_mitm_desc {
    uint32_t k;
    uint32_t n_rings1;          /* rings of the large half S1 (<= 32), decoded in the kernel */
    uint32_t n_rings2;          /* rings of the small half S2 (<= 32), materialised and sorted */
    uint32_t n_filters;
    uint64_t M_lo, M_hi;        /* wheel modulus, 2 <= M < 2^126 */
    const uint32_t* radix1;     /* [n_rings1] residues per ring */
    const uint64_t* term1_lo;   /* [sum radix1] a * c_p mod M, low 64 bits */
    const uint64_t* term1_hi;
    const uint32_t* radix2;     /* [n_rings2]; |S2| = prod radix2 must stay below 2^31 */
    const uint64_t* term2_lo;
    const uint64_t* term2_hi;
    const uint32_t* filter_q;   /* [n_filters] residual moduli in cascade order */
    const uint32_t* allowed;    /* packed admissible-residue bits, ceil(q/32) words each */
} es_mitm_desc;
/* Builds S2 (every sum mod M, sorted) and its directory on the host and uploads all tables. */
int es_mitm_create(const es_mitm_desc* desc, es_mitm** out);
int es_mitm_destroy(es_mitm* m);
int es_mitm_info(const es_mitm* m, uint64_t* n1, uint64_t* n2);
/* Survivor capacity (default 2^20 records); the reference's out_cap (sieve/gpu_mitm.py:133). */
int es_mitm_set_capacity(es_mitm* m, uint64_t cap);
/* Zeroes the survivor and candidate counters (the reference's d_on.fill(0), gpu_mitm.py:193). */
int es_mitm_reset(es_mitm* m);
/* Every n < B (1 <= B <= M) with s1 index in [s1_begin, s1_end) through the cascade;
 * asynchronous; survivors and the count of n tested accumulate until es_mitm_reset.  A bound
 * with lo + B >= M for lo = (M - s1) mod M wraps to the front of S2 (B = M covers all of S2),
 * as the reference kernel does (gpu_mitm.py:78-85). */
int es_mitm_scan(es_mitm* m, uint64_t B_lo, uint64_t B_hi, uint64_t s1_begin, uint64_t s1_end);
/* Synchronises; survivors as n = n_hi * 2^64 + n_lo in device order, their count and the count
 * of n tested.  ES_ERR_OVERFLOW when the count exceeded the capacity (the reference's
 * SURVIVOR_OVERFLOW, gpu_mitm.py:203-204). */
int es_mitm_results(es_mitm* m, uint64_t* n_lo, uint64_t* n_hi, uint64_t cap, uint64_t* n_surv,
                    uint64_t* n_cand);

/* ---- learned planner: 3-layer FP32 MLP trained and evaluated by this library's kernels -------
 * No counterpart in the reference: it stands in for the knapsack planner's analytic cost
 * estimate (sieve/gpu_sieve_v9.py:187-227 ranks wheels by expected checks only).  Parameters are
 * flat FP32: W1[H][D], b1[H], W2[H][H], b2[H], W3[O][H], b3[O]; loss = mean squared error. */
typedef struct es_mlp es_mlp;
const char* es_mlp_last_error(void);
int es_mlp_create(uint32_t in_dim, uint32_t hidden, uint32_t out_dim, uint64_t seed, es_mlp** out);
int es_mlp_destroy(es_mlp* m);
int es_mlp_num_params(const es_mlp* m, uint64_t* n);
int es_mlp_get_params(es_mlp* m, float* out, uint64_t n);
int es_mlp_set_params(es_mlp* m, const float* in, uint64_t n);   /* also resets the optimiser */
int es_mlp_forward(es_mlp* m, const float* X, uint64_t n, float* Y);
int es_mlp_loss_grad(es_mlp* m, const float* X, const float* T, uint64_t n, float* loss, float* grad);
int es_mlp_train(es_mlp* m, const float* X, const float* T, uint64_t n, uint32_t epochs,
                 uint32_t batch, float lr, uint64_t seed, float* final_loss);

/* ---- measurement -------------------------------------------------------------------------- */
/* Integer peak microbenchmarks over the whole GPU (ops = lanes x instructions, dependent-free
 * chains).  es_int_peak: IADD3 and LOP3 only, the ALU pipe's ceiling.  es_int_peak_mixed: LOP3
 * paired with IMAD (mad.lo.u32, FMA pipe), the two integer pipes together -- the integer
 * ceiling of a kernel such as the scan, which issues both (the roofline denominator). */
int es_int_peak(double* ops_per_s, double* ms);
int es_int_peak_mixed(double* ops_per_s, double* ms);

#ifdef __cplusplus
}
#endif
#endif /* ES_GB300_H */

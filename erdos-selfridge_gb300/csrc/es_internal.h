// Internal layout shared by the host table builder (es_abi.cu) and the kernels (es_scan.cu).
//
// Data layout in HBM (one arena per plan context, uploaded once):
//   small block   contiguous tables staged verbatim into shared memory by every CTA:
//                   T1[r1]      ring-1 terms (128-bit)                      16 B each
//                   K1[r1]      32-bit keys of T1 (ring-1 wrap and split keys) 4 B each
//                   TQ1[r1][8]  ring-1 terms mod q_f, f < 8                  32 B each
//                   D2[r2]      ring-2 step deltas term2[d+1]-term2[d] mod M 16 B each
//                   DQ2[r2][8]  those deltas mod q_f                        32 B each
//                   S0[r0]      inner-ring terms sorted ascending            16 B each
//                   K0[r0]      top-32-bit keys of S0 (carry-split search)    4 B each
//                   I0[r0]      original inner digit of each sorted slot      4 B each
//                   Q0[8][r0]   S0 mod q_f (scalar layout, residue stage)     4 B each
//                   BK[513]     carry-split buckets over the keys' top 9 bits:
//                               first slot at or above the bucket, its key and
//                               the next two keys                            16 B each
//                   FC[nf]      per-filter constants (EsFilterC)             32 B each
//   fast tables   for the first F_built filters: word-mask phase tables
//                   P_f[phi][w] bit i = admissible((phi + S0[32w+i]) mod q_f), q_f rows of
//                   mask_stride words (W, or 4 for W = 3: padded to one 16-byte load)
//   bit tables    every filter's packed admissible-residue bits (ceil(q/32) words)
//   ring terms    all rings' 128-bit terms (decode of rings >= 2 at strip starts)
#pragma once
#include <stdint.h>

#define ES_FMAX 8
#define ES_NBUCKET_LOG2 9
#define ES_NBUCKET (1u << ES_NBUCKET_LOG2)   // carry-split buckets over the 32-bit keys
#define ES_QUEUE_BYTES 2304   // per-warp shared slot: entry queue, lane records, tail context
#define ES_MAX_RINGS 64
#define ES_MAX_FILTERS 192   // pi(1024) = 172 residual primes at most

struct EsFilterC {
    uint32_t q;      // modulus p^t_p (< 2^20)
    uint32_t corr;   // (q - M mod q) mod q: residue correction when a sum wraps mod M
    uint32_t w1;     // 2^32 mod q
    uint32_t w2;     // 2^64 mod q
    uint32_t w3;     // 2^96 mod q
    uint32_t off;    // word offset of this filter's bit table
    uint64_t rcp;    // floor(2^64 / q): Barrett reciprocal for 64-bit residues
};

struct EsInst {
    uint64_t M_lo, M_hi;
    uint64_t n_outer;     // R / r0 outer indices per block
    uint64_t n_cycles;    // n_outer / r1 ring-1 cycles per block
    uint32_t k;
    uint32_t n_rings;     // >= 3 after padding with radix-1 rings
    uint32_t r0, W, r1, r2;
    uint32_t n_filters;
    uint32_t F_built;     // filters with word-mask tables (<= ES_FMAX)
    uint32_t sh;          // key shift: keys = value >> sh (top 32 bits of M's width)
    uint32_t bsh;         // bucket shift: bucket = key >> bsh
    uint32_t tail_mask;   // valid bits of the last inner word
    uint32_t small_bytes; // size of the small block (multiple of 16)
    uint32_t km;          // M >> sh (32-bit key of M)
    // byte offsets inside the small block
    uint32_t o_T1, o_TQ1, o_D2, o_DQ2, o_S0, o_K0, o_I0, o_Q0, o_BK, o_FC, o_K1;
    // word offsets of the fast (word-mask) tables, F_built + 1 entries (prefix sums)
    uint32_t mask_off[ES_FMAX + 1];
    uint32_t mask_stride;            // words per phase row of P_f: W, or 4 for W = 3 (16-byte rows)
    const unsigned char* small;      // device copy of the small block
    const uint32_t* masks;           // word-mask tables
    const uint32_t* pairs;           // pair tables (W <= 2): row phi = P_f[phi], P_f[(phi + corr_f) mod q_f]
    const uint32_t* allowed;         // bit tables of all filters
    const uint64_t* ring_terms;      // [sum radix][2] lo,hi
    const uint32_t* ring_off;        // [n_rings]
    const uint32_t* radix;           // [n_rings]
};

// One work item of a launch, device-resident.
struct EsItem {
    const EsInst* inst;      // device pointer
    const uint32_t* tconst;  // [n_filters] per-block residue constants (device)
    const uint64_t* list;    // explicit outer-index list or nullptr (range mode)
    unsigned long long* counts;  // [n_filters] stage counts (device) or nullptr
    uint64_t t;
    uint64_t o_begin, o_end; // range mode: outer range; list mode: list index range
    uint64_t c_begin, c_end; // range mode: cycle range covering the outer range
    uint64_t unit_begin;     // first global unit of this item
    uint64_t n_units;
    uint32_t group;
    uint32_t inst_id;        // distinct per plan context within a launch
    uint32_t caller;         // the item's index in the caller's list (survivor records carry it)
    uint32_t pad;
};

struct EsLaunch {
    const EsItem* items;
    uint32_t n_items;
    uint32_t threads;
    uint32_t strip;
    uint32_t mask_filters;   // F requested (template F is the rounded-up instance)
    uint64_t total_units;          // warp-units: 32 lanes x <= strip ring-1 cycles (or list entries)
    uint32_t nf_max;               // largest filter count among the launch's plans
    uint32_t direct;               // 1: every item uses one plan (no CTA barriers after staging)
    unsigned long long* unit_counter;     // single-plan launches: next warp-unit
    unsigned long long* item_next;        // several plans: next warp-unit of each item
    struct es_survivor* surv;
    unsigned long long* surv_n;
    uint64_t surv_cap;
    unsigned long long* group_found;  // per group: least block with a good survivor
    uint32_t smem_bytes;              // dynamic shared memory of the launch
    uint32_t cnt_off;                 // byte offset of the per-warp tail-stage counters in smem
    uint32_t queue_off;               // byte offset of the per-warp survivor queues in smem
    uint32_t stage_off;               // byte offset of the staged tables (ES_LAYOUT_SMEM, _SMEM_PAIR)
    // single-plan launches carry their one item and block constants by value
    EsItem item0;
    uint32_t tconst0[ES_MAX_FILTERS];
};

// Scan kernel instances by layout (es_scan_wm.cu / es_scan_wmc.cu, es_scan_pair.cu, es_scan_sc.cu,
// es_scan_sm.cu, es_scan_sp.cu).
typedef void (*ScanFn)(const EsLaunch);
ScanFn es_pick_wordmask_fast(uint32_t words, uint32_t mask_filters);
ScanFn es_pick_wordmask_count(uint32_t words, uint32_t mask_filters);
ScanFn es_pick_pair(int count, uint32_t words, uint32_t mask_filters);
ScanFn es_pick_scalar(int count, uint32_t mask_filters);
ScanFn es_pick_smem(int count, uint32_t words, uint32_t mask_filters);
ScanFn es_pick_smem_pair(int count, uint32_t words, uint32_t mask_filters);

// Host-side launchers implemented in es_scan.cu (return a cudaError_t value).
int es_scan_prepare(int smem_optin_bytes);
// words: inner-ring words per outer index (1, 2, or anything else for the generic instance)
int es_scan_occupancy(int layout, int count, uint32_t words, uint32_t mask_filters, int threads,
                      int smem_bytes, int* ctas_per_sm);
int es_launch_scan(const EsLaunch& L, int layout, int count, uint32_t words, int grid, void* stream);
// group_min: [n_groups][4] = {found, t, s_lo, s_hi}; items == nullptr means one group (0).
// found = 2 flags a survivor count above cap; t is then group_found[g] (or ~0 when null).
int es_launch_min(const struct es_survivor* surv, const unsigned long long* surv_n,
                  uint64_t cap, const EsItem* items, uint32_t n_groups,
                  const unsigned long long* group_found, unsigned long long* group_min,
                  void* stream);
// mix = 0: ALU-pipe probe (IADD3 + LOP3); mix = 1: ALU + FMA-pipe probe (LOP3 + IMAD)
int es_launch_int_peak(unsigned long long* sink, int grid, int threads, int iters, int mix, void* stream);

// The library-wide "last error" message of the calling thread (es_last_error), for translation
// units other than es_abi.cu.
void es_set_last_error(const char* msg);

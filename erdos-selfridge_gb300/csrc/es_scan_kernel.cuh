// The scan kernel of the GB300 Erdős–Selfridge CRT-wheel sieve (sm_103a), as a template that
// es_scan_wm.cu / es_scan_wmc.cu, es_scan_pair.cu and es_scan_sc.cu instantiate (compiled in
// parallel); es_scan.cu holds the dispatch, the min-reduction and the peak probe.
//
// What one launch computes (semantics of the reference kernel, sieve/gpu_sieve_v9.py:240-330,
// sieve/gpu_sieve_v11.py:250-354, sieve/es_word_masks.py:39-92): for every work item (a plan,
// a block t, an outer-index range) and every position idx = oidx*r0 + d0 in the range,
//   n = t*M + ((sum_j term_j[d_j]) mod M)        (mixed radix, ring 0 fastest)
// passes iff (n mod q_f) is admissible for every residual filter f, in cascade order.
// Survivors are emitted with their ORIGINAL inner digit d0; per-stage pass counts are
// accumulated on request.  All arithmetic is exact integer arithmetic.
//
// How it is organised (GB300-first, not the reference's per-plan NVRTC source):
//  * One persistent kernel per launch; warps claim work units from atomic counters (one for a
//    single-plan launch, one per item when a launch holds several plans) -- no spin waits
//    anywhere.  A group's later blocks are skipped once a good survivor is known (block-ordered
//    search).
//  * Two-level strip mining.  A lane owns up to `strip` consecutive ring-1 cycles (cycle index
//    = oidx / r1).  Rings >= 2 give b2 = sum term_j mod M, decoded once per strip and then
//    stepped with a 128-bit delta table when the ring-2 digit advances.  The 32 lanes of a warp
//    take 32 consecutive ring-2 rows over the same window of ring-2 digits, so the per-step
//    delta rows are broadcast loads (lanes on different digits of a 21-digit ring 2 read up to
//    21 rows of a 32-byte stride: a 6-way bank conflict per load).  Ring 1 is swept in a
//    warp-uniform loop (b = b2 + T1[d1], broadcast loads) and ring 0, the inner ring, is
//    handled 32 candidates at a time as bit masks.
//  * 128-bit values are four 32-bit limbs with PTX carry chains; filter residues are carried
//    incrementally in 32-bit arithmetic: BQ_f = n mod q_f for the ring-0 base, updated from
//    precomputed term residues and the wrap correction corr_f = -M mod q_f (the reference's v7
//    identity, sieve/gpu_sieve_v9.py:9-18), reduced with unsigned min instead of branches.
//  * Inner ring: its terms are sorted once on the host, so the wrap (s >= M) is a suffix of the
//    sorted slots; its start (the carry split) comes from 32-bit keys through a 512-bucket
//    table.  Word-mask layout: a filter costs two phase-table loads, P_f[phase] and the row a
//    wrap selects, per word (or per 16-byte row of up to four words); the shared-memory layout
//    is the same with the inner-stage filters' tables copied into shared memory at launch (the
//    random 4- or 8-byte gathers then cost a few bank wavefronts instead of one L1 sector per
//    lane); pair layout: one load that holds both rows; scalar layout: one residue + bit test
//    per live candidate.
//  * Inner words that still hold candidates after the inner-ring stage are queued per warp as
//    one 16-byte entry per lane; a flush takes 32 entries, one candidate per lane (full warps,
//    not single lanes), runs the next filters from 32-bit term residues, and gives only the
//    few candidates left the exact tail: n mod M rebuilt in 128 bits, then limb weights and a
//    Barrett reduction per filter.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/es_gb300.h"
#include "es_internal.h"

namespace {

// 128-bit value as little-endian 32-bit limbs.
struct U4 {
    uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 u4(const uint4 v) { return U4{v.x, v.y, v.z, v.w}; }

__device__ __forceinline__ U4 add128(const U4 a, const U4 b) {
    U4 r;
    asm("add.cc.u32 %0, %4, %8;\n\t"
        "addc.cc.u32 %1, %5, %9;\n\t"
        "addc.cc.u32 %2, %6, %10;\n\t"
        "addc.u32 %3, %7, %11;"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w));
    return r;
}

// r = a - b; borrow = 0xffffffff when a < b, else 0.
__device__ __forceinline__ U4 sub128(const U4 a, const U4 b, uint32_t& borrow) {
    U4 r;
    asm("sub.cc.u32 %0, %5, %9;\n\t"
        "subc.cc.u32 %1, %6, %10;\n\t"
        "subc.cc.u32 %2, %7, %11;\n\t"
        "subc.cc.u32 %3, %8, %12;\n\t"
        "subc.u32 %4, 0, 0;"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w), "=r"(borrow)
        : "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w));
    return r;
}

__device__ __forceinline__ U4 sel128(uint32_t mask, const U4 a, const U4 b) {  // mask ? a : b
    return U4{(a.x & mask) | (b.x & ~mask), (a.y & mask) | (b.y & ~mask), (a.z & mask) | (b.z & ~mask),
              (a.w & mask) | (b.w & ~mask)};
}

// (a + b) mod M for a, b < M < 2^126; wmask = 0xffffffff when M was subtracted.
__device__ __forceinline__ U4 addmod(const U4 a, const U4 b, const U4 M, uint32_t& wmask) {
    const U4 s = add128(a, b);
    uint32_t br;
    const U4 d = sub128(s, M, br);
    wmask = ~br;
    return sel128(br, s, d);
}

__device__ __forceinline__ bool lt128(const U4 a, const U4 b) {
    uint32_t br;
    sub128(a, b, br);
    return br != 0u;
}

__device__ __forceinline__ uint64_t lo64(const U4 a) { return ((uint64_t)a.y << 32) | a.x; }
__device__ __forceinline__ uint64_t hi64(const U4 a) { return ((uint64_t)a.w << 32) | a.z; }

// x mod q for a 128-bit x, q < 2^20: limb weights (2^32i mod q) then one Barrett step.
__device__ __forceinline__ uint32_t mod128(const U4 x, const EsFilterC& f) {
    const uint64_t y = (uint64_t)x.x + (uint64_t)x.y * f.w1 + (uint64_t)x.z * f.w2 + (uint64_t)x.w * f.w3;
    const uint64_t qt = __umul64hi(y, f.rcp);
    uint64_t r = y - qt * f.q;
    if (r >= f.q) r -= f.q;
    return (uint32_t)r;
}

// v mod q for v < 2q (unsigned min: v - q wraps to a huge value when v < q)
__device__ __forceinline__ uint32_t red1(uint32_t v, uint32_t q) { return min(v, v - q); }
// v mod q for v < 3q
__device__ __forceinline__ uint32_t red2(uint32_t v, uint32_t q) { return red1(red1(v, q), q); }

// Phase-table loads: through L1 (read-only path) for tables in global memory, or from shared
// memory (a 32-bit shared address) when the launch staged the tables there (ES_LAYOUT_SMEM).
__device__ __forceinline__ uint32_t lds32(uint32_t saddr) {
    uint32_t v;
    asm("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(saddr));
    return v;
}
__device__ __forceinline__ uint2 lds64(uint32_t saddr) {
    uint2 v;
    asm("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(saddr));
    return v;
}
__device__ __forceinline__ uint4 lds128(uint32_t saddr) {
    uint4 v;
    asm("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(saddr));
    return v;
}

// Volatile shared loads: values the ring-1 sweep needs only on its rare paths are re-read where
// they are used instead of being held in registers across the sweep.
__device__ __forceinline__ uint32_t ldv32(const void* p) {
    uint32_t v;
    asm volatile("ld.volatile.shared.u32 %0, [%1];" : "=r"(v) : "r"((uint32_t)__cvta_generic_to_shared(p)));
    return v;
}
__device__ __forceinline__ U4 ldv128(const void* p) {
    U4 v;
    asm volatile("ld.volatile.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "r"((uint32_t)__cvta_generic_to_shared(p)));
    return v;
}
__device__ __forceinline__ U4 ldv_M(const EsInst& si) {   // M_lo, M_hi are adjacent
    return ldv128(&si.M_lo);
}
// 32 bits of x from bit sh (sh < 96): the carry-split key
__device__ __forceinline__ uint32_t key32(const U4 x, uint32_t sh) {
    const uint32_t kl = sh >> 5, ko = sh & 31u;
    return __funnelshift_r(kl == 0 ? x.x : (kl == 1 ? x.y : x.z), kl == 0 ? x.y : (kl == 1 ? x.z : x.w), ko);
}

// b2 = sum_{j>=2} term_j[d_j] mod M for ring-1 cycle c; also returns the ring-2 digit.
__device__ __noinline__ U4 decode_cycle(const EsInst& I, uint64_t c, const U4 M, uint32_t& d2) {
    uint64_t rem = c;
    U4 acc{0u, 0u, 0u, 0u};
    d2 = 0;
    for (uint32_t j = 2; j < I.n_rings; ++j) {
        const uint32_t r = __ldg(I.radix + j);
        uint64_t d;
        if ((rem >> 32) == 0) {
            const uint32_t r32 = (uint32_t)rem;
            d = r32 % r;
            rem = r32 / r;
        } else {
            d = rem % r;
            rem = rem / r;
        }
        if (j == 2) d2 = (uint32_t)d;
        const uint4 tv = __ldg(reinterpret_cast<const uint4*>(I.ring_terms) + (__ldg(I.ring_off + j) + d));
        uint32_t wm;
        acc = addmod(acc, u4(tv), M, wm);
    }
    return acc;
}

__device__ __forceinline__ void copy_words(uint32_t* dst, const uint32_t* __restrict__ src,
                                           uint32_t nwords) {
    // 16-byte vector copies (both ends 16-byte aligned by construction), then the tail
    const uint32_t n4 = nwords >> 2;
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    for (uint32_t i = threadIdx.x; i < n4; i += blockDim.x) d4[i] = __ldg(s4 + i);
    for (uint32_t i = (n4 << 2) + threadIdx.x; i < nwords; i += blockDim.x) dst[i] = __ldg(src + i);
}

// Everything the flush, the cascade tail and the emit need for one warp-unit.  It lives in the
// warp's slot in shared memory, written once per warp-unit and read only on the flush path, so
// none of it occupies registers across the ring-1 sweep.
struct TailCtx {
    U4 M;
    uint64_t M_lo;
    uint64_t t_blk;
    uint64_t e_base;                   // strip entry of lane 0 (ring-1 cycle or list position)
    const unsigned long long* list;    // outer-index list of the item, or null (a range)
    const uint32_t* tc;
    const uint32_t* allowed_g;
    es_survivor* surv;
    unsigned long long* surv_n;
    unsigned long long* group_found;
    uint64_t surv_cap;
    uint32_t kp1, Feff, FR, nf, wcnt_saddr, item_id, group, r0, r1;
    uint32_t lstride;                  // entries between the strips of consecutive lanes
    bool M_big;
};

// Per-warp queue of inner-word pairs that still hold candidates after the inner-ring stage.  An
// entry is one lane's words w, w+1 of one outer index: {candidate bits of word w, of word w+1,
// d1 | carry split << 16, lane | ring-1 wrap << 5 | w << 6}.
// The lane's ring-1 cycle is described once per strip step by its record (b2 and the residues
// of b2 for the residue-stage filters), so a push is one 16-byte store per lane; the queue is
// drained before the records change.  The flush runs 32 entries at a time (whole warps): first
// the next ES_NRES filters from 32-bit residues (the tables of the inner-ring stage carry them),
// then, for the few candidates left, n mod M and the exact tail.
#define ES_QCAP 64
#define ES_NRES 4
struct EsQueue {
    uint4 ent[ES_QCAP];
    uint4 rec0[32];                    // per lane: b2 (limbs)
    uint4 rec1[32];                    // per lane: residues of b2 + block term (residue stage)
    TailCtx ctx;                       // the warp's current item (see TailCtx)
};
static_assert(sizeof(EsQueue) <= ES_QUEUE_BYTES, "per-warp slot overflows its shared-memory share");

__device__ __forceinline__ void red_add_shared(uint32_t saddr, uint32_t v) {
    // Not visible to the compiler as a store: the counters are read only after a __syncwarp.
    asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(saddr), "r"(v));
}

#ifndef ES_LB_THREADS
#define ES_LB_THREADS 512   // largest CTA the scan kernel is compiled for
#endif
#ifndef ES_LB_MINB
#define ES_LB_MINB 1
#endif

// First F entries of an 8-entry residue row (two 16-byte loads at most).
template <int F>
__device__ __forceinline__ void row8(const uint4* row, uint32_t (&v)[8]) {
    if (F > 0) {
        const uint4 a = row[0];
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    }
    if (F > 4) {
        const uint4 b = row[1];
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    }
}

// exact tail of the cascade for one candidate (filters f0..nf-1), then the emit
template <bool COUNT>
__device__ __forceinline__ void tail_one(const TailCtx& C, const EsFilterC* sFC, uint32_t f0, const U4 s,
                                         uint64_t idx) {
    for (uint32_t f = f0; f < C.nf; ++f) {
        const EsFilterC fc = sFC[f];
        uint32_t r = mod128(s, fc) + C.tc[f];
        if (r >= fc.q) r -= fc.q;
        const uint32_t wv = __ldg(C.allowed_g + fc.off + (r >> 5));
        if (!((wv >> (r & 31u)) & 1u)) return;
        if (COUNT) red_add_shared(C.wcnt_saddr + 4u * f, 1u);
    }
    bool good;
    if (C.M_big) {
        good = (C.t_blk > 0) || s.w || s.z || s.y || (s.x > C.kp1);
    } else {
        const uint64_t n = C.t_blk * C.M_lo + s.x;   // M <= k+1 <= 1025: n fits easily
        good = n > C.kp1;
    }
    const unsigned long long slot = atomicAdd(C.surv_n, 1ull);
    if (slot < C.surv_cap) {
        es_survivor* rec = C.surv + slot;
        rec->idx = idx;
        rec->s_lo = lo64(s);
        rec->s_hi = hi64(s);
        rec->t = C.t_blk;
        rec->item = C.item_id;
        rec->good = good ? 1u : 0u;
    }
    if (good && C.group_found) atomicMin(C.group_found + C.group, (unsigned long long)C.t_blk);
}

// warp-uniform: one pass over up to 32 queued entries.  Each lane takes the lowest candidate of
// its entry (the rest of the entry goes back on the queue), so the residue stage runs converged
// and the warp leaves it as soon as no lane has a live candidate; the few candidates left take
// n mod M and the exact tail.
// Entry formats: words (w, w + 1) of one ring-1 digit: {bits of w, bits of w + 1, d1 | split <<
// 16, lane | wrap << 5 | w << 6}; or, with PD (one-word inner rings), the words of two
// consecutive digits d1, d1 + 1: {bits of d1, bits of d1 + 1, d1 | split(d1) << 16 |
// split(d1 + 1) << 24, lane | wrap(d1) << 5 | wrap(d1 + 1) << 6}.
template <bool COUNT, bool PD>
__device__ __forceinline__ void flush(EsQueue* Q, const unsigned char* smem, const EsInst& si, uint32_t lane,
                                      uint32_t step, uint32_t& qhead, uint32_t& qsize) {
    __syncwarp();
    const TailCtx& C = Q->ctx;
    const uint4* sT1 = reinterpret_cast<const uint4*>(smem + si.o_T1);
    const uint4* sS0 = reinterpret_cast<const uint4*>(smem + si.o_S0);
    const uint32_t* sI0 = reinterpret_cast<const uint32_t*>(smem + si.o_I0);
    const uint32_t* sTQ1 = reinterpret_cast<const uint32_t*>(smem + si.o_TQ1);
    const uint32_t* sQ0 = reinterpret_cast<const uint32_t*>(smem + si.o_Q0);
    const EsFilterC* sFC = reinterpret_cast<const EsFilterC*>(smem + si.o_FC);
    const uint32_t n = qsize < 32u ? qsize : 32u;
    const uint4 en = Q->ent[(qhead + lane) & (ES_QCAP - 1)];
    const uint64_t bits = lane < n ? ((uint64_t)en.y << 32) | en.x : 0ull;
    const uint64_t rest = bits & (bits - 1ull);
    const uint32_t back = __ballot_sync(0xffffffffu, rest != 0u);
    __syncwarp();   // every lane holds its entry before any slot is reused
    qhead = (qhead + n) & (ES_QCAP - 1);
    qsize -= n;
    if (rest) {
        // lands on a free or just-consumed slot: qsize - n + popc(back) <= old qsize < ES_QCAP
        const uint32_t pos = (qhead + qsize + __popc(back & ((1u << lane) - 1u))) & (ES_QCAP - 1);
        Q->ent[pos] = make_uint4((uint32_t)rest, (uint32_t)(rest >> 32), en.z, en.w);
    }
    qsize += __popc(back);
    const bool has = bits != 0ull;
    const uint32_t i = has ? __ffsll((long long)bits) - 1u : 0u;
    const uint32_t hw = PD ? (i >> 5) : 0u;        // PD: the candidate is in the second digit's word
    const uint32_t d1 = has ? (en.z & 0xffffu) + hw : 0u;
    const uint32_t slot = has ? (PD ? (i & 31u) : ((en.w >> 6) << 5) + i) : 0u;
    const uint32_t own = has ? (en.w & 31u) : 0u;
    const bool wrap1 = has && ((en.w >> (5u + hw)) & 1u);
    const uint32_t split = PD ? (hw ? (en.z >> 24) : ((en.z >> 16) & 0xffu)) : (en.z >> 16);
    const bool cw = has && slot >= split;          // sorted slots from the split on wrap past M
    // lanes without an entry run the residue stage's loads too: give them zero residues, not
    // another lane's record (lane 0 of a unit may not have reached its first cycle yet)
    const uint4 bq = has ? Q->rec1[own] : make_uint4(0u, 0u, 0u, 0u);
    const uint32_t bqv[ES_NRES] = {bq.x, bq.y, bq.z, bq.w};
    const uint32_t f0 = C.Feff, fr = C.FR, r0 = C.r0;
    bool ok = has;
#pragma unroll
    for (uint32_t j = 0; j < ES_NRES; ++j) {
        const uint32_t f = f0 + j;
        if (f < fr && __any_sync(0xffffffffu, ok)) {
            const EsFilterC& fc = sFC[f];
            const uint32_t q = fc.q, corr = fc.corr;
            // n mod q_f = b2 + T1[d1] + S0[slot] mod q_f, with -M mod q_f per wrap
            uint32_t x = red2(bqv[j] + sTQ1[d1 * ES_FMAX + f] + (wrap1 ? corr : 0u), q);
            x = red2(x + sQ0[f * r0 + slot] + (cw ? corr : 0u), q);
            const uint32_t wv = __ldg(C.allowed_g + fc.off + (x >> 5));
            ok = ok && ((wv >> (x & 31u)) & 1u);
            if (COUNT && ok) red_add_shared(C.wcnt_saddr + 4u * f, 1u);
        }
    }
    if (ok) {
        uint32_t wm;
        const U4 b = addmod(u4(Q->rec0[own]), u4(sT1[d1]), C.M, wm);
        const U4 s = addmod(b, u4(sS0[slot]), C.M, wm);
        const uint64_t e = C.e_base + (uint64_t)own * C.lstride + step;
        const uint64_t oidx = C.list ? __ldg(C.list + e) : e * C.r1 + d1;
        tail_one<COUNT>(C, sFC, fr, s, oidx * (uint64_t)r0 + sI0[slot]);
    }
    __syncwarp();
}

// warp-uniform (has = ballot of (lo | hi) != 0, nonzero; qsize < 32 on entry): queue the entry
// {lo, hi, ez, ew} (formats above flush) of every lane that has candidates, then flush while 32
// entries are waiting
template <bool COUNT, bool PD>
__device__ __forceinline__ void push(EsQueue* Q, const unsigned char* smem, const EsInst& si, uint32_t lane,
                                     uint32_t step, uint32_t& qhead,
                                     uint32_t& qsize, uint32_t has, uint32_t lo, uint32_t hi,
                                     uint32_t ez, uint32_t ew) {
    if (lo | hi) {
        const uint32_t pos = (qhead + qsize + __popc(has & ((1u << lane) - 1u))) & (ES_QCAP - 1);
        Q->ent[pos] = make_uint4(lo, hi, ez, ew);
    }
    qsize += __popc(has);
    // each pass retires one candidate per lane, so this ends
    while (qsize >= 32u) flush<COUNT, PD>(Q, smem, si, lane, step, qhead, qsize);
}

// entry fields of the words (wd, wd + 1) of digit d1
__device__ __forceinline__ uint32_t ent_z(uint32_t d1, uint32_t split) { return d1 | (split << 16); }
__device__ __forceinline__ uint32_t ent_w(uint32_t lane, uint32_t wm1, uint32_t wd) {
    return lane | (wm1 & 32u) | (wd << 6);
}

// The exact carry split of digit d1 for a lane whose key difference sits in the +-1 band (or ties
// with A): b = b2 + T1[d1] in 128 bits, thr = M - b, then the first sorted slot whose term is
// >= thr, found from the bucket of thr's key (S0[r0] = M stops the walk).  Also returns the
// exact ring-1 wrap in wm1.  It runs for a tiny share of (lane, digit) pairs; one-word rings
// call it out of line (rare_split_call), which frees registers in their sweep (+1.9 % at
// k = 300), while wider rings keep it inline (out of line they lose 1-3 %).
__device__ __forceinline__ uint32_t rare_split(EsQueue* Q, const unsigned char* smem, const EsInst& si, uint32_t lane,
                                               uint32_t d1, uint32_t bsh, uint32_t& wm1) {
    uint32_t wx, brw;
    const U4 Mr = ldv_M(si);
    const U4 b = addmod(ldv128(&Q->rec0[lane]), ldv128(smem + ldv32(&si.o_T1) + 16u * d1), Mr, wx);
    wm1 = wx;
    const U4 thr = sub128(Mr, b, brw);
    const uint32_t te = key32(thr, ldv32(&si.sh));
    const uint32_t* rK0 = reinterpret_cast<const uint32_t*>(smem + ldv32(&si.o_K0));
    const uint4* rS0 = reinterpret_cast<const uint4*>(smem + ldv32(&si.o_S0));
    const uint4* sBK = reinterpret_cast<const uint4*>(smem + si.o_BK);
    uint32_t split = sBK[te >> bsh].x;
    while (rK0[split] < te) ++split;
    while (rK0[split] == te && lt128(u4(rS0[split]), thr)) ++split;
    return split;
}
__device__ __noinline__ uint32_t rare_split_call(EsQueue* Q, const unsigned char* smem, const EsInst& si,
                                                 uint32_t lane, uint32_t d1, uint32_t bsh, uint32_t& wm1) {
    return rare_split(Q, smem, si, lane, d1, bsh, wm1);
}

// Warp-uniform: scan one warp-unit w of `item`, whose plan is staged in smem / si.
template <int F, int LAYOUT, bool COUNT, int WT>
__device__ __forceinline__ void scan_unit(const EsLaunch& L, const EsInst& si, unsigned char* smem,
                                          EsQueue* Q, uint32_t* wcnt,
                                          uint32_t wcnt_saddr, uint32_t lane, unsigned long long w,
                                          const EsItem& item, uint32_t item_id) {
    const U4 M{(uint32_t)si.M_lo, (uint32_t)(si.M_lo >> 32), (uint32_t)si.M_hi, (uint32_t)(si.M_hi >> 32)};
    const EsFilterC* sFC = reinterpret_cast<const EsFilterC*>(smem + si.o_FC);
    const uint32_t* tcv = L.items ? item.tconst : L.tconst0;
    const uint32_t nf = si.n_filters;
    const uint32_t r0 = si.r0, r1 = si.r1, r2 = si.r2;
    // words per inner ring (WT = 4 serves rings of three and four words) and per phase-table row
    const uint32_t Wn = (WT == 1 || WT == 2) ? (uint32_t)WT : si.W;
    const uint32_t RSn = (WT == 1 || WT == 2) ? (uint32_t)WT : (WT == 4 ? 4u : si.mask_stride);
    const uint32_t bsh = si.bsh, tail = si.tail_mask;
    const uint32_t* __restrict__ masks_g = si.masks;
    const uint4* sTQ1 = reinterpret_cast<const uint4*>(smem + si.o_TQ1);
    const uint4* sD2 = reinterpret_cast<const uint4*>(smem + si.o_D2);
    const uint4* sDQ2 = reinterpret_cast<const uint4*>(smem + si.o_DQ2);
    const uint32_t* sDQ2w = reinterpret_cast<const uint32_t*>(sDQ2);
    const uint32_t* sQ0 = reinterpret_cast<const uint32_t*>(smem + si.o_Q0);
    const uint4* sBK = reinterpret_cast<const uint4*>(smem + si.o_BK);   // {slot, 3 keys}
    const uint32_t* sK1 = reinterpret_cast<const uint32_t*>(smem + si.o_K1);
    const uint32_t KM = si.km;
    const uint64_t ob = item.o_begin, oe = item.o_end;
    const uint64_t* list = item.list;
    // word-mask: exactly F filters in the inner-ring stage (the host guarantees F <= filters and
    // F <= tables built); scalar: a runtime count Feff <= F
    uint32_t Feff = (uint32_t)F;
    if (LAYOUT == ES_LAYOUT_SCALAR) {
        if (Feff > L.mask_filters) Feff = L.mask_filters;
        if (Feff > nf) Feff = nf;
    }
    // residue stage: the next ES_NRES filters that carry 32-bit term residues
    const uint32_t FR = min(si.F_built, Feff + ES_NRES) > Feff ? min(si.F_built, Feff + ES_NRES) : Feff;
    // This unit's entries.  Ranges with a ring 2: unit u is ring-2 rows row0 + 32*(u / J) + lane
    // (lane by lane) over the digit window [j*r2/J, (j+1)*r2/J), j = u mod J, J = ceil(r2 /
    // strip) (J windows of at most `strip` digits, balanced); cycles outside [c_begin, c_end) are
    // skipped.  Lists, and ranges without a ring 2: `strip` consecutive entries per lane, lane
    // after lane.
    const uint64_t u = w - item.unit_begin;
    uint64_t e_base, e_lo, e_min, e_hi;
    uint32_t lstride, nsteps;
    if (!list && r2 > 1u) {
        const uint32_t J = (r2 + L.strip - 1u) / L.strip;
        const uint64_t rb = u / J;
        const uint32_t j = (uint32_t)(u - rb * J);
        const uint32_t wlo = j * r2 / J;
        nsteps = (j + 1u) * r2 / J - wlo;
        lstride = r2;
        e_base = (item.c_begin / r2 + rb * 32ull) * r2 + wlo;
        e_lo = e_base + (uint64_t)lane * r2;
        e_min = max(e_lo, item.c_begin);
        e_hi = min(e_lo + nsteps, item.c_end);
    } else {
        nsteps = L.strip;
        lstride = L.strip;
        e_base = (list ? ob : item.c_begin) + u * 32ull * L.strip;
        e_lo = e_min = e_base + (uint64_t)lane * L.strip;
        e_hi = min(e_lo + L.strip, list ? oe : item.c_end);
    }
    TailCtx& C = Q->ctx;
    if (lane == 0) {
        C.M = M;
        C.M_lo = si.M_lo;
        C.kp1 = si.k + 1u;
        C.M_big = (si.M_hi != 0) || (si.M_lo > C.kp1);
        C.nf = nf;
        C.r0 = si.r0;
        C.tc = tcv;
        C.allowed_g = si.allowed;
        C.surv = L.surv;
        C.surv_n = L.surv_n;
        C.group_found = L.group_found;
        C.surv_cap = L.surv_cap;
        C.wcnt_saddr = wcnt_saddr;
        C.item_id = item.caller;
        C.group = item.group;
        C.t_blk = item.t;
        C.Feff = Feff;
        C.FR = FR;
        C.r1 = si.r1;
        C.lstride = lstride;
        C.list = reinterpret_cast<const unsigned long long*>(item.list);
        C.e_base = e_base;
    }
    __syncwarp();
    constexpr int FA = F > 0 ? F : 1;   // array extent
    // word-mask phase tables, in global memory or staged in shared memory by the launch
    constexpr bool WMASK = LAYOUT == ES_LAYOUT_WORDMASK || LAYOUT == ES_LAYOUT_SMEM;
    constexpr bool PAIRL = LAYOUT == ES_LAYOUT_PAIR || LAYOUT == ES_LAYOUT_SMEM_PAIR;
    // one-word inner rings on the word-by-word path queue two ring-1 digits per entry
    constexpr bool PD = WT == 1 && !PAIRL;
    uint32_t pbits = 0u, psplit = 0u, pwrap = 0u;   // PD: the even digit's word, waiting
    uint32_t qf[FA], corr[FA];
    const uint32_t* tab[FA];
    uint32_t tabs[FA];   // shared address of each staged table (ES_LAYOUT_SMEM, ES_LAYOUT_SMEM_PAIR)
#pragma unroll
    for (int f = 0; f < F; ++f) {
        const bool on = (uint32_t)f < Feff;
        qf[f] = on ? sFC[f].q : 1u;
        corr[f] = on ? sFC[f].corr : 0u;
        tab[f] = LAYOUT == ES_LAYOUT_WORDMASK ? masks_g + si.mask_off[f]
                 : PAIRL                      ? si.pairs + 2u * si.mask_off[f]
                                              : si.allowed + (on ? sFC[f].off : 0u);
        tabs[f] = (uint32_t)__cvta_generic_to_shared(smem + L.stage_off) +
                  4u * (LAYOUT == ES_LAYOUT_SMEM_PAIR ? 2u : 1u) * si.mask_off[f];
    }
    uint32_t cnt[FA];
#pragma unroll
    for (int f = 0; f < FA; ++f) cnt[f] = 0u;
    uint32_t qhead = 0, qsize = 0;

    uint32_t d2 = 0;
    uint32_t BQ2[FA];
#pragma unroll
    for (int f = 0; f < FA; ++f) BQ2[f] = 0u;
    bool have = false;
    uint64_t prev_c = 0;
    // every lane runs the unit's steps so the warp-wide votes below see 32 lanes
    for (uint32_t step = 0; step < nsteps; ++step) {
        const uint64_t e = e_lo + step;
        const bool live = e >= e_min && e < e_hi;
        if (__ballot_sync(0xffffffffu, e < e_hi) == 0u) break;   // no lane has entries left
        uint64_t c = prev_c;
        uint32_t lo1 = 0u, hi1 = 0u;
        // b2 of the lane's last cycle lives in its record (0 before the first decode)
        const U4 Mv = ldv_M(si);
        U4 b2 = have ? ldv128(&Q->rec0[lane]) : U4{0u, 0u, 0u, 0u};
        if (live) {
            if (list) {
                const uint64_t o = __ldg(reinterpret_cast<const unsigned long long*>(list) + e);
                c = o / r1;
                lo1 = (uint32_t)(o - c * r1);
                hi1 = lo1 + 1u;
            } else {
                c = e;
                const uint64_t o0 = c * r1;
                lo1 = ob > o0 ? (uint32_t)(ob - o0) : 0u;
                const uint64_t span = oe - o0;
                hi1 = span < r1 ? (uint32_t)span : r1;
            }
            // rings >= 2: one delta step while the ring-2 digit advances, else a decode
            if (have && c == prev_c + 1 && d2 + 1u < r2) {
                uint32_t wm;
                b2 = addmod(b2, u4(sD2[d2]), Mv, wm);
                uint32_t dq[8];
                row8<F>(sDQ2 + d2 * (ES_FMAX / 4), dq);
#pragma unroll
                for (int f = 0; f < F; ++f) BQ2[f] = red2(BQ2[f] + dq[f] + (corr[f] & wm), qf[f]);
                // this lane's record: b2 and the residue-stage residues, stepped the same way
                const uint4 rq = Q->rec1[lane];
                uint32_t rv[ES_NRES] = {rq.x, rq.y, rq.z, rq.w};
#pragma unroll
                for (uint32_t j = 0; j < ES_NRES; ++j) {
                    const uint32_t f = Feff + j;
                    if (f < FR) rv[j] = red2(rv[j] + sDQ2w[d2 * ES_FMAX + f] + (sFC[f].corr & wm), sFC[f].q);
                }
                Q->rec0[lane] = make_uint4(b2.x, b2.y, b2.z, b2.w);
                Q->rec1[lane] = make_uint4(rv[0], rv[1], rv[2], rv[3]);
                ++d2;
            } else if (!(have && c == prev_c)) {
                b2 = decode_cycle(si, c, Mv, d2);
#pragma unroll
                for (int f = 0; f < F; ++f) {
                    if ((uint32_t)f < Feff) BQ2[f] = red1(mod128(b2, sFC[f]) + tcv[f], qf[f]);
                }
                uint32_t rv[ES_NRES] = {0u, 0u, 0u, 0u};
#pragma unroll
                for (uint32_t j = 0; j < ES_NRES; ++j) {
                    const uint32_t f = Feff + j;
                    if (f < FR) rv[j] = red1(mod128(b2, sFC[f]) + tcv[f], sFC[f].q);
                }
                Q->rec0[lane] = make_uint4(b2.x, b2.y, b2.z, b2.w);
                Q->rec1[lane] = make_uint4(rv[0], rv[1], rv[2], rv[3]);
                have = true;
            }
            prev_c = c;
        }
        // the inner-stage residues with the ring-1 wrap correction added, once per cycle
        uint32_t BQ2c[FA];
#pragma unroll
        for (int f = 0; f < FA; ++f) BQ2c[f] = red1(BQ2[f] + corr[f], qf[f]);
        // A = M - b2 and its 32-bit key, once per ring-1 cycle
        uint32_t brA;
        const uint32_t KA = key32(sub128(Mv, b2, brA), ldv32(&si.sh));

        // ---- ring 1: warp-uniform sweep (broadcast loads) --------------------------------
        // one-word rings with at most four inner filters: two digits per iteration give the
        // scheduler independent chains (+2.4 % at k = 300); elsewhere it spills or loses
#pragma unroll(WT == 1 && F <= 4 ? 2 : 1)
        for (uint32_t d1 = 0; d1 < r1; ++d1) {
            const bool act = (d1 - lo1) < (hi1 - lo1);          // lo1 <= d1 < hi1
            // ring-1 wrap (b2 + T1 >= M, i.e. T1 >= A) from the 32-bit keys
            const uint32_t k1 = sK1[d1];
            uint32_t wm1 = k1 > KA ? 0xffffffffu : 0u;
            uint32_t tq[8];
            row8<F>(sTQ1 + d1 * (ES_FMAX / 4), tq);
            // carry split of the inner ring: slots [split, r0) wrap past M.  Away from a key tie,
            // t is the key of thr = M - b to within +-1 and fits 32 bits (0 <= t <= KM); keys
            // below t-1 are certainly below thr, keys above t+1 certainly not.
            const uint32_t t = KA - k1 + (KM & wm1);          // KM - (k1 - KA) on a wrap
            const uint32_t tl = max(t, 1u) - 1u;
            const uint32_t th = min(t, 0xfffffffeu) + 1u;
            // the bucket of tl holds its first slot and the next three keys (sorted): the split
            // is that slot plus the keys below tl among the first two
            const uint4 bk = sBK[tl >> bsh];
            const bool s1 = bk.y < tl, s2 = bk.z < tl;
            uint32_t split = bk.x + (s1 ? 1u : 0u) + (s2 ? 1u : 0u);
            const uint32_t ks = s2 ? bk.w : (s1 ? bk.z : bk.y);   // key of slot `split`
            // rare: a key tie with A, a key inside the +-1 band, or a crowded bucket -> exact
            // (only lanes with candidates here: their record holds b2)
            const bool rare = act && ((k1 == KA) || (ks <= th));
            if (__any_sync(0xffffffffu, rare)) {
                if (rare)
                    split = WT == 1 ? rare_split_call(Q, smem, si, lane, d1, bsh, wm1)
                                    : rare_split(Q, smem, si, lane, d1, bsh, wm1);
            }

            if (PAIRL) {
                // pair tables: the row of phase x0 holds the masks for both sides of the carry
                // split, so a filter costs one load (8 B for one word, 16 B for two)
                uint32_t b0 = act ? (WT == 1 ? tail : 0xffffffffu) : 0u, b1 = act && WT == 2 ? tail : 0u;
                const uint32_t cm0 = __funnelshift_lc(0u, 0xffffffffu, split) & (WT == 1 ? tail : 0xffffffffu);
                const uint32_t cm1 = __funnelshift_lc(0u, 0xffffffffu, max(split, 32u) - 32u) & tail;
#pragma unroll
                for (int f = 0; f < F; ++f) {
                    const uint32_t x0 = red1((wm1 ? BQ2c[f] : BQ2[f]) + tq[f], qf[f]);
                    if (WT == 1) {
                        const uint2 m = LAYOUT == ES_LAYOUT_SMEM_PAIR ? lds64(tabs[f] + 8u * x0)
                                                                      : __ldg(reinterpret_cast<const uint2*>(tab[f]) + x0);
                        b0 &= (m.x & ~cm0) | (m.y & cm0);
                    } else {
                        const uint4 m = LAYOUT == ES_LAYOUT_SMEM_PAIR ? lds128(tabs[f] + 16u * x0)
                                                                      : __ldg(reinterpret_cast<const uint4*>(tab[f]) + x0);
                        b0 &= (m.x & ~cm0) | (m.z & cm0);
                        b1 &= (m.y & ~cm1) | (m.w & cm1);
                    }
                    if (COUNT) cnt[f] += __popc(b0) + __popc(b1);
                }
                const uint32_t has = __ballot_sync(0xffffffffu, (b0 | b1) != 0u);
                if (has) push<COUNT, PD>(Q, smem, si, lane, step, qhead, qsize, has, b0, b1, ent_z(d1, split), ent_w(lane, wm1, 0u));
                continue;
            }
            if (WMASK && WT == 4) {
                // three or four inner words: rows padded to four words, so each side of the
                // carry split is one 16-byte load per filter; two pair entries per outer index
                uint32_t b[4], cmw[4];
#pragma unroll
                for (uint32_t w = 0; w < 4; ++w) {
                    const uint32_t valid = w + 1u < Wn ? 0xffffffffu : (w + 1u == Wn ? tail : 0u);
                    b[w] = act ? valid : 0u;
                    cmw[w] = __funnelshift_lc(0u, 0xffffffffu, max(split, 32u * w) - 32u * w) & valid;
                }
#pragma unroll
                for (int f = 0; f < F; ++f) {
                    const uint32_t x0 = red1((wm1 ? BQ2c[f] : BQ2[f]) + tq[f], qf[f]);
                    const uint32_t x1 = red1(x0 + corr[f], qf[f]);
                    const uint4 m0 = __ldg(reinterpret_cast<const uint4*>(tab[f]) + x0);
                    const uint4 m1 = __ldg(reinterpret_cast<const uint4*>(tab[f]) + x1);
                    b[0] &= (m0.x & ~cmw[0]) | (m1.x & cmw[0]);
                    b[1] &= (m0.y & ~cmw[1]) | (m1.y & cmw[1]);
                    b[2] &= (m0.z & ~cmw[2]) | (m1.z & cmw[2]);
                    b[3] &= (m0.w & ~cmw[3]) | (m1.w & cmw[3]);
                    if (COUNT) cnt[f] += __popc(b[0]) + __popc(b[1]) + __popc(b[2]) + __popc(b[3]);
                }
                const uint32_t h0 = __ballot_sync(0xffffffffu, (b[0] | b[1]) != 0u);
                if (h0) push<COUNT, PD>(Q, smem, si, lane, step, qhead, qsize, h0, b[0], b[1], ent_z(d1, split), ent_w(lane, wm1, 0u));
                const uint32_t h1 = __ballot_sync(0xffffffffu, (b[2] | b[3]) != 0u);
                if (h1) push<COUNT, PD>(Q, smem, si, lane, step, qhead, qsize, h1, b[2], b[3], ent_z(d1, split), ent_w(lane, wm1, 2u));
                continue;
            }
            if (WMASK && WT == 2) {
                // two inner words: both words of a phase are adjacent in P_f, so one 8-byte load
                // per filter and phase serves them, and the pair is queued as one entry
                uint32_t b0 = act ? 0xffffffffu : 0u, b1 = act ? tail : 0u;
                const uint32_t cm0 = __funnelshift_lc(0u, 0xffffffffu, split);
                const uint32_t cm1 = __funnelshift_lc(0u, 0xffffffffu, max(split, 32u) - 32u) & tail;
#pragma unroll
                for (int f = 0; f < F; ++f) {
                    const uint32_t x0 = red1((wm1 ? BQ2c[f] : BQ2[f]) + tq[f], qf[f]);
                    const uint32_t x1 = red1(x0 + corr[f], qf[f]);
                    const uint2 m0 = LAYOUT == ES_LAYOUT_SMEM ? lds64(tabs[f] + 8u * x0)
                                                              : __ldg(reinterpret_cast<const uint2*>(tab[f]) + x0);
                    const uint2 m1 = LAYOUT == ES_LAYOUT_SMEM ? lds64(tabs[f] + 8u * x1)
                                                              : __ldg(reinterpret_cast<const uint2*>(tab[f]) + x1);
                    b0 &= (m0.x & ~cm0) | (m1.x & cm0);
                    b1 &= (m0.y & ~cm1) | (m1.y & cm1);
                    if (COUNT) cnt[f] += __popc(b0) + __popc(b1);
                }
                const uint32_t has = __ballot_sync(0xffffffffu, (b0 | b1) != 0u);
                if (has) push<COUNT, PD>(Q, smem, si, lane, step, qhead, qsize, has, b0, b1, ent_z(d1, split), ent_w(lane, wm1, 0u));
                continue;
            }
            uint32_t lo = 0u;   // bits of an even word, queued with the odd word after it
            for (uint32_t wd = 0; wd < Wn; ++wd) {
                const uint32_t valid = (wd + 1u == Wn) ? tail : 0xffffffffu;
                uint32_t bits = act ? valid : 0u;
                const uint32_t base = wd << 5;
                // slots >= split of this word wrap: all-ones shifted left by (split - base) in [0, 32]
                const uint32_t cm = __funnelshift_lc(0u, 0xffffffffu, max(split, base) - base) & valid;
                if (WMASK) {
                    // straight-line cascade: two table loads per filter per 32 candidates
#pragma unroll
                    for (int f = 0; f < F; ++f) {
                        const uint32_t x0 = red1((wm1 ? BQ2c[f] : BQ2[f]) + tq[f], qf[f]);   // n mod q_f, ring-0 base
                        const uint32_t x1 = red1(x0 + corr[f], qf[f]);                      // the same after a wrap
                        const uint32_t m0 = LAYOUT == ES_LAYOUT_SMEM ? lds32(tabs[f] + 4u * (x0 * RSn + wd))
                                                                     : __ldg(tab[f] + x0 * RSn + wd);
                        const uint32_t m1 = LAYOUT == ES_LAYOUT_SMEM ? lds32(tabs[f] + 4u * (x1 * RSn + wd))
                                                                     : __ldg(tab[f] + x1 * RSn + wd);
                        bits &= (m0 & ~cm) | (m1 & cm);
                        if (COUNT) cnt[f] += __popc(bits);
                    }
                } else {
                    bool alive = true;   // warp-uniform: some lane still has a live candidate
#pragma unroll
                    for (int f = 0; f < F; ++f) {
                        if (alive && (uint32_t)f < Feff) {
                            const uint32_t bqf = red1((wm1 ? BQ2c[f] : BQ2[f]) + tq[f], qf[f]);
                            uint32_t nb = 0u, live_bits = bits;
                            while (live_bits) {
                                const uint32_t i = __ffs(live_bits) - 1u;
                                live_bits &= live_bits - 1u;
                                const uint32_t slot = base + i;
                                const uint32_t m = red2(bqf + sQ0[f * r0 + slot] + ((slot >= split) ? corr[f] : 0u), qf[f]);
                                const uint32_t wv = __ldg(tab[f] + (m >> 5));
                                nb |= ((wv >> (m & 31u)) & 1u) << i;
                            }
                            bits = nb;
                            if (COUNT) cnt[f] += __popc(bits);
                            if (f + 1 < F && (uint32_t)(f + 1) < Feff) alive = __ballot_sync(0xffffffffu, bits != 0u) != 0u;
                        }
                    }
                }
                // ---- queue the survivors of the inner-ring stage -----------------------------
                if (PD) {
                    // one-word ring: an even digit's word waits for the next digit's, and the two
                    // go out as one entry (half the queue pushes)
                    if ((d1 & 1u) == 0u && d1 + 1u < r1) {
                        pbits = bits;
                        psplit = split;
                        pwrap = wm1 & 32u;
                        continue;
                    }
                    const bool odd = (d1 & 1u) != 0u;
                    const uint32_t plo = odd ? pbits : bits, phi = odd ? bits : 0u;
                    const uint32_t has = __ballot_sync(0xffffffffu, (plo | phi) != 0u);
                    if (has) {
                        const uint32_t ez = odd ? ((d1 - 1u) | (psplit << 16) | (split << 24)) : ent_z(d1, split);
                        const uint32_t ew = lane | (odd ? (pwrap | ((wm1 & 32u) << 1)) : (wm1 & 32u));
                        push<COUNT, PD>(Q, smem, si, lane, step, qhead, qsize, has, plo, phi, ez, ew);
                    }
                    continue;
                }
                if ((wd & 1u) == 0u && wd + 1u < Wn) {
                    lo = bits;
                    continue;
                }
                const bool odd = (wd & 1u) != 0u;
                const uint32_t plo = odd ? lo : bits, phi = odd ? bits : 0u;
                const uint32_t has = __ballot_sync(0xffffffffu, (plo | phi) != 0u);
                if (has) push<COUNT, PD>(Q, smem, si, lane, step, qhead, qsize, has, plo, phi, ent_z(d1, split),
                                         ent_w(lane, wm1, wd & ~1u));
            }
        }
        // the records change with the next strip step: drain the queue
        while (qsize) flush<COUNT, PD>(Q, smem, si, lane, step, qhead, qsize);
    }
    // ---- per-stage counts of this warp-unit into the item's totals ----------------------
    if (COUNT) {
        unsigned long long* gc = item.counts;
#pragma unroll
        for (int f = 0; f < F; ++f) {
            const uint32_t v = __reduce_add_sync(0xffffffffu, cnt[f]);
            if (lane == 0 && v && gc && (uint32_t)f < Feff) atomicAdd(gc + f, (unsigned long long)v);
        }
        __syncwarp();
        for (uint32_t f = Feff + lane; f < nf; f += 32u) {
            const uint32_t v = wcnt[f];
            if (v) {
                if (gc) atomicAdd(gc + f, (unsigned long long)v);
                wcnt[f] = 0u;
            }
        }
        __syncwarp();
    }
}

// Work distribution.  A warp-unit is 32 lanes x up to `strip` ring-1 cycles (or list entries)
// of one item (lanes on consecutive ring-2 rows, see scan_unit).  Single-plan launches: the CTA stages the plan's tables once, then each
// warp claims warp-units from the global counter on its own -- no CTA barrier after staging.
// Several plans: a CTA works on one item at a time, its warps claim the item's warp-units from
// the item's own counter, and the CTA synchronises only when it moves to another item (and
// restages when that item's plan differs).
//
// Template: F = filters evaluated in the inner-ring stage (upper bound, runtime Feff <= F),
// LAYOUT = word-mask or scalar tables, COUNT = per-stage pass counts, WT = words per inner ring
// when known at compile time (1: r0 <= 32, 2: r0 <= 64, 4: r0 <= 128, rows of four words),
// 0 = runtime.
template <int F, int LAYOUT, bool COUNT, int WT>
__global__ void __launch_bounds__(ES_LB_THREADS, ES_LB_MINB) es_scan_kernel(const __grid_constant__ EsLaunch L) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ EsInst si;
    __shared__ uint32_t s_item;

    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31u;
    const uint32_t warp = tid >> 5;
    EsQueue* Q = reinterpret_cast<EsQueue*>(smem + L.queue_off + warp * ES_QUEUE_BYTES);
    uint32_t* wcnt = reinterpret_cast<uint32_t*>(smem + L.cnt_off) + warp * L.nf_max;
    const uint32_t wcnt_saddr = (uint32_t)__cvta_generic_to_shared(wcnt);
    const EsItem* items = L.items ? L.items : &L.item0;
    const unsigned long long total = L.total_units;

    if (COUNT)
        for (uint32_t f = lane; f < L.nf_max; f += 32u) wcnt[f] = 0u;

    if (L.direct) {
        // ---- stage the one plan, then warps claim warp-units on their own ---------------
        if (tid == 0) si = *items[0].inst;
        __syncthreads();
        copy_words(reinterpret_cast<uint32_t*>(smem), reinterpret_cast<const uint32_t*>(si.small), si.small_bytes >> 2);
        if (LAYOUT == ES_LAYOUT_SMEM)   // the inner-stage filters' phase tables (16-byte aligned)
            copy_words(reinterpret_cast<uint32_t*>(smem + L.stage_off), si.masks, si.mask_off[F]);
        if (LAYOUT == ES_LAYOUT_SMEM_PAIR)
            copy_words(reinterpret_cast<uint32_t*>(smem + L.stage_off), si.pairs, 2u * si.mask_off[F]);
        __syncthreads();
        for (;;) {
            unsigned long long w = 0;
            uint32_t it_id = 0;
            int skip = 0;
            if (lane == 0) {
                w = atomicAdd(L.unit_counter, 1ull);
                if (w < total) {
                    uint32_t lo = 0, hi = L.n_items;
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (items[mid].unit_begin <= w) lo = mid; else hi = mid;
                    }
                    it_id = lo;
                    if (L.group_found) {
                        const unsigned long long fnd =
                            *reinterpret_cast<volatile unsigned long long*>(L.group_found + items[lo].group);
                        if (items[lo].t > fnd) skip = 1;
                    }
                }
            }
            w = __shfl_sync(0xffffffffu, w, 0);
            if (w >= total) break;
            it_id = __shfl_sync(0xffffffffu, it_id, 0);
            skip = __shfl_sync(0xffffffffu, skip, 0);
            if (skip) continue;
            scan_unit<F, LAYOUT, COUNT, WT>(L, si, smem, Q, wcnt, wcnt_saddr, lane, w, items[it_id], it_id);
        }
        return;
    }

    // ---- several plans: a CTA works on one item at a time and its warps claim that item's
    // warp-units from the item's own counter (no CTA barrier per unit); the CTA synchronises
    // only to move to another item, restaging the plan when it changes.  CTAs start spread over
    // the unit space in proportion to the items' work.
    uint32_t cur_inst = 0xffffffffu;
    if (tid == 0) {
        const unsigned long long u0 = (unsigned long long)blockIdx.x * total / gridDim.x;
        uint32_t lo = 0, hi = L.n_items;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (items[mid].unit_begin <= u0) lo = mid; else hi = mid;
        }
        s_item = lo;
    }
    __syncthreads();
    for (;;) {
        const uint32_t item_id = s_item;
        if (item_id >= L.n_items) break;
        const EsItem& item = items[item_id];
        if (item.inst_id != cur_inst) {
            // restage: the header and the small tables of this item's plan
            if (tid == 0) si = *item.inst;
            __syncthreads();
            copy_words(reinterpret_cast<uint32_t*>(smem), reinterpret_cast<const uint32_t*>(si.small),
                       si.small_bytes >> 2);
            if (LAYOUT == ES_LAYOUT_SMEM)
                copy_words(reinterpret_cast<uint32_t*>(smem + L.stage_off), si.masks, si.mask_off[F]);
            if (LAYOUT == ES_LAYOUT_SMEM_PAIR)
                copy_words(reinterpret_cast<uint32_t*>(smem + L.stage_off), si.pairs, 2u * si.mask_off[F]);
            __syncthreads();
            cur_inst = item.inst_id;
        }
        for (;;) {
            unsigned long long w = 0;
            int stop = 0;
            if (lane == 0) {
                const unsigned long long c = atomicAdd(L.item_next + item_id, 1ull);
                if (c >= item.n_units) {
                    stop = 1;
                } else if (L.group_found) {
                    const unsigned long long fnd =
                        *reinterpret_cast<volatile unsigned long long*>(L.group_found + item.group);
                    if (item.t > fnd) stop = 1;
                }
                w = item.unit_begin + c;
            }
            stop = __shfl_sync(0xffffffffu, stop, 0);
            w = __shfl_sync(0xffffffffu, w, 0);
            if (stop) break;
            scan_unit<F, LAYOUT, COUNT, WT>(L, si, smem, Q, wcnt, wcnt_saddr, lane, w, item, item_id);
        }
        __syncthreads();   // every warp is done with this item before its tables may be replaced
        if (tid == 0) {
            // the next item with unclaimed warp-units, after this one cyclically; each pass of
            // the loop above claims at least one unit, so the counters only grow and this ends
            uint32_t nxt = L.n_items;
            for (uint32_t j = 1; j <= L.n_items; ++j) {
                const uint32_t i = (item_id + j) % L.n_items;
                const EsItem& it = items[i];
                const unsigned long long c = *reinterpret_cast<volatile unsigned long long*>(L.item_next + i);
                if (c >= it.n_units) continue;
                if (L.group_found) {
                    const unsigned long long fnd =
                        *reinterpret_cast<volatile unsigned long long*>(L.group_found + it.group);
                    if (it.t > fnd) continue;
                }
                nxt = i;
                break;
            }
            s_item = nxt;
        }
        __syncthreads();
    }
}

}  // namespace

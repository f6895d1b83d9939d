// Device kernels of the GB300 Erdős–Selfridge CRT-wheel sieve (sm_103a).
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
//  * One persistent kernel per launch; CTAs claim work units (threads x strip ring-1 cycles
//    of one item) from a global atomic counter -- no spin waits anywhere.  Items are ordered
//    by (group, block), and a group's later blocks are skipped once a good survivor is known.
//  * Two-level strip mining.  A thread owns `strip` consecutive ring-1 cycles (cycle index =
//    oidx / r1).  Rings >= 2 give b2 = sum term_j mod M, decoded once per strip and then
//    stepped with a 128-bit delta table when the ring-2 digit advances.  Ring 1 is swept in a
//    warp-uniform loop (b = b2 + T1[d1], broadcast loads), and ring 0 (the inner ring) is
//    handled 32 candidates at a time as bit masks.
//  * Filter residues are carried incrementally in 32-bit arithmetic: BQ_f = n mod q_f for the
//    ring-0 base, updated with precomputed term residues and the wrap correction
//    corr_f = -M mod q_f (the reference's v7 identity, sieve/gpu_sieve_v9.py:9-18).
//  * Inner ring: the terms are sorted once on the host, so the wrap (s >= M) is a suffix of
//    the sorted slots; its start (the carry split) is found from 32-bit keys via a 1024-bucket
//    table.  Word-mask layout: a filter is one or two table loads per 32 candidates,
//    P_f[phase][w]; scalar layout: one residue + bit test per live candidate.  A warp leaves
//    the cascade early as soon as a ballot shows no live candidate.
//  * Filters after the inner-ring stage are evaluated per surviving candidate from the exact
//    128-bit residue with limb weights and a Barrett reduction.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/es_gb300.h"
#include "es_internal.h"

typedef unsigned __int128 u128;

namespace {

__device__ __forceinline__ u128 mk128(uint64_t lo, uint64_t hi) {
    return ((u128)hi << 64) | (u128)lo;
}

// (a + b) mod M for a, b < M < 2^126; wrap = 1 when M was subtracted.
__device__ __forceinline__ u128 addmod(u128 a, u128 b, u128 M, uint32_t& wrap) {
    u128 s = a + b;
    wrap = (s >= M) ? 1u : 0u;
    return wrap ? s - M : s;
}

// x mod q for a 128-bit x, q < 2^20: limb weights then one Barrett step.
__device__ __forceinline__ uint32_t mod128(u128 x, const EsFilterC& f) {
    const uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
    const uint64_t y = (lo & 0xffffffffull) + (lo >> 32) * f.w1 + (hi & 0xffffffffull) * f.w2 +
                       (hi >> 32) * f.w3;
    const uint64_t qt = __umul64hi(y, f.rcp);
    uint64_t r = y - qt * f.q;
    if (r >= f.q) r -= f.q;
    return (uint32_t)r;
}

__device__ __forceinline__ uint32_t red2(uint32_t v, uint32_t q) {
    v = (v >= q) ? v - q : v;
    return (v >= q) ? v - q : v;
}

// b2 = sum_{j>=2} term_j[d_j] mod M for ring-1 cycle c; also returns the ring-2 digit.
__device__ __noinline__ u128 decode_cycle(const EsInst& I, uint64_t c, u128 M, uint32_t& d2) {
    uint64_t rem = c;
    u128 acc = 0;
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
        const uint64_t* tp = I.ring_terms + 2ull * ((uint64_t)__ldg(I.ring_off + j) + d);
        uint32_t w;
        acc = addmod(acc, mk128(__ldg(tp), __ldg(tp + 1)), M, w);
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

struct EsSmemView {
    const ulonglong2* T1;
    const uint32_t* TQ1;
    const ulonglong2* D2;
    const uint32_t* DQ2;
    const ulonglong2* S0;
    const uint32_t* K0;
    const uint32_t* I0;
    const uint32_t* Q0;
    const uint16_t* BK;
    const EsFilterC* FC;
    const uint32_t* tc;
    const uint32_t* fast;
};

template <bool COUNT>
__device__ __forceinline__ void emit(const EsLaunch& L, const EsItem& item, const EsInst& I,
                                     uint32_t item_id, uint64_t idx, u128 s, u128 M) {
    const u128 kp1 = (u128)(I.k + 1u);
    bool good;
    if (M > kp1) {
        good = (item.t > 0) || (s > kp1);
    } else {
        good = ((u128)item.t * M + s) > kp1;
    }
    const unsigned long long slot = atomicAdd(L.surv_n, 1ull);
    if (slot < L.surv_cap) {
        es_survivor* r = L.surv + slot;
        r->idx = idx;
        r->s_lo = (uint64_t)s;
        r->s_hi = (uint64_t)(s >> 64);
        r->t = item.t;
        r->item = item_id;
        r->good = good ? 1u : 0u;
    }
    if (good && L.group_found) atomicMin(L.group_found + item.group, (unsigned long long)item.t);
}

// Exact cascade tail for one candidate: filters [f0, nf) from the 128-bit residue s.
template <bool COUNT>
__device__ __forceinline__ bool tail_filters(const EsSmemView& V, const EsInst& I, uint32_t f0,
                                             u128 s, uint32_t* sm_cnt) {
    for (uint32_t f = f0; f < I.n_filters; ++f) {
        const EsFilterC fc = V.FC[f];
        uint32_t r = mod128(s, fc) + V.tc[f];
        if (r >= fc.q) r -= fc.q;
        const uint32_t w = __ldg(I.allowed + fc.off + (r >> 5));
        if (!((w >> (r & 31u)) & 1u)) return false;
        if (COUNT) atomicAdd(sm_cnt + f, 1u);
    }
    return true;
}

template <int F, int LAYOUT, bool COUNT>
__global__ void __launch_bounds__(512) es_scan_kernel(const __grid_constant__ EsLaunch L) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ EsInst si;
    __shared__ unsigned long long s_unit;
    __shared__ uint32_t s_item;
    __shared__ int s_skip;

    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31u;
    uint32_t* sm_cnt = reinterpret_cast<uint32_t*>(smem + L.cnt_off);
    uint32_t* sm_tc = reinterpret_cast<uint32_t*>(smem + L.tconst_off);
    uint32_t* sm_fast = reinterpret_cast<uint32_t*>(smem + L.fast_off);
    uint32_t cur_inst = 0xffffffffu, cur_item = 0xffffffffu;
    const EsItem* items = L.items ? L.items : &L.item0;

    for (;;) {
        if (tid == 0) {
            const unsigned long long u = atomicAdd(L.unit_counter, 1ull);
            uint32_t it = 0;
            int skip = 0;
            if (u < L.total_units) {
                uint32_t lo = 0, hi = L.n_items;
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (items[mid].unit_begin <= u) lo = mid; else hi = mid;
                }
                it = lo;
                if (L.group_found) {
                    const unsigned long long fnd =
                        *reinterpret_cast<volatile unsigned long long*>(L.group_found + items[lo].group);
                    if (items[lo].t > fnd) skip = 1;
                }
            }
            s_unit = u;
            s_item = it;
            s_skip = skip;
        }
        __syncthreads();
        const unsigned long long u = s_unit;
        if (u >= L.total_units) break;
        const uint32_t item_id = s_item;
        if (s_skip) {
            __syncthreads();
            continue;
        }
        const EsItem& item = items[item_id];
        const uint32_t* tc_src = L.items ? item.tconst : L.tconst0;
        // ---- stage the instance tables (on change) and the block constants -------------
        if (item.inst_id != cur_inst) {
            if (tid == 0) si = *item.inst;
            __syncthreads();
            copy_words(reinterpret_cast<uint32_t*>(smem), reinterpret_cast<const uint32_t*>(si.small),
                       si.small_bytes >> 2);
            if (item.sm_fast_words)
                copy_words(sm_fast, LAYOUT == ES_LAYOUT_WORDMASK ? si.masks : si.allowed,
                           item.sm_fast_words);
        }
        if (item.inst_id != cur_inst || item_id != cur_item) {
            for (uint32_t f = tid; f < si.n_filters; f += blockDim.x) sm_tc[f] = tc_src[f];
        }
        if (COUNT)
            for (uint32_t f = tid; f < si.n_filters; f += blockDim.x) sm_cnt[f] = 0u;
        cur_inst = item.inst_id;
        cur_item = item_id;
        __syncthreads();

        const EsInst& I = si;
        EsSmemView V;
        V.T1 = reinterpret_cast<const ulonglong2*>(smem + I.o_T1);
        V.TQ1 = reinterpret_cast<const uint32_t*>(smem + I.o_TQ1);
        V.D2 = reinterpret_cast<const ulonglong2*>(smem + I.o_D2);
        V.DQ2 = reinterpret_cast<const uint32_t*>(smem + I.o_DQ2);
        V.S0 = reinterpret_cast<const ulonglong2*>(smem + I.o_S0);
        V.K0 = reinterpret_cast<const uint32_t*>(smem + I.o_K0);
        V.I0 = reinterpret_cast<const uint32_t*>(smem + I.o_I0);
        V.Q0 = reinterpret_cast<const uint32_t*>(smem + I.o_Q0);
        V.BK = reinterpret_cast<const uint16_t*>(smem + I.o_BK);
        V.FC = reinterpret_cast<const EsFilterC*>(smem + I.o_FC);
        V.tc = sm_tc;
        V.fast = sm_fast;

        const u128 M = mk128(I.M_lo, I.M_hi);
        const uint32_t r0 = I.r0, r1 = I.r1, r2 = I.r2, W = I.W;
        uint32_t Feff = (uint32_t)F < L.mask_filters ? (uint32_t)F : L.mask_filters;
        if (Feff > I.n_filters) Feff = I.n_filters;
        if (LAYOUT == ES_LAYOUT_WORDMASK && Feff > I.F_built) Feff = I.F_built;
        const uint32_t n_sm = item.n_sm;
        uint32_t qf[F], corr[F];
#pragma unroll
        for (int f = 0; f < F; ++f) {
            const bool on = (uint32_t)f < Feff;
            qf[f] = on ? V.FC[f].q : 1u;
            corr[f] = on ? V.FC[f].corr : 0u;
        }
        uint32_t cnt[F];
#pragma unroll
        for (int f = 0; f < F; ++f) cnt[f] = 0u;

        // ---- this thread's strip of ring-1 cycles (or list entries) ---------------------
        const uint64_t rel = (u - item.unit_begin) * L.cycles_per_unit + (uint64_t)tid * L.strip;
        const bool listed = item.list != nullptr;
        uint64_t e_lo, e_hi;
        if (listed) {
            e_lo = item.o_begin + rel;
            e_hi = e_lo + L.strip;
            if (e_hi > item.o_end) e_hi = item.o_end;
        } else {
            e_lo = item.c_begin + rel;
            e_hi = e_lo + L.strip;
            if (e_hi > item.c_end) e_hi = item.c_end;
        }
        u128 b2 = 0;
        uint32_t d2 = 0;
        uint32_t BQ2[F];
#pragma unroll
        for (int f = 0; f < F; ++f) BQ2[f] = 0u;
        bool have = false;
        uint64_t prev_c = 0;

        // Every lane runs L.strip iterations so the warp-wide ballots below see all 32 lanes;
        // lanes past the end of their strip take part with an empty candidate set.
        for (uint32_t step = 0; step < L.strip; ++step) {
            const uint64_t e = e_lo + step;
            const bool live = e < e_hi;
            if (__ballot_sync(0xffffffffu, live) == 0u) break;
            uint64_t c = prev_c;
            uint32_t lo1 = 0u, hi1 = 0u;
            if (!live) {
                // keep the decoded state; no positions
            } else if (listed) {
                const uint64_t o = __ldg(reinterpret_cast<const unsigned long long*>(item.list) + e);
                c = o / r1;
                lo1 = (uint32_t)(o - c * r1);
                hi1 = lo1 + 1u;
            } else {
                c = e;
                const uint64_t o0 = c * r1;
                lo1 = item.o_begin > o0 ? (uint32_t)(item.o_begin - o0) : 0u;
                const uint64_t span = item.o_end - o0;
                hi1 = span < r1 ? (uint32_t)span : r1;
            }
            // ---- rings >= 2: decode at strip start / ring-3 carry, else one delta step ----
            if (!live) {
            } else if (have && c == prev_c + 1 && d2 + 1u < r2) {
                uint32_t w;
                b2 = addmod(b2, mk128(V.D2[d2].x, V.D2[d2].y), M, w);
#pragma unroll
                for (int f = 0; f < F; ++f)
                    BQ2[f] = red2(BQ2[f] + V.DQ2[d2 * ES_FMAX + f] + (w ? corr[f] : 0u), qf[f]);
                ++d2;
            } else if (!(have && c == prev_c)) {
                b2 = decode_cycle(I, c, M, d2);
#pragma unroll
                for (int f = 0; f < F; ++f) {
                    if ((uint32_t)f < Feff) {
                        uint32_t v = mod128(b2, V.FC[f]) + V.tc[f];
                        BQ2[f] = v >= qf[f] ? v - qf[f] : v;
                    }
                }
                have = true;
            }
            prev_c = c;

            // ---- ring 1: warp-uniform sweep --------------------------------------------
            for (uint32_t d1 = 0; d1 < r1; ++d1) {
                const bool act = (d1 >= lo1) && (d1 < hi1);
                const ulonglong2 tv = V.T1[d1];
                uint32_t w1;
                const u128 b = addmod(b2, mk128(tv.x, tv.y), M, w1);
                uint32_t BQ[F];
#pragma unroll
                for (int f = 0; f < F; ++f)
                    BQ[f] = red2(BQ2[f] + V.TQ1[d1 * ES_FMAX + f] + (w1 ? corr[f] : 0u), qf[f]);
                // carry split: slots [split, r0) wrap past M
                const u128 thr = M - b;
                const uint32_t t32 = (uint32_t)(thr >> I.sh);
                uint32_t split = V.BK[t32 >> I.bsh];
                while (split < r0 && V.K0[split] < t32) ++split;
                while (split < r0 && V.K0[split] == t32 &&
                       mk128(V.S0[split].x, V.S0[split].y) < thr)
                    ++split;
                const uint64_t oidx = c * r1 + d1;

                for (uint32_t wd = 0; wd < W; ++wd) {
                    const uint32_t valid = (wd + 1u == W) ? I.tail_mask : 0xffffffffu;
                    uint32_t bits = act ? valid : 0u;
                    const uint32_t base = wd << 5;
                    const uint32_t cm = split <= base ? valid
                                      : (split >= base + 32u ? 0u : ((0xffffffffu << (split - base)) & valid));
#pragma unroll
                    for (int f = 0; f < F; ++f) {
                        if ((uint32_t)f < Feff) {
                            if (LAYOUT == ES_LAYOUT_WORDMASK) {
                                const uint32_t ph0 = BQ[f];
                                uint32_t ph1 = ph0 + corr[f];
                                ph1 = ph1 >= qf[f] ? ph1 - qf[f] : ph1;
                                uint32_t m0, m1;
                                if ((uint32_t)f < n_sm) {
                                    const uint32_t* tab = V.fast + I.mask_off[f];
                                    m0 = tab[ph0 * W + wd];
                                    m1 = tab[ph1 * W + wd];
                                } else {
                                    const uint32_t* tab = I.masks + I.mask_off[f];
                                    m0 = __ldg(tab + ph0 * W + wd);
                                    m1 = __ldg(tab + ph1 * W + wd);
                                }
                                bits &= (m0 & ~cm) | (m1 & cm);
                            } else {
                                const uint32_t* tab = ((uint32_t)f < n_sm) ? (V.fast + V.FC[f].off)
                                                                           : (I.allowed + V.FC[f].off);
                                uint32_t nb = 0u, live = bits;
                                while (live) {
                                    const uint32_t i = __ffs(live) - 1u;
                                    live &= live - 1u;
                                    const uint32_t slot = base + i;
                                    const uint32_t m = red2(BQ[f] + V.Q0[f * r0 + slot] +
                                                                ((slot >= split) ? corr[f] : 0u),
                                                            qf[f]);
                                    const uint32_t wv = ((uint32_t)f < n_sm) ? tab[m >> 5] : __ldg(tab + (m >> 5));
                                    nb |= ((wv >> (m & 31u)) & 1u) << i;
                                }
                                bits = nb;
                            }
                            if (COUNT) cnt[f] += __popc(bits);
                        }
                        if (__ballot_sync(0xffffffffu, bits != 0u) == 0u) break;
                    }
                    // ---- survivors of the inner-ring stage: exact tail of the cascade ----
                    while (bits) {
                        const uint32_t i = __ffs(bits) - 1u;
                        bits &= bits - 1u;
                        const uint32_t slot = base + i;
                        u128 s = b + mk128(V.S0[slot].x, V.S0[slot].y);
                        if (slot >= split) s -= M;
                        if (tail_filters<COUNT>(V, I, Feff, s, sm_cnt)) {
                            emit<COUNT>(L, item, I, item_id, oidx * (uint64_t)r0 + V.I0[slot], s, M);
                        }
                    }
                }
            }
        }
        // ---- flush per-stage counts ------------------------------------------------------
        if (COUNT) {
#pragma unroll
            for (int f = 0; f < F; ++f) {
                const uint32_t v = __reduce_add_sync(0xffffffffu, cnt[f]);
                if (lane == 0 && v) atomicAdd(sm_cnt + f, v);
            }
            __syncthreads();
            if (item.counts)
                for (uint32_t f = tid; f < I.n_filters; f += blockDim.x)
                    if (sm_cnt[f]) atomicAdd(item.counts + f, (unsigned long long)sm_cnt[f]);
        }
        __syncthreads();
    }
}

// Block-ordered minimum per search group: least (t, s) over good survivors.
// out[g*4 + 0] = found, [1] = t, [2] = s_lo, [3] = s_hi.
__global__ void es_min_kernel(const es_survivor* __restrict__ surv,
                              const unsigned long long* __restrict__ surv_n, uint64_t cap,
                              const EsItem* __restrict__ items, unsigned long long* out) {
    const uint32_t g = blockIdx.x;
    uint64_t n = *surv_n;
    if (n > cap) n = cap;
    uint64_t bt = ~0ull, bhi = ~0ull, blo = ~0ull;
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const es_survivor r = surv[i];
        const uint32_t grp = items ? items[r.item].group : 0u;
        if (!r.good || grp != g) continue;
        const bool less = (r.t < bt) || (r.t == bt && (r.s_hi < bhi || (r.s_hi == bhi && r.s_lo < blo)));
        if (less) {
            bt = r.t;
            bhi = r.s_hi;
            blo = r.s_lo;
        }
    }
    __shared__ unsigned long long st[256], sh[256], sl[256];
    st[threadIdx.x] = bt;
    sh[threadIdx.x] = bhi;
    sl[threadIdx.x] = blo;
    __syncthreads();
    for (uint32_t w = blockDim.x >> 1; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const uint32_t o = threadIdx.x + w;
            const bool less = (st[o] < st[threadIdx.x]) ||
                              (st[o] == st[threadIdx.x] &&
                               (sh[o] < sh[threadIdx.x] || (sh[o] == sh[threadIdx.x] && sl[o] < sl[threadIdx.x])));
            if (less) {
                st[threadIdx.x] = st[o];
                sh[threadIdx.x] = sh[o];
                sl[threadIdx.x] = sl[o];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const bool found = !(st[0] == ~0ull && sh[0] == ~0ull && sl[0] == ~0ull);
        out[4 * g + 0] = found ? 1ull : 0ull;
        out[4 * g + 1] = st[0];
        out[4 * g + 2] = sl[0];
        out[4 * g + 3] = sh[0];
    }
}

// Integer-pipe throughput probe: 8 independent chains per thread of IADD3 / LOP3 pairs.
__global__ void __launch_bounds__(256) es_int_peak_kernel(unsigned long long* sink, int iters,
                                                         uint32_t seed) {
    uint32_t a0 = seed ^ threadIdx.x, a1 = a0 * 3u + 1u, a2 = a0 * 5u + 7u, a3 = a0 * 7u + 3u;
    uint32_t a4 = a0 + 11u, a5 = a1 ^ 0x55u, a6 = a2 + 0x99u, a7 = a3 ^ 0x1234u;
    const uint32_t c1 = seed * 13u + 5u, c2 = seed * 29u + 17u;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            // one IADD3 and one LOP3 per chain per step (ops counted = 16 per step per thread)
            a0 = a0 + a1 + c1;
            a1 = a1 + a2 + c2;
            a2 = a2 + a3 + c1;
            a3 = a3 + a4 + c2;
            a4 = a4 + a5 + c1;
            a5 = a5 + a6 + c2;
            a6 = a6 + a7 + c1;
            a7 = a7 + a0 + c2;
            asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a0) : "r"(a1), "r"(c1));
            asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a1) : "r"(a2), "r"(c2));
            asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a2) : "r"(a3), "r"(c1));
            asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a3) : "r"(a4), "r"(c2));
            asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a4) : "r"(a5), "r"(c1));
            asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a5) : "r"(a6), "r"(c2));
            asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a6) : "r"(a7), "r"(c1));
            asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a7) : "r"(a0), "r"(c2));
        }
    }
    const uint32_t x = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
    if (x == 0x9e3779b9u) atomicAdd(sink, 1ull);  // keeps the chains live
}

typedef void (*ScanFn)(const EsLaunch);

template <int LAYOUT, bool COUNT>
ScanFn pick_f(uint32_t f) {
    if (f <= 2) return es_scan_kernel<2, LAYOUT, COUNT>;
    if (f <= 4) return es_scan_kernel<4, LAYOUT, COUNT>;
    if (f <= 6) return es_scan_kernel<6, LAYOUT, COUNT>;
    return es_scan_kernel<8, LAYOUT, COUNT>;
}

ScanFn pick(int layout, int count, uint32_t f) {
    if (layout == ES_LAYOUT_WORDMASK)
        return count ? pick_f<ES_LAYOUT_WORDMASK, true>(f) : pick_f<ES_LAYOUT_WORDMASK, false>(f);
    return count ? pick_f<ES_LAYOUT_SCALAR, true>(f) : pick_f<ES_LAYOUT_SCALAR, false>(f);
}

}  // namespace

// Raise the dynamic shared-memory limit of every scan instance once per process/device.
int es_scan_prepare(int smem_optin_bytes) {
    const uint32_t fs[4] = {2, 4, 6, 8};
    for (int layout = 0; layout < 2; ++layout)
        for (int count = 0; count < 2; ++count)
            for (uint32_t f : fs) {
                cudaError_t e = cudaFuncSetAttribute(pick(layout, count, f),
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     smem_optin_bytes);
                if (e != cudaSuccess) return (int)e;
            }
    return 0;
}

int es_scan_occupancy(int layout, int count, uint32_t mask_filters, int threads, int smem_bytes,
                      int* ctas_per_sm) {
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        ctas_per_sm, pick(layout, count, mask_filters), threads, (size_t)smem_bytes);
}

int es_launch_scan(const EsLaunch& L, int layout, int count, int grid, void* stream) {
    pick(layout, count, L.mask_filters)<<<grid, L.threads, L.smem_bytes, (cudaStream_t)stream>>>(L);
    return (int)cudaGetLastError();
}

int es_launch_min(const es_survivor* surv, const unsigned long long* surv_n, uint64_t cap,
                  const EsItem* items, uint32_t n_groups, unsigned long long* group_min,
                  void* stream) {
    if (n_groups == 0) return 0;
    es_min_kernel<<<n_groups, 256, 0, (cudaStream_t)stream>>>(surv, surv_n, cap, items, group_min);
    return (int)cudaGetLastError();
}

int es_launch_int_peak(unsigned long long* sink, int grid, int threads, int iters, void* stream) {
    es_int_peak_kernel<<<grid, threads, 0, (cudaStream_t)stream>>>(sink, iters, 0x2545f491u);
    return (int)cudaGetLastError();
}

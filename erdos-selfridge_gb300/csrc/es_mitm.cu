// Meet-in-the-middle search kernel of the GB300 Erdős–Selfridge engine (sm_103a) and its C ABI
// (es_mitm_* in include/es_gb300.h).
//
// What one scan computes (the semantics of sieve/gpu_mitm.py:33-125): the wheel residues are
// n = (s1 + s2) mod M with s1 a sum of one term per prime of the large half W1 and s2 one per
// prime of the small half W2 (terms a * c_p mod M, c_p the CRT basis).  For a bound B <= M and
// every s1 index in [s1_begin, s1_end), the n < B are exactly s1 + S2[u] for the u of one
// circular run of the sorted S2: [lower_bound(M - s1), lower_bound(M - s1 + B)) mod M, the run
// wrapping to the front of S2 when M - s1 + B >= M.  Each such n runs through the residual-prime
// cascade (n mod q for every filter in order, early exit) and the survivors are emitted; the
// number of n tested is counted.
//
// GB300-first organisation (not the reference's one-thread-per-s1 kernel with two full binary
// searches): S2 is sorted once on the host and uploaded with a directory over the top bits of
// its values (bucket b -> first index whose value >= b << shift), sized at about four entries
// per bucket, so each search is one directory load and a binary search over a handful of entries
// instead of log2|S2| dependent loads; warps claim chunks of s1 indices from an atomic counter
// (persistent grid, no waits); s1 is decoded from its index by mixed radix with precomputed
// 64-bit reciprocals; n mod q uses 32-bit limb weights and one Barrett step against packed bit
// tables, exactly the exact tail of the block-sieve kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/es_gb300.h"
#include "es_internal.h"
#include "es_scan_kernel.cuh"

typedef unsigned __int128 u128m;

namespace {

int mfail(int code, const std::string& msg) {
    es_set_last_error(msg.c_str());
    return code;
}

int mcuda(cudaError_t e, const char* what) {
    es_set_last_error((std::string(what) + ": " + cudaGetErrorString(e)).c_str());
    return ES_ERR_CUDA;
}

#define ES_MCUDA(call, what)                               \
    do {                                                   \
        cudaError_t _e = (call);                           \
        if (_e != cudaSuccess) return mcuda(_e, what);     \
    } while (0)

constexpr uint32_t kMitmMaxRings = 32;
constexpr uint32_t kMitmThreads = 256;
constexpr uint32_t kMitmChunk = 8;   // s1 indices per lane per claimed chunk

struct MitmParams {
    const uint4* S2;              // sorted small half: {lo.x, lo.y, hi.x, hi.y} per entry
    const uint32_t* dir;          // [2^D + 1] first S2 index with value >= b << shift
    const uint4* terms1;          // large half's terms, ring after ring
    const EsFilterC* filt;        // residual filters (q, limb weights, Barrett reciprocal, offset)
    const uint32_t* allowed;      // packed admissible-residue bits of every filter
    uint4* out;                   // survivors {n_lo, n_hi} as uint4
    unsigned long long* counters; // [0] survivors, [1] candidates tested, [2] work counter
    uint64_t out_cap;
    uint64_t n2;
    uint64_t s1_begin, s1_end;
    uint64_t M_lo, M_hi, B_lo, B_hi;
    uint32_t shift;               // directory bucket = value >> shift
    uint32_t n_rings1;
    uint32_t n_filters;
    uint32_t radix1[kMitmMaxRings];
    uint32_t off1[kMitmMaxRings];
    unsigned long long magic1[kMitmMaxRings];   // ceil(2^64 / radix) (0 for radix 1)
};

__device__ __forceinline__ U4 ld_s2(const uint4* S2, uint64_t i) { return u4(__ldg(S2 + i)); }

// 128-bit value >> shift (shift < 128), low 32 bits (the directory bucket of a value < M)
__device__ __forceinline__ uint32_t bucket_of(const U4 v, uint32_t shift) {
    const uint64_t lo = lo64(v), hi = hi64(v);
    uint64_t r;
    if (shift >= 64) r = hi >> (shift - 64);
    else if (shift == 0) r = lo;
    else r = (lo >> shift) | (hi << (64 - shift));
    return (uint32_t)r;
}

// first index u with S2[u] >= v (n2 when none): the directory narrows it to one bucket
__device__ __forceinline__ uint64_t lower_bound_s2(const MitmParams& P, const U4 v) {
    const uint32_t b = bucket_of(v, P.shift);
    uint64_t a = __ldg(P.dir + b), e = __ldg(P.dir + b + 1);
    while (a < e) {
        const uint64_t m = (a + e) >> 1;
        if (lt128(ld_s2(P.S2, m), v)) a = m + 1; else e = m;
    }
    return a;
}

// s1 of index idx: mixed radix over the large half's rings, ring 0 fastest
__device__ __forceinline__ U4 decode_s1(const MitmParams& P, uint64_t idx, const U4 M) {
    U4 acc{0u, 0u, 0u, 0u};
    uint64_t rem = idx;
    for (uint32_t j = 0; j < P.n_rings1; ++j) {
        const uint32_t r = P.radix1[j];
        uint64_t q;
        if (r <= 1) {
            q = rem;
        } else if ((rem >> 48) == 0) {
            q = __umul64hi(rem, P.magic1[j]);   // exact for rem < 2^48, r < 2^16
        } else {
            q = rem / r;
        }
        const uint64_t d = rem - q * r;
        rem = q;
        uint32_t wm;
        acc = addmod(acc, u4(__ldg(P.terms1 + P.off1[j] + d)), M, wm);
    }
    return acc;
}

__global__ void __launch_bounds__(kMitmThreads) es_mitm_kernel(const __grid_constant__ MitmParams P) {
    const uint32_t lane = threadIdx.x & 31u;
    const U4 M{(uint32_t)P.M_lo, (uint32_t)(P.M_lo >> 32), (uint32_t)P.M_hi, (uint32_t)(P.M_hi >> 32)};
    const U4 B{(uint32_t)P.B_lo, (uint32_t)(P.B_lo >> 32), (uint32_t)P.B_hi, (uint32_t)(P.B_hi >> 32)};
    const uint64_t total = P.s1_end - P.s1_begin;
    const uint64_t per_claim = 32ull * kMitmChunk;
    unsigned long long tested = 0;
    for (;;) {
        unsigned long long c = 0;
        if (lane == 0) c = atomicAdd(P.counters + 2, 1ull);
        c = __shfl_sync(0xffffffffu, c, 0);
        const uint64_t base = c * per_claim;
        if (base >= total) break;
        for (uint32_t it = 0; it < kMitmChunk; ++it) {
            const uint64_t rel = base + (uint64_t)it * 32u + lane;
            if (rel >= total) break;
            const U4 s1 = decode_s1(P, P.s1_begin + rel, M);
            // lo = (M - s1) mod M, hi = lo + B (mod M, wrapping past M when lo + B >= M)
            uint32_t br;
            U4 lo = sub128(M, s1, br);
            if ((s1.x | s1.y | s1.z | s1.w) == 0u) lo = U4{0u, 0u, 0u, 0u};
            const U4 hs = add128(lo, B);
            const U4 hm = sub128(hs, M, br);
            const bool wrap = br == 0u;            // lo + B >= M
            const U4 hi = wrap ? hm : hs;
            const uint64_t i0 = lower_bound_s2(P, lo);
            const uint64_t j0 = lower_bound_s2(P, hi);
            // the run: [i0, j0) without a wrap; [i0, n2) then [0, j0) with one
            uint64_t u = i0;
            const uint64_t end0 = wrap ? P.n2 : j0;
            uint64_t todo = (end0 > i0 ? end0 - i0 : 0) + (wrap ? j0 : 0);
            tested += todo;
            while (todo) {
                if (u >= end0 && wrap) u -= end0;   // continue at the front of S2
                const U4 s2 = ld_s2(P.S2, u);
                uint32_t wm;
                const U4 n = addmod(s1, s2, M, wm);
                bool ok = true;
                for (uint32_t f = 0; f < P.n_filters && ok; ++f) {
                    const EsFilterC fc = P.filt[f];
                    const uint32_t r = mod128(n, fc);
                    ok = (__ldg(P.allowed + fc.off + (r >> 5)) >> (r & 31u)) & 1u;
                }
                if (ok) {
                    const unsigned long long slot = atomicAdd(P.counters + 0, 1ull);
                    if (slot < P.out_cap) P.out[slot] = make_uint4(n.x, n.y, n.z, n.w);
                }
                ++u;
                --todo;
            }
        }
    }
    for (uint32_t o = 16; o > 0; o >>= 1) tested += __shfl_down_sync(0xffffffffu, tested, o);
    if (lane == 0 && tested) atomicAdd(P.counters + 1, tested);
}

}  // namespace

struct es_mitm {
    cudaStream_t stream = nullptr;
    MitmParams P{};
    uint4* d_S2 = nullptr;
    uint32_t* d_dir = nullptr;
    uint4* d_terms1 = nullptr;
    EsFilterC* d_filt = nullptr;
    uint32_t* d_allowed = nullptr;
    uint4* d_out = nullptr;
    unsigned long long* d_cnt = nullptr;
    unsigned long long* h_cnt = nullptr;
    uint64_t n1 = 0, n2 = 0, cap = 0;
    int grid = 0;
};

extern "C" {

int es_mitm_destroy(es_mitm* m) {
    if (!m) return ES_OK;
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->d_S2);
    cudaFree(m->d_dir);
    cudaFree(m->d_terms1);
    cudaFree(m->d_filt);
    cudaFree(m->d_allowed);
    cudaFree(m->d_out);
    cudaFree(m->d_cnt);
    if (m->h_cnt) cudaFreeHost(m->h_cnt);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return ES_OK;
}

namespace {

// Sorts v (values below 2^bits) on the host cores: each thread counts its share of the values
// per partition of their top P bits, the values are scattered to their partitions, and the
// partitions are sorted, shared out among the threads.  The result equals std::sort's.
void parallel_sort(std::vector<u128m>& v, uint32_t bits) {
    const size_t n = v.size();
    const unsigned T = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if (n < (1u << 16) || T == 1 || bits == 0) {
        std::sort(v.begin(), v.end());
        return;
    }
    const uint32_t P = std::min<uint32_t>(12, bits);
    const uint32_t sh = bits - P;
    const size_t np = (size_t)1 << P;
    auto run = [T](auto&& body) {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < T; ++t) th.emplace_back(body, t);
        for (auto& x : th) x.join();
    };
    std::vector<std::vector<size_t>> at(T, std::vector<size_t>(np, 0));
    run([&](unsigned t) {
        for (size_t i = n * t / T, e = n * (t + 1) / T; i < e; ++i) ++at[t][(size_t)(v[i] >> sh)];
    });
    std::vector<size_t> start(np + 1);
    size_t acc = 0;
    for (size_t p = 0; p < np; ++p) {   // partition-major, thread-minor write positions
        start[p] = acc;
        for (unsigned t = 0; t < T; ++t) {
            const size_t c = at[t][p];
            at[t][p] = acc;
            acc += c;
        }
    }
    start[np] = acc;
    std::vector<u128m> out(n);
    run([&](unsigned t) {
        for (size_t i = n * t / T, e = n * (t + 1) / T; i < e; ++i) out[at[t][(size_t)(v[i] >> sh)]++] = v[i];
    });
    std::atomic<size_t> next(0);
    run([&](unsigned) {
        for (size_t p = next++; p < np; p = next++) std::sort(out.begin() + start[p], out.begin() + start[p + 1]);
    });
    v.swap(out);
}

}  // namespace

int es_mitm_create(const es_mitm_desc* d, es_mitm** out) {
    if (!d || !out) return mfail(ES_ERR_ARG, "null descriptor or output pointer");
    *out = nullptr;
    const u128m M = ((u128m)d->M_hi << 64) | d->M_lo;
    if (M < 2 || (M >> 126) != 0) return mfail(ES_ERR_RANGE, "wheel modulus must be in [2, 2^126)");
    if (d->n_rings1 > kMitmMaxRings || d->n_rings2 > kMitmMaxRings)
        return mfail(ES_ERR_RANGE, "too many wheel primes in one half (max 32)");
    if (d->n_filters > ES_MAX_FILTERS) return mfail(ES_ERR_RANGE, "too many residual filters");
    if ((d->n_rings1 && (!d->radix1 || !d->term1_lo || !d->term1_hi)) ||
        (d->n_rings2 && (!d->radix2 || !d->term2_lo || !d->term2_hi)) ||
        (d->n_filters && (!d->filter_q || !d->allowed)))
        return mfail(ES_ERR_ARG, "null array in descriptor");
    int dev = 0, major = 0, minor = 0, sms = 0;
    ES_MCUDA(cudaGetDevice(&dev), "cudaGetDevice");
    ES_MCUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev), "attr");
    ES_MCUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev), "attr");
    ES_MCUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr");
    if (major != 10 || minor != 3) return mfail(ES_ERR_NODEV, "this library is built for sm_103a only");

    // ---- the two halves --------------------------------------------------------------------
    uint64_t n1 = 1, n2 = 1;
    std::vector<u128m> t1, t2;
    std::vector<uint32_t> r1(d->radix1, d->radix1 + d->n_rings1), r2(d->radix2, d->radix2 + d->n_rings2);
    for (uint32_t j = 0; j < d->n_rings1; ++j) {
        const uint32_t r = r1[j];
        if (r == 0 || r > 65535) return mfail(ES_ERR_RANGE, "radix must be in [1, 65535]");
        if (n1 > (1ull << 62) / r) return mfail(ES_ERR_RANGE, "|S1| exceeds 2^62");
        n1 *= r;
    }
    for (uint32_t j = 0; j < d->n_rings2; ++j) {
        const uint32_t r = r2[j];
        if (r == 0 || r > 65535) return mfail(ES_ERR_RANGE, "radix must be in [1, 65535]");
        if (n2 > (1ull << 31) / r) return mfail(ES_ERR_RANGE, "|S2| must stay below 2^31 entries");
        n2 *= r;
    }
    size_t pos = 0;
    for (uint32_t j = 0; j < d->n_rings1; ++j)
        for (uint32_t i = 0; i < r1[j]; ++i, ++pos) {
            const u128m v = ((u128m)d->term1_hi[pos] << 64) | d->term1_lo[pos];
            if (v >= M) return mfail(ES_ERR_ARG, "term not reduced mod M");
            t1.push_back(v);
        }
    pos = 0;
    for (uint32_t j = 0; j < d->n_rings2; ++j)
        for (uint32_t i = 0; i < r2[j]; ++i, ++pos) {
            const u128m v = ((u128m)d->term2_hi[pos] << 64) | d->term2_lo[pos];
            if (v >= M) return mfail(ES_ERR_ARG, "term not reduced mod M");
            t2.push_back(v);
        }
    // S2: every sum of one term per ring of the small half, mod M, sorted
    std::vector<u128m> S2(1, 0);
    pos = 0;
    for (uint32_t j = 0; j < d->n_rings2; ++j) {
        const size_t have = S2.size();
        std::vector<u128m> next;
        next.reserve(have * r2[j]);
        for (size_t a = 0; a < have; ++a)
            for (uint32_t i = 0; i < r2[j]; ++i) {
                u128m v = S2[a] + t2[pos + i];
                if (v >= M) v -= M;
                next.push_back(v);
            }
        S2.swap(next);
        pos += r2[j];
    }
    uint32_t bits = 0;   // values < M < 2^bits
    for (u128m x = M - 1; x; x >>= 1) ++bits;
    parallel_sort(S2, bits);
    // directory over the top bits of values < M: about four entries per bucket
    uint32_t D = 8;
    while (D < 26 && (1ull << (D + 2)) < n2) ++D;
    if (D > bits) D = bits;
    const uint32_t shift = bits - D;
    std::vector<uint32_t> dir((1ull << D) + 1);
    {
        size_t i = 0;
        for (uint64_t b = 0; b <= (1ull << D); ++b) {
            const u128m lim = (u128m)b << shift;
            while (i < S2.size() && S2[i] < lim) ++i;
            dir[b] = (uint32_t)i;
        }
    }
    // ---- filters ---------------------------------------------------------------------------
    std::vector<EsFilterC> fc(d->n_filters);
    uint32_t words = 0;
    for (uint32_t f = 0; f < d->n_filters; ++f) {
        const uint32_t q = d->filter_q[f];
        if (q < 2 || q >= ES_MAX_Q) return mfail(ES_ERR_RANGE, "filter modulus must be in [2, 2^20)");
        fc[f].q = q;
        fc[f].corr = 0;
        fc[f].w1 = (uint32_t)(((u128m)1 << 32) % q);
        fc[f].w2 = (uint32_t)(((u128m)1 << 64) % q);
        fc[f].w3 = (uint32_t)(((u128m)1 << 96) % q);
        fc[f].off = words;
        fc[f].rcp = (uint64_t)(((u128m)1 << 64) / q);
        words += (q + 31) / 32;
    }

    es_mitm* m = new (std::nothrow) es_mitm();
    if (!m) return mfail(ES_ERR_NOMEM, "host allocation");
    m->n1 = n1;
    m->n2 = n2;
    std::vector<uint4> h_S2(S2.size()), h_t1(std::max<size_t>(t1.size(), 1));
    auto pack = [](u128m v) {
        const uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
        return make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
    };
    for (size_t i = 0; i < S2.size(); ++i) h_S2[i] = pack(S2[i]);
    for (size_t i = 0; i < t1.size(); ++i) h_t1[i] = pack(t1[i]);
    cudaError_t ce = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaMalloc(&m->d_S2, sizeof(uint4) * h_S2.size());
    if (ce == cudaSuccess) ce = cudaMalloc(&m->d_dir, 4ull * dir.size());
    if (ce == cudaSuccess) ce = cudaMalloc(&m->d_terms1, sizeof(uint4) * h_t1.size());
    if (ce == cudaSuccess) ce = cudaMalloc(&m->d_filt, sizeof(EsFilterC) * std::max<size_t>(fc.size(), 1));
    if (ce == cudaSuccess) ce = cudaMalloc(&m->d_allowed, 4ull * std::max<uint32_t>(words, 1));
    if (ce == cudaSuccess) ce = cudaMalloc(&m->d_cnt, 8ull * 4);
    if (ce == cudaSuccess) ce = cudaHostAlloc(&m->h_cnt, 8ull * 4, cudaHostAllocDefault);
    if (ce == cudaSuccess) ce = cudaMemcpy(m->d_S2, h_S2.data(), sizeof(uint4) * h_S2.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(m->d_dir, dir.data(), 4ull * dir.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(m->d_terms1, h_t1.data(), sizeof(uint4) * h_t1.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess && !fc.empty())
        ce = cudaMemcpy(m->d_filt, fc.data(), sizeof(EsFilterC) * fc.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess && words) ce = cudaMemcpy(m->d_allowed, d->allowed, 4ull * words, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemset(m->d_cnt, 0, 8ull * 4);
    if (ce != cudaSuccess) {
        es_mitm_destroy(m);
        return mcuda(ce, "MITM setup");
    }
    MitmParams& P = m->P;
    P.S2 = m->d_S2;
    P.dir = m->d_dir;
    P.terms1 = m->d_terms1;
    P.filt = m->d_filt;
    P.allowed = m->d_allowed;
    P.counters = m->d_cnt;
    P.n2 = n2;
    P.M_lo = d->M_lo;
    P.M_hi = d->M_hi;
    P.shift = shift;
    P.n_rings1 = d->n_rings1;
    P.n_filters = d->n_filters;
    uint32_t o = 0;
    for (uint32_t j = 0; j < d->n_rings1; ++j) {
        P.radix1[j] = r1[j];
        P.off1[j] = o;
        P.magic1[j] = r1[j] > 1 ? (unsigned long long)((~0ull) / r1[j]) + 1ull : 0ull;
        o += r1[j];
    }
    int occ = 0;
    ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, es_mitm_kernel, kMitmThreads, 0);
    if (ce != cudaSuccess || occ < 1) {
        es_mitm_destroy(m);
        return mcuda(ce == cudaSuccess ? cudaErrorInvalidConfiguration : ce, "MITM occupancy");
    }
    m->grid = sms * occ;
    if (int e = es_mitm_set_capacity(m, 1u << 20)) {
        es_mitm_destroy(m);
        return e;
    }
    *out = m;
    return ES_OK;
}

int es_mitm_info(const es_mitm* m, uint64_t* n1, uint64_t* n2) {
    if (!m) return mfail(ES_ERR_ARG, "null MITM engine");
    if (n1) *n1 = m->n1;
    if (n2) *n2 = m->n2;
    return ES_OK;
}

int es_mitm_set_capacity(es_mitm* m, uint64_t cap) {
    if (!m || cap == 0 || cap > (1ull << 32)) return mfail(ES_ERR_ARG, "capacity must be in [1, 2^32]");
    ES_MCUDA(cudaStreamSynchronize(m->stream), "sync");
    cudaFree(m->d_out);
    m->d_out = nullptr;
    ES_MCUDA(cudaMalloc(&m->d_out, sizeof(uint4) * cap), "cudaMalloc(survivors)");
    m->cap = cap;
    m->P.out = m->d_out;
    m->P.out_cap = cap;
    return ES_OK;
}

int es_mitm_reset(es_mitm* m) {
    if (!m) return mfail(ES_ERR_ARG, "null MITM engine");
    ES_MCUDA(cudaMemsetAsync(m->d_cnt, 0, 8ull * 2, m->stream), "memset");
    return ES_OK;
}

int es_mitm_scan(es_mitm* m, uint64_t B_lo, uint64_t B_hi, uint64_t s1_begin, uint64_t s1_end) {
    if (!m) return mfail(ES_ERR_ARG, "null MITM engine");
    const u128m B = ((u128m)B_hi << 64) | B_lo;
    const u128m M = ((u128m)m->P.M_hi << 64) | m->P.M_lo;
    if (B == 0 || B > M) return mfail(ES_ERR_RANGE, "bound B must be in [1, M]");
    if (s1_begin > s1_end || s1_end > m->n1) return mfail(ES_ERR_RANGE, "s1 range outside [0, |S1|)");
    if (s1_begin == s1_end) return ES_OK;
    MitmParams P = m->P;
    P.B_lo = B_lo;
    P.B_hi = B_hi;
    P.s1_begin = s1_begin;
    P.s1_end = s1_end;
    ES_MCUDA(cudaMemsetAsync(m->d_cnt + 2, 0, 8, m->stream), "memset");
    // persistent grid, no more CTAs than there are chunks of s1 indices for their warps
    const uint64_t claims = (s1_end - s1_begin + 32ull * kMitmChunk - 1) / (32ull * kMitmChunk);
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(m->grid, (claims + kMitmThreads / 32 - 1) /
                                                                              (kMitmThreads / 32)));
    es_mitm_kernel<<<grid, kMitmThreads, 0, m->stream>>>(P);
    ES_MCUDA(cudaGetLastError(), "MITM launch");
    return ES_OK;
}

int es_mitm_results(es_mitm* m, uint64_t* n_lo, uint64_t* n_hi, uint64_t cap, uint64_t* n_surv,
                    uint64_t* n_cand) {
    if (!m || !n_surv) return mfail(ES_ERR_ARG, "null argument");
    ES_MCUDA(cudaMemcpyAsync(m->h_cnt, m->d_cnt, 16, cudaMemcpyDeviceToHost, m->stream), "copy");
    ES_MCUDA(cudaStreamSynchronize(m->stream), "MITM kernel execution");
    const uint64_t cnt = m->h_cnt[0];
    *n_surv = cnt;
    if (n_cand) *n_cand = m->h_cnt[1];
    if (cnt > m->cap)
        return mfail(ES_ERR_OVERFLOW, "MITM survivor buffer overflow (" + std::to_string(cnt) + " > " +
                                          std::to_string(m->cap) + ")");
    if (cnt > cap) return mfail(ES_ERR_OVERFLOW, "output buffer smaller than the survivor count");
    if (!cnt) return ES_OK;
    std::vector<uint4> tmp(cnt);
    ES_MCUDA(cudaMemcpy(tmp.data(), m->d_out, sizeof(uint4) * cnt, cudaMemcpyDeviceToHost), "copy");
    for (uint64_t i = 0; i < cnt; ++i) {
        if (n_lo) n_lo[i] = ((uint64_t)tmp[i].y << 32) | tmp[i].x;
        if (n_hi) n_hi[i] = ((uint64_t)tmp[i].w << 32) | tmp[i].z;
    }
    return ES_OK;
}

}  // extern "C"

// Dispatch of the scan kernel instances, the block-ordered min-reduction and the integer-pipe
// peak probe of the GB300 Erdős–Selfridge CRT-wheel sieve (sm_103a).  The scan kernel itself is
// es_scan_kernel.cuh, instantiated per layout in es_scan_wm.cu / es_scan_wmc.cu (word masks,
// production and counting launches), es_scan_pair.cu, es_scan_sc.cu, es_scan_sm.cu (word masks
// staged in shared memory) and es_scan_sp.cu (pair tables staged in shared memory).
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <tuple>

#include "../../include/es_gb300.h"
#include "es_internal.h"

namespace {

// Block-ordered minimum per search group: least (t, s) over good survivors.
// out[g*4 + 0] = found, [1] = t, [2] = s_lo, [3] = s_hi.  When the survivor count exceeds the
// buffer (records were dropped), the stored records may miss the least one: found = 2 then
// flags the overflow, t is the least block holding a good survivor as the scan kernel recorded
// it in group_found (exact; ~0 when there is none or group_found is null) and s = 0.
__global__ void es_min_kernel(const es_survivor* __restrict__ surv,
                              const unsigned long long* __restrict__ surv_n, uint64_t cap,
                              const EsItem* __restrict__ items,
                              const unsigned long long* __restrict__ group_found,
                              unsigned long long* out) {
    const uint32_t g = blockIdx.x;
    uint64_t n = *surv_n;
    if (n > cap) {
        if (threadIdx.x == 0) {
            out[4 * g + 0] = 2ull;
            out[4 * g + 1] = group_found ? group_found[g] : ~0ull;
            out[4 * g + 2] = 0ull;
            out[4 * g + 3] = 0ull;
        }
        return;
    }
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

// Integer throughput probes, 8 independent chains per thread, 16 steps per iteration.
// MIX = false: one IADD3-class add and one LOP3 per chain and step, both on the ALU pipe (the
//   ALU pipe's ceiling, 16 lanes per clock per scheduler).
// MIX = true: one LOP3 (ALU pipe) and one IMAD (mad.lo.u32 with a run-time multiplier, FMA pipe)
//   per chain and step: the two integer pipes together, up to the issue limit of one warp
//   instruction per clock per scheduler -- the ceiling of an integer kernel that, like the scan,
//   issues both.
// Ops counted = 16 per step per thread (lanes x instructions) in both modes.
template <bool MIX>
__global__ void __launch_bounds__(256) es_int_peak_kernel(unsigned long long* sink, int iters,
                                                         uint32_t seed) {
    uint32_t a0 = seed ^ threadIdx.x, a1 = a0 * 3u + 1u, a2 = a0 * 5u + 7u, a3 = a0 * 7u + 3u;
    uint32_t a4 = a0 + 11u, a5 = a1 ^ 0x55u, a6 = a2 + 0x99u, a7 = a3 ^ 0x1234u;
    const uint32_t c1 = seed * 13u + 5u, c2 = seed * 29u + 17u;
    const uint32_t m1 = (seed | 1u) * 0x9e3779b1u, m2 = (seed | 3u) * 0x85ebca6bu;   // run-time odd
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            if (MIX) {
                asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a0) : "r"(m1), "r"(a1));
                asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a1) : "r"(m2), "r"(a2));
                asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a2) : "r"(m1), "r"(a3));
                asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a3) : "r"(m2), "r"(a4));
                asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a4) : "r"(m1), "r"(a5));
                asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a5) : "r"(m2), "r"(a6));
                asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a6) : "r"(m1), "r"(a7));
                asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a7) : "r"(m2), "r"(a0));
            } else {
                a0 = a0 + a1 + c1;
                a1 = a1 + a2 + c2;
                a2 = a2 + a3 + c1;
                a3 = a3 + a4 + c2;
                a4 = a4 + a5 + c1;
                a5 = a5 + a6 + c2;
                a6 = a6 + a7 + c1;
                a7 = a7 + a0 + c2;
            }
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

ScanFn pick(int layout, int count, uint32_t words, uint32_t f) {
    if (layout == ES_LAYOUT_SCALAR) return es_pick_scalar(count, f);
    // staged tables exist for inner rings of one or two words (the host resolves any other
    // ring to the word-mask layout before it asks)
    if (layout == ES_LAYOUT_SMEM) return (words == 1 || words == 2) ? es_pick_smem(count, words, f) : nullptr;
    if (layout == ES_LAYOUT_SMEM_PAIR) return (words == 1 || words == 2) ? es_pick_smem_pair(count, words, f) : nullptr;
    // pair tables exist for inner rings of one or two words.  words == 0 (a batch whose plans
    // differ in width) and wider rings take the generic word-mask instance, which reads each
    // plan's own width: a fixed-width instance would index past a narrower plan's tables.
    if (layout == ES_LAYOUT_PAIR && (words == 1 || words == 2)) return es_pick_pair(count, words, f);
    return count ? es_pick_wordmask_count(words, f) : es_pick_wordmask_fast(words, f);
}

}  // namespace

// Raise the dynamic shared-memory limit of every scan instance once per process/device.
int es_scan_prepare(int smem_optin_bytes) {
    const uint32_t fs[8] = {0, 1, 2, 3, 4, 5, 6, 8};
    const uint32_t ws[4] = {1, 2, 3, 5};   // every word-count instance: 1, 2, 3-4, generic
    for (int layout = 0; layout < 5; ++layout)
        for (int count = 0; count < 2; ++count)
            for (uint32_t w : ws)
                for (uint32_t f : fs) {
                    if ((layout == ES_LAYOUT_SMEM || layout == ES_LAYOUT_SMEM_PAIR) && w > 2) continue;
                    const ScanFn fn = pick(layout, count, w, f);
                    if (!fn) return (int)cudaErrorInvalidDeviceFunction;
                    cudaError_t e = cudaFuncSetAttribute(fn,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         smem_optin_bytes);
                    if (e != cudaSuccess) return (int)e;
                }
    return 0;
}

// Resident CTAs per SM of one instance and launch shape, cached: every launch asks, and the
// answer only depends on the instance, the CTA size and the shared memory.
int es_scan_occupancy(int layout, int count, uint32_t words, uint32_t mask_filters, int threads,
                      int smem_bytes, int* ctas_per_sm) {
    const ScanFn fn = pick(layout, count, words, mask_filters);
    if (!fn) return (int)cudaErrorInvalidDeviceFunction;
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(reinterpret_cast<const void*>(fn), threads, smem_bytes, dev);
    static std::mutex mu;
    static std::map<std::tuple<const void*, int, int, int>, int> cache;
    {
        std::lock_guard<std::mutex> lock(mu);
        const auto it = cache.find(key);
        if (it != cache.end()) {
            *ctas_per_sm = it->second;
            return 0;
        }
    }
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, threads, (size_t)smem_bytes);
    if (e == cudaSuccess) {
        std::lock_guard<std::mutex> lock(mu);
        cache[key] = *ctas_per_sm;
    }
    return (int)e;
}

int es_launch_scan(const EsLaunch& L, int layout, int count, uint32_t words, int grid, void* stream) {
    const ScanFn fn = pick(layout, count, words, L.mask_filters);
    if (!fn) return (int)cudaErrorInvalidDeviceFunction;
    fn<<<grid, L.threads, L.smem_bytes, (cudaStream_t)stream>>>(L);
    return (int)cudaGetLastError();
}

int es_launch_min(const es_survivor* surv, const unsigned long long* surv_n, uint64_t cap,
                  const EsItem* items, uint32_t n_groups, const unsigned long long* group_found,
                  unsigned long long* group_min, void* stream) {
    if (n_groups == 0) return 0;
    es_min_kernel<<<n_groups, 256, 0, (cudaStream_t)stream>>>(surv, surv_n, cap, items, group_found,
                                                              group_min);
    return (int)cudaGetLastError();
}

int es_launch_int_peak(unsigned long long* sink, int grid, int threads, int iters, int mix, void* stream) {
    if (mix)
        es_int_peak_kernel<true><<<grid, threads, 0, (cudaStream_t)stream>>>(sink, iters, 0x2545f491u);
    else
        es_int_peak_kernel<false><<<grid, threads, 0, (cudaStream_t)stream>>>(sink, iters, 0x2545f491u);
    return (int)cudaGetLastError();
}

// Host side of the C ABI (include/es_gb300.h): validates a plan descriptor, derives every
// device table in C++ (sorted inner ring, carry-split keys and buckets, ring-1 residue table,
// ring-2 delta table, word-mask phase tables), uploads them in one arena per plan, and drives
// single-plan launches (the reference GpuSieve._launch surface) and persistent batch launches
// with CUDA-graph replay.  No exception crosses the ABI: every entry point returns an int.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/es_gb300.h"
#include "es_internal.h"

typedef unsigned __int128 u128;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return ES_ERR_CUDA;
}

#define ES_CUDA(call, what)                                  \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return cuda_fail(_e, what);   \
    } while (0)

u128 mk(uint64_t lo, uint64_t hi) { return ((u128)hi << 64) | lo; }
uint32_t bitlen128(u128 x) {
    uint32_t n = 0;
    while (x) { ++n; x >>= 1; }
    return n;
}
uint32_t mod_q(u128 x, uint32_t q) { return (uint32_t)(x % q); }

struct DeviceFacts {
    int dev = -1;
    int sms = 0;
    int smem_optin = 0;
    bool prepared = false;
};
DeviceFacts g_dev;

int device_facts() {
    int dev = 0;
    ES_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (g_dev.dev == dev && g_dev.prepared) return ES_OK;
    int major = 0, minor = 0;
    ES_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev), "attr");
    ES_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev), "attr");
    if (major != 10 || minor != 3)
        return fail(ES_ERR_NODEV, "device is sm_" + std::to_string(major * 10 + minor) +
                                      ", this library is built for sm_103a only");
    g_dev.dev = dev;
    ES_CUDA(cudaDeviceGetAttribute(&g_dev.sms, cudaDevAttrMultiProcessorCount, dev), "attr");
    ES_CUDA(cudaDeviceGetAttribute(&g_dev.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
            "attr");
    int e = es_scan_prepare(g_dev.smem_optin - 1024);
    if (e) return cuda_fail((cudaError_t)e, "cudaFuncSetAttribute(scan)");
    g_dev.prepared = true;
    return ES_OK;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int check_tune(const es_tune& t) {
    if (t.layout > ES_LAYOUT_AUTO)
        return fail(ES_ERR_ARG, "tune.layout must be 0 (word-mask), 1 (scalar), 2 (pair), 3 (word masks in shared "
                                "memory), 4 (pair tables in shared memory) or 5 (chosen per launch)");
    if (t.mask_filters < 1 || t.mask_filters > ES_MAX_MASK_FILTERS)
        return fail(ES_ERR_ARG, "tune.mask_filters must be in 1..8");
    if (t.threads < 64 || t.threads > 1024 || t.threads % 32)
        return fail(ES_ERR_ARG, "tune.threads must be a multiple of 32 in [64, 1024]");
    if (t.strip < 1 || t.strip > 4096) return fail(ES_ERR_ARG, "tune.strip must be in 1..4096");
    if (t.ctas_per_sm < 1 || t.ctas_per_sm > 16)
        return fail(ES_ERR_ARG, "tune.ctas_per_sm must be in 1..16");
    return ES_OK;
}

es_tune default_tune() {
    es_tune t;
    t.layout = ES_LAYOUT_WORDMASK;
    t.mask_filters = 4;
    t.threads = 512;
    t.strip = 8;
    t.smem_kb = 0;
    t.ctas_per_sm = 4;
    t.count_stages = 0;
    t.reserved = 0;
    return t;
}

}  // namespace

// ------------------------------------------------------------------------------------------
struct es_ctx {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    es_tune tune{};
    EsInst h_inst{};
    EsInst* d_inst = nullptr;
    unsigned char* d_arena = nullptr;
    size_t arena_bytes = 0;
    uint64_t table_bytes = 0;
    std::vector<uint32_t> q;
    u128 M = 1;
    uint32_t tconst[ES_MAX_FILTERS] = {0};
    uint64_t t = 0;
    // launch state
    unsigned long long* d_counts = nullptr;
    es_survivor* d_surv = nullptr;
    uint64_t surv_cap = 0;
    unsigned long long* d_surv_n = nullptr;
    unsigned long long* d_unit = nullptr;
    unsigned long long* d_found = nullptr;
    unsigned long long* d_min = nullptr;
    unsigned long long* h_pin = nullptr;  // pinned scalars for small readbacks
    uint64_t* d_list = nullptr;
    uint64_t list_cap = 0;
    bool launched = false;
};

struct es_batch {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    es_tune tune{};
    std::vector<es_ctx*> ctxs;
    std::vector<EsItem> h_items;
    std::vector<uint32_t> nf_of_item;
    uint32_t n_groups = 0;
    EsItem* d_items = nullptr;
    uint32_t* d_tconst = nullptr;
    unsigned long long* d_counts = nullptr;
    uint64_t counts_words = 0;
    std::vector<uint64_t> count_off;
    es_survivor* d_surv = nullptr;
    uint64_t surv_cap = 0;
    unsigned long long* d_surv_n = nullptr;
    unsigned long long* d_unit = nullptr;
    unsigned long long* d_found = nullptr;
    unsigned long long* d_min = nullptr;
    unsigned long long* d_item_next = nullptr;   // per-item warp-unit counters (several plans)
    uint32_t n_items = 0;
    EsItem* d_items_launch = nullptr;  // the items grouped by width class, as the launches see them
    // One persistent launch per inner-ring width class (1, 2, 3-4 words, wider): each runs the
    // kernel instance specialised for its width instead of one generic instance for all.
    struct Sub {
        EsLaunch L{};
        int grid = 0;
        uint32_t words = 0;
        uint32_t layout = 0;   // the layout this launch runs (launch_layout)
    };
    std::vector<Sub> subs;
    bool ran = false;
};

namespace {

// Shared-memory plan of one launch:
// [small tables | staged phase tables (ES_LAYOUT_SMEM, _SMEM_PAIR) | per-warp stage counters |
//  per-warp slots].
struct SmemPlan {
    uint32_t stage_off, cnt_off, queue_off, bytes;
};

// per-warp slot: entry queue, lane records, tail context (the kernel's EsQueue)
constexpr uint32_t kQueueBytes = ES_QUEUE_BYTES;

SmemPlan plan_smem(uint32_t small_max, uint32_t nf_max, const es_tune& tune, uint32_t stage_words = 0) {
    SmemPlan p;
    const uint32_t warps = tune.threads / 32u;
    const uint32_t queues = kQueueBytes * warps;
    // per-warp stage counters exist only in counting launches; shared memory is kept small so
    // that the CUDA driver's carveout leaves the rest of the SM's 256 KB to L1 (the phase tables),
    // unless the launch stages those tables in shared memory itself
    const uint32_t counters = tune.count_stages ? (uint32_t)align_up(4ull * nf_max * warps, 16) : 0u;
    p.stage_off = small_max;
    p.cnt_off = p.stage_off + (uint32_t)align_up(4ull * stage_words, 16);
    p.queue_off = p.cnt_off + counters;
    p.bytes = p.queue_off + queues;
    return p;
}

// Words of inner-stage tables a launch of `layout` copies into shared memory, given the word-mask
// words of its first F filters (EsInst::mask_off[F]): those words (ES_LAYOUT_SMEM), twice them as
// pair tables (ES_LAYOUT_SMEM_PAIR), or none.
uint32_t staged_words(uint32_t layout, uint32_t mask_words) {
    if (layout == ES_LAYOUT_SMEM) return mask_words;
    if (layout == ES_LAYOUT_SMEM_PAIR) return 2u * mask_words;
    return 0u;
}

// Launches per batch: four width classes, each split into staged and unstaged plans.
constexpr uint32_t kMaxSubs = 8;

// Word-mask bytes of the inner-stage tables that fit the L1 beside the scan's own shared memory.
constexpr uint32_t kL1TableBudget = 180u * 1024u;

// The layout a launch actually runs, given the word-mask words of its inner-stage tables (the
// largest among its plans).  A staged layout only for inner rings of one or two words whose
// staged tables fit the opt-in shared memory beside the rest of the launch's shared memory;
// otherwise the same tables read through L1 (word masks, or pair tables).  ES_LAYOUT_AUTO: staged
// word masks where they fit, else word masks through L1 when those fit L1 and pair tables would
// not, else pair tables (wider rings: word masks).  No choice changes which candidates pass.
uint32_t launch_layout(uint32_t layout, uint32_t words, uint32_t small_max, uint32_t nf_max,
                       const es_tune& tune, uint32_t mask_words) {
    auto fits = [&](uint32_t l) {
        return plan_smem(small_max, nf_max, tune, staged_words(l, mask_words)).bytes <=
               (uint32_t)g_dev.smem_optin - 1024u;
    };
    const bool narrow = words == 1 || words == 2;
    if (layout == ES_LAYOUT_AUTO) {
        if (!narrow) return ES_LAYOUT_WORDMASK;
        if (fits(ES_LAYOUT_SMEM)) return ES_LAYOUT_SMEM;
        const uint64_t bytes = 4ull * mask_words;
        return (bytes <= kL1TableBudget && kL1TableBudget < 2 * bytes) ? ES_LAYOUT_WORDMASK : ES_LAYOUT_PAIR;
    }
    if (layout != ES_LAYOUT_SMEM && layout != ES_LAYOUT_SMEM_PAIR) return layout;
    if (!narrow) return ES_LAYOUT_WORDMASK;
    if (fits(layout)) return layout;
    return layout == ES_LAYOUT_SMEM ? ES_LAYOUT_WORDMASK : ES_LAYOUT_PAIR;
}

// Filters of the inner-ring stage actually compiled into the launched kernel: word-mask kernels
// are instantiated for exactly 0..6 and 8 filters (never more than the plan has or the tables
// built); the scalar layout takes a runtime count.
uint32_t stage_filters(uint32_t layout, uint32_t requested, uint32_t nf, uint32_t built) {
    if (layout == ES_LAYOUT_SCALAR) return std::max<uint32_t>(requested, 1);
    uint32_t f = std::min(std::min(requested, nf), built);
    return f == 7 ? 6 : f;
}

int grid_for(uint32_t layout, uint32_t count, uint32_t words, uint32_t filters, const es_tune& tune,
             uint32_t smem, uint64_t units, int* grid) {
    int occ = 0;
    int e = es_scan_occupancy((int)layout, (int)count, words, filters, (int)tune.threads,
                              (int)smem, &occ);
    if (e) return cuda_fail((cudaError_t)e, "occupancy");
    if (occ < 1) return fail(ES_ERR_ARG, "launch shape does not fit one SM (threads/smem)");
    uint64_t g = (uint64_t)g_dev.sms * (uint64_t)std::min<uint32_t>((uint32_t)occ, tune.ctas_per_sm);
    if (units < g) g = units;
    if (g < 1) g = 1;
    *grid = (int)g;
    return ES_OK;
}

uint64_t cycles_of(const EsInst& I, uint64_t ob, uint64_t oe, uint64_t* cb) {
    *cb = ob / I.r1;
    const uint64_t ce = (oe + I.r1 - 1) / I.r1;
    return ce - *cb;
}

// Warp-units of the ring-1 cycles [cb, ce) (the kernel's unit decode follows the same rule):
// with a ring 2, 32 ring-2 rows x one window of at most `strip` ring-2 digits (ceil(r2 / strip)
// balanced windows per row); without one, 32 lanes x `strip` consecutive cycles.
uint64_t units_of(const EsInst& I, uint64_t cb, uint64_t ce, uint32_t strip) {
    if (ce <= cb) return 0;
    if (I.r2 <= 1) return (ce - cb + 32ull * strip - 1) / (32ull * strip);
    const uint64_t rows = (ce + I.r2 - 1) / I.r2 - cb / I.r2;
    return (rows + 31) / 32 * ((I.r2 + strip - 1) / strip);
}

}  // namespace

void es_set_last_error(const char* msg) { g_err = msg ? msg : ""; }

// ------------------------------------------------------------------------------------------
extern "C" {

const char* es_last_error(void) { return g_err.c_str(); }

int es_abi_version(void) { return ES_ABI_VERSION; }

int es_device_info(int* sm_count, int* cc_major, int* cc_minor, uint64_t* smem_optin_bytes) {
    int dev = 0;
    ES_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    int a = 0, b = 0, s = 0, o = 0;
    ES_CUDA(cudaDeviceGetAttribute(&a, cudaDevAttrComputeCapabilityMajor, dev), "attr");
    ES_CUDA(cudaDeviceGetAttribute(&b, cudaDevAttrComputeCapabilityMinor, dev), "attr");
    ES_CUDA(cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev), "attr");
    ES_CUDA(cudaDeviceGetAttribute(&o, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "attr");
    if (sm_count) *sm_count = s;
    if (cc_major) *cc_major = a;
    if (cc_minor) *cc_minor = b;
    if (smem_optin_bytes) *smem_optin_bytes = (uint64_t)o;
    return ES_OK;
}

int es_device_name(char* out, uint32_t cap) {
    if (!out || cap == 0) return fail(ES_ERR_ARG, "null or empty output buffer");
    int dev = 0;
    ES_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    cudaDeviceProp prop;
    ES_CUDA(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
    snprintf(out, cap, "%s", prop.name);
    return ES_OK;
}

int es_ctx_destroy(es_ctx* c) {
    if (!c) return ES_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->d_arena);
    cudaFree(c->d_counts);
    cudaFree(c->d_surv);
    cudaFree(c->d_surv_n);
    cudaFree(c->d_list);
    if (c->h_pin) cudaFreeHost(c->h_pin);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return ES_OK;
}

int es_ctx_create(const es_plan_desc* d, const es_tune* tune_in, es_ctx** out) {
    if (!d || !out) return fail(ES_ERR_ARG, "null descriptor or output pointer");
    *out = nullptr;
    es_tune tune = tune_in ? *tune_in : default_tune();
    if (int e = check_tune(tune)) return e;
    if (d->flags != 0) return fail(ES_ERR_ARG, "descriptor flags must be 0");
    const u128 M = mk(d->M_lo, d->M_hi);
    if (M == 0 || bitlen128(M) > 126) return fail(ES_ERR_RANGE, "wheel modulus must be in [1, 2^126)");
    if (d->n_filters > ES_MAX_FILTERS)
        return fail(ES_ERR_RANGE, "too many residual filters (max " + std::to_string(ES_MAX_FILTERS) + ")");
    if (d->n_rings > ES_MAX_RINGS - 3) return fail(ES_ERR_RANGE, "too many wheel rings");
    if (d->n_rings && (!d->radix || !d->term_lo || !d->term_hi))
        return fail(ES_ERR_ARG, "null ring arrays");
    if (d->n_filters && (!d->filter_q || !d->allowed)) return fail(ES_ERR_ARG, "null filter arrays");
    if (int e = device_facts()) return e;

    // ---- rings (padded to >= 3 with radix-1 rings whose only term is 0) -------------------
    std::vector<uint32_t> radix;
    std::vector<u128> terms;
    std::vector<uint32_t> roff;
    uint64_t R = 1;
    size_t pos = 0;
    for (uint32_t j = 0; j < d->n_rings; ++j) {
        const uint32_t r = d->radix[j];
        if (r == 0 || r > 65535) return fail(ES_ERR_RANGE, "ring radix must be in [1, 65535]");
        roff.push_back((uint32_t)terms.size());
        radix.push_back(r);
        for (uint32_t i = 0; i < r; ++i, ++pos) {
            const u128 v = mk(d->term_lo[pos], d->term_hi[pos]);
            if (v >= M) return fail(ES_ERR_ARG, "ring term not reduced mod M");
            terms.push_back(v);
        }
        if (R > (1ull << 62) / r) return fail(ES_ERR_RANGE, "residues per block exceed 2^62");
        R *= r;
    }
    while (radix.size() < 3) {
        roff.push_back((uint32_t)terms.size());
        radix.push_back(1);
        terms.push_back(0);
    }
    const uint32_t nr = (uint32_t)radix.size();
    const uint32_t r0 = radix[0], r1 = radix[1], r2 = radix[2];
    const uint32_t nf = d->n_filters;
    const uint32_t FB = std::min<uint32_t>(ES_FMAX, nf);
    const uint32_t W = (r0 + 31) / 32;

    es_ctx* c = new (std::nothrow) es_ctx();
    if (!c) return fail(ES_ERR_NOMEM, "host allocation");
    c->tune = tune;
    c->M = M;
    c->q.assign(d->filter_q, d->filter_q + nf);

    // ---- filters ------------------------------------------------------------------------
    std::vector<EsFilterC> fc(nf);
    std::vector<uint32_t> bit_off(nf + 1, 0);
    for (uint32_t f = 0; f < nf; ++f) {
        const uint32_t q = c->q[f];
        if (q < 2 || q >= ES_MAX_Q) {
            es_ctx_destroy(c);
            return fail(ES_ERR_RANGE, "filter modulus must be in [2, 2^20)");
        }
        bit_off[f + 1] = bit_off[f] + (q + 31) / 32;
        fc[f].q = q;
        fc[f].corr = (uint32_t)((q - mod_q(M, q)) % q);
        fc[f].w1 = mod_q((u128)1 << 32, q);
        fc[f].w2 = mod_q((u128)1 << 64, q);
        fc[f].w3 = mod_q((u128)1 << 96, q);
        fc[f].off = bit_off[f];
        fc[f].rcp = (uint64_t)(((u128)1 << 64) / q);
    }
    auto admissible = [&](uint32_t f, uint32_t r) -> uint32_t {
        return (d->allowed[bit_off[f] + (r >> 5)] >> (r & 31u)) & 1u;
    };

    // ---- inner ring: sorted slots, keys, buckets ----------------------------------------
    std::vector<uint32_t> order(r0);
    for (uint32_t i = 0; i < r0; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return terms[roff[0] + a] < terms[roff[0] + b]; });
    std::vector<u128> S0(r0);
    for (uint32_t i = 0; i < r0; ++i) S0[i] = terms[roff[0] + order[i]];
    const uint32_t bl = bitlen128(M);
    const uint32_t sh = bl > 32 ? bl - 32 : 0;
    const uint32_t kbits = bitlen128(M >> sh);
    const uint32_t bsh = kbits > ES_NBUCKET_LOG2 ? kbits - ES_NBUCKET_LOG2 : 0;
    std::vector<uint32_t> K0(r0);
    for (uint32_t i = 0; i < r0; ++i) K0[i] = (uint32_t)(S0[i] >> sh);
    // bucket b: the first sorted slot whose key is >= b << bsh, and the keys of that slot and
    // the next two (0xffffffff past the end), so that one 16-byte load settles the split
    std::vector<uint32_t> BK(4ull * (ES_NBUCKET + 1));
    for (uint32_t bkt = 0; bkt <= ES_NBUCKET; ++bkt) {
        const uint64_t lim = (uint64_t)bkt << bsh;
        uint32_t n = 0;
        while (n < r0 && (uint64_t)K0[n] < lim) ++n;
        BK[4 * bkt] = n;
        for (uint32_t j = 0; j < 3; ++j) BK[4 * bkt + 1 + j] = n + j < r0 ? K0[n + j] : 0xffffffffu;
    }

    // ---- small block ----------------------------------------------------------------------
    EsInst& I = c->h_inst;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 16); return (uint32_t)o; };
    I.o_T1 = take(16ull * r1);
    I.o_TQ1 = take(4ull * ES_FMAX * r1);
    I.o_D2 = take(16ull * r2);
    I.o_DQ2 = take(4ull * ES_FMAX * r2);
    I.o_S0 = take(16ull * (r0 + 1));   // + sentinel S0[r0] = M
    I.o_K0 = take(4ull * (r0 + 1));    // + sentinel K0[r0] = 0xffffffff
    I.o_I0 = take(4ull * r0);
    I.o_Q0 = take(4ull * ES_FMAX * r0);
    I.o_BK = take(16ull * (ES_NBUCKET + 1));
    I.o_FC = take(sizeof(EsFilterC) * std::max<uint32_t>(nf, 1));
    I.o_K1 = take(4ull * r1);
    const size_t small_bytes = off;
    std::vector<unsigned char> small(small_bytes, 0);
    auto put128 = [&](uint32_t o, uint32_t i, u128 v) {
        uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
        memcpy(&small[o + 16ull * i], &lo, 8);
        memcpy(&small[o + 16ull * i + 8], &hi, 8);
    };
    auto put32 = [&](uint32_t o, uint32_t i, uint32_t v) { memcpy(&small[o + 4ull * i], &v, 4); };
    for (uint32_t i = 0; i < r1; ++i) {
        const u128 v = terms[roff[1] + i];
        put128(I.o_T1, i, v);
        put32(I.o_K1, i, (uint32_t)(v >> sh));
        for (uint32_t f = 0; f < FB; ++f) put32(I.o_TQ1, i * ES_FMAX + f, mod_q(v, c->q[f]));
    }
    for (uint32_t i = 0; i < r2; ++i) {
        const u128 a = terms[roff[2] + i], b = terms[roff[2] + (i + 1) % r2];
        const u128 dlt = b >= a ? b - a : b + (M - a);
        put128(I.o_D2, i, dlt);
        for (uint32_t f = 0; f < FB; ++f) put32(I.o_DQ2, i * ES_FMAX + f, mod_q(dlt, c->q[f]));
    }
    for (uint32_t i = 0; i < r0; ++i) {
        put128(I.o_S0, i, S0[i]);
        put32(I.o_K0, i, K0[i]);
        put32(I.o_I0, i, order[i]);
        for (uint32_t f = 0; f < FB; ++f) put32(I.o_Q0, f * r0 + i, mod_q(S0[i], c->q[f]));
    }
    put128(I.o_S0, r0, M);             // stops the tie scan: M < thr never holds (thr <= M)
    put32(I.o_K0, r0, 0xffffffffu);    // stops the key scan: never < t32
    memcpy(&small[I.o_BK], BK.data(), 16ull * (ES_NBUCKET + 1));
    if (nf) memcpy(&small[I.o_FC], fc.data(), sizeof(EsFilterC) * nf);

    // ---- word-mask phase tables for the first FB filters ---------------------------------
    // rows of RS words: W, except three-word rings, whose rows are padded to four words so that
    // one 16-byte load reads a row
    const uint32_t RS = W == 3 ? 4u : W;
    std::vector<uint32_t> mask_off(ES_FMAX + 1, 0);
    for (uint32_t f = 0; f < ES_FMAX; ++f)
        mask_off[f + 1] = mask_off[f] + (f < FB ? (uint32_t)align_up((uint64_t)c->q[f] * RS, 4) : 0u);
    std::vector<uint32_t> masks(std::max<uint32_t>(mask_off[ES_FMAX], 4), 0u);
    for (uint32_t f = 0; f < FB; ++f) {
        const uint32_t q = c->q[f];
        uint32_t* P = masks.data() + mask_off[f];
        for (uint32_t i = 0; i < r0; ++i) {
            const uint32_t a = mod_q(S0[i], q);
            const uint32_t wd = i >> 5, bit = 1u << (i & 31u);
            uint32_t r = a;
            for (uint32_t ph = 0; ph < q; ++ph) {
                if (admissible(f, r)) P[(uint64_t)ph * RS + wd] |= bit;
                if (++r == q) r = 0;
            }
        }
    }
    // pair tables (inner rings of at most two words): phase row phi holds P_f[phi] and then the
    // row a wrap past M selects, P_f[(phi + corr_f) mod q_f], so one load serves both sides of
    // the carry split; filter f starts at word 2 * mask_off[f]
    std::vector<uint32_t> pairs;
    if (W <= 2) {
        pairs.assign(2ull * masks.size(), 0u);
        for (uint32_t f = 0; f < FB; ++f) {
            const uint32_t q = c->q[f], corr = fc[f].corr;
            const uint32_t* P = masks.data() + mask_off[f];
            uint32_t* D = pairs.data() + 2ull * mask_off[f];
            for (uint32_t ph = 0; ph < q; ++ph) {
                const uint32_t ph1 = (uint32_t)(((uint64_t)ph + corr) % q);
                for (uint32_t wd = 0; wd < W; ++wd) {
                    D[(uint64_t)ph * 2 * W + wd] = P[(uint64_t)ph * W + wd];
                    D[(uint64_t)ph * 2 * W + W + wd] = P[(uint64_t)ph1 * W + wd];
                }
            }
        }
    }

    // ---- arena ----------------------------------------------------------------------------
    size_t aoff = 0;
    auto atake = [&](size_t bytes) { size_t o = aoff; aoff = align_up(aoff + bytes, 256); return o; };
    const size_t a_inst = atake(sizeof(EsInst));
    const size_t a_small = atake(small_bytes);
    const size_t a_masks = atake(4ull * masks.size());
    const size_t a_pairs = atake(4ull * std::max<size_t>(pairs.size(), 4));
    const size_t a_bits = atake(4ull * std::max<uint32_t>(bit_off[nf], 4));
    const size_t a_terms = atake(16ull * terms.size());
    const size_t a_roff = atake(4ull * nr);
    const size_t a_radix = atake(4ull * nr);
    c->arena_bytes = aoff;
    std::vector<unsigned char> img(aoff, 0);
    memcpy(&img[a_small], small.data(), small_bytes);
    memcpy(&img[a_masks], masks.data(), 4ull * masks.size());
    if (!pairs.empty()) memcpy(&img[a_pairs], pairs.data(), 4ull * pairs.size());
    if (bit_off[nf]) memcpy(&img[a_bits], d->allowed, 4ull * bit_off[nf]);
    for (size_t i = 0; i < terms.size(); ++i) {
        uint64_t lo = (uint64_t)terms[i], hi = (uint64_t)(terms[i] >> 64);
        memcpy(&img[a_terms + 16 * i], &lo, 8);
        memcpy(&img[a_terms + 16 * i + 8], &hi, 8);
    }
    memcpy(&img[a_roff], roff.data(), 4ull * nr);
    memcpy(&img[a_radix], radix.data(), 4ull * nr);

    cudaError_t ce = cudaMalloc(&c->d_arena, aoff);
    if (ce != cudaSuccess) { es_ctx_destroy(c); return cuda_fail(ce, "cudaMalloc(arena)"); }
    I.M_lo = (uint64_t)M;
    I.M_hi = (uint64_t)(M >> 64);
    I.n_outer = R / r0;
    I.n_cycles = I.n_outer / r1;
    I.k = d->k;
    I.n_rings = nr;
    I.r0 = r0; I.W = W; I.r1 = r1; I.r2 = r2;
    I.n_filters = nf;
    I.F_built = FB;
    I.sh = sh;
    I.bsh = bsh;
    I.tail_mask = (r0 % 32) ? ((1u << (r0 % 32)) - 1u) : 0xffffffffu;
    I.km = (uint32_t)(M >> sh);
    I.small_bytes = (uint32_t)small_bytes;
    for (uint32_t f = 0; f <= ES_FMAX; ++f) I.mask_off[f] = mask_off[f];
    I.mask_stride = RS;
    I.small = c->d_arena + a_small;
    I.masks = reinterpret_cast<const uint32_t*>(c->d_arena + a_masks);
    I.pairs = reinterpret_cast<const uint32_t*>(c->d_arena + a_pairs);
    I.allowed = reinterpret_cast<const uint32_t*>(c->d_arena + a_bits);
    I.ring_terms = reinterpret_cast<const uint64_t*>(c->d_arena + a_terms);
    I.ring_off = reinterpret_cast<const uint32_t*>(c->d_arena + a_roff);
    I.radix = reinterpret_cast<const uint32_t*>(c->d_arena + a_radix);
    memcpy(&img[a_inst], &I, sizeof(EsInst));
    c->d_inst = reinterpret_cast<EsInst*>(c->d_arena + a_inst);
    c->table_bytes = aoff;

    ce = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaMemcpy(c->d_arena, img.data(), aoff, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaEventCreate(&c->ev0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&c->ev1);
    if (ce == cudaSuccess) ce = cudaMalloc(&c->d_counts, 8ull * std::max<uint32_t>(nf, 1));
    if (ce == cudaSuccess) ce = cudaMalloc(&c->d_surv_n, 8ull * 8);
    if (ce == cudaSuccess) ce = cudaHostAlloc(&c->h_pin, 8ull * 8, cudaHostAllocDefault);
    if (ce == cudaSuccess) ce = cudaMemset(c->d_counts, 0, 8ull * std::max<uint32_t>(nf, 1));
    if (ce == cudaSuccess) ce = cudaMemset(c->d_surv_n, 0, 8ull * 8);
    if (ce != cudaSuccess) { es_ctx_destroy(c); return cuda_fail(ce, "context setup"); }
    // d_surv_n block: [0] survivor count, [1] unit counter, [2] group found, [3..6] group min
    c->d_unit = c->d_surv_n + 1;
    c->d_found = c->d_surv_n + 2;
    c->d_min = c->d_surv_n + 3;
    ce = cudaMemset(c->d_found, 0xff, 8);
    if (ce != cudaSuccess) { es_ctx_destroy(c); return cuda_fail(ce, "context setup"); }
    int e = es_set_capacity(c, 1u << 20);
    if (e) { es_ctx_destroy(c); return e; }
    *out = c;
    return ES_OK;
}

int es_ctx_set_tune(es_ctx* c, const es_tune* t) {
    if (!c || !t) return fail(ES_ERR_ARG, "null argument");
    if (int e = check_tune(*t)) return e;
    c->tune = *t;
    return ES_OK;
}

int es_ctx_get_tune(const es_ctx* c, es_tune* t) {
    if (!c || !t) return fail(ES_ERR_ARG, "null argument");
    *t = c->tune;
    return ES_OK;
}

int es_ctx_info(const es_ctx* c, uint64_t* n_outer, uint32_t* r0, uint32_t* n_filters,
                uint64_t* table_bytes) {
    if (!c) return fail(ES_ERR_ARG, "null context");
    if (n_outer) *n_outer = c->h_inst.n_outer;
    if (r0) *r0 = c->h_inst.r0;
    if (n_filters) *n_filters = c->h_inst.n_filters;
    if (table_bytes) *table_bytes = c->table_bytes;
    return ES_OK;
}

int es_set_capacity(es_ctx* c, uint64_t cap) {
    if (!c || cap == 0 || cap > (1ull << 32)) return fail(ES_ERR_ARG, "capacity must be in [1, 2^32]");
    ES_CUDA(cudaStreamSynchronize(c->stream), "sync");
    cudaFree(c->d_surv);
    c->d_surv = nullptr;
    ES_CUDA(cudaMalloc(&c->d_surv, sizeof(es_survivor) * cap), "cudaMalloc(survivors)");
    c->surv_cap = cap;
    return ES_OK;
}

int es_set_block(es_ctx* c, const uint32_t* tconst, uint32_t n, uint64_t t) {
    if (!c) return fail(ES_ERR_ARG, "null context");
    if (n != c->h_inst.n_filters || (n && !tconst))
        return fail(ES_ERR_ARG, "tconst length must equal the number of filters");
    for (uint32_t f = 0; f < n; ++f) {
        if (tconst[f] >= c->q[f]) return fail(ES_ERR_ARG, "tconst[j] must be < q_j");
        c->tconst[f] = tconst[f];
    }
    c->t = t;
    return ES_OK;
}

int es_reset_survivors(es_ctx* c) {
    if (!c) return fail(ES_ERR_ARG, "null context");
    ES_CUDA(cudaMemsetAsync(c->d_surv_n, 0, 8, c->stream), "memset");
    ES_CUDA(cudaMemsetAsync(c->d_found, 0xff, 8, c->stream), "memset");
    return ES_OK;
}

int es_reset_counts(es_ctx* c) {
    if (!c) return fail(ES_ERR_ARG, "null context");
    ES_CUDA(cudaMemsetAsync(c->d_counts, 0, 8ull * std::max<uint32_t>(c->h_inst.n_filters, 1),
                            c->stream), "memset");
    return ES_OK;
}

static int ctx_launch(es_ctx* c, uint64_t ob, uint64_t oe, const uint64_t* d_list) {
    const EsInst& I = c->h_inst;
    const es_tune& tn = c->tune;
    EsLaunch L;
    memset(&L, 0, sizeof(L));
    EsItem& it = L.item0;
    it.inst = c->d_inst;
    it.tconst = nullptr;
    it.list = d_list;
    it.counts = tn.count_stages ? c->d_counts : nullptr;
    it.t = c->t;
    it.o_begin = ob;
    it.o_end = oe;
    uint64_t n_work;
    if (d_list) {
        it.c_begin = it.c_end = 0;
        n_work = oe - ob;
    } else {
        n_work = cycles_of(I, ob, oe, &it.c_begin);
        it.c_end = it.c_begin + n_work;
    }
    const uint64_t per_unit = 32ull * tn.strip;
    it.unit_begin = 0;
    it.n_units = d_list ? (n_work + per_unit - 1) / per_unit : units_of(I, it.c_begin, it.c_end, tn.strip);
    it.group = 0;
    it.inst_id = 0;
    const uint32_t F = stage_filters(tn.layout, tn.mask_filters, I.n_filters, I.F_built);
    const uint32_t layout = launch_layout(tn.layout, I.W, I.small_bytes, I.n_filters, tn, I.mask_off[F]);
    const SmemPlan sp = plan_smem((uint32_t)I.small_bytes, I.n_filters, tn, staged_words(layout, I.mask_off[F]));
    it.caller = 0;
    L.items = nullptr;
    L.n_items = 1;
    L.threads = tn.threads;
    L.strip = tn.strip;
    L.mask_filters = F;
    L.total_units = it.n_units;
    L.nf_max = std::max<uint32_t>(I.n_filters, 1);
    L.direct = 1;
    L.unit_counter = c->d_unit;
    L.surv = c->d_surv;
    L.surv_n = c->d_surv_n;
    L.surv_cap = c->surv_cap;
    L.group_found = nullptr;
    L.smem_bytes = sp.bytes;
    L.cnt_off = sp.cnt_off;
    L.queue_off = sp.queue_off;
    L.stage_off = sp.stage_off;
    memcpy(L.tconst0, c->tconst, 4ull * I.n_filters);
    if (it.n_units == 0) return ES_OK;
    int grid = 0;
    if (int e = grid_for(layout, tn.count_stages, I.W, F, tn, sp.bytes, it.n_units, &grid)) return e;
    ES_CUDA(cudaMemsetAsync(c->d_unit, 0, 8, c->stream), "memset");
    int e = es_launch_scan(L, (int)layout, (int)tn.count_stages, I.W, grid, c->stream);
    if (e) return cuda_fail((cudaError_t)e, "scan launch");
    c->launched = true;
    return ES_OK;
}

int es_launch(es_ctx* c, uint64_t ostart, uint64_t ocount) {
    if (!c) return fail(ES_ERR_ARG, "null context");
    if (ostart > c->h_inst.n_outer || ocount > c->h_inst.n_outer - ostart)
        return fail(ES_ERR_RANGE, "outer range outside [0, R/r0)");
    return ctx_launch(c, ostart, ostart + ocount, nullptr);
}

int es_launch_list(es_ctx* c, const uint64_t* outer, uint64_t n) {
    if (!c || (n && !outer)) return fail(ES_ERR_ARG, "null argument");
    for (uint64_t i = 0; i < n; ++i)
        if (outer[i] >= c->h_inst.n_outer) return fail(ES_ERR_RANGE, "outer index outside [0, R/r0)");
    if (n == 0) return ES_OK;
    ES_CUDA(cudaStreamSynchronize(c->stream), "sync");
    if (n > c->list_cap) {
        cudaFree(c->d_list);
        c->d_list = nullptr;
        ES_CUDA(cudaMalloc(&c->d_list, 8ull * n), "cudaMalloc(list)");
        c->list_cap = n;
    }
    ES_CUDA(cudaMemcpy(c->d_list, outer, 8ull * n, cudaMemcpyHostToDevice), "copy list");
    return ctx_launch(c, 0, n, c->d_list);
}

int es_sync(es_ctx* c) {
    if (!c) return fail(ES_ERR_ARG, "null context");
    ES_CUDA(cudaStreamSynchronize(c->stream), "kernel execution");
    return ES_OK;
}

int es_survivor_count(es_ctx* c, uint64_t* n) {
    if (!c || !n) return fail(ES_ERR_ARG, "null argument");
    ES_CUDA(cudaMemcpyAsync(c->h_pin, c->d_surv_n, 8, cudaMemcpyDeviceToHost, c->stream), "copy");
    ES_CUDA(cudaStreamSynchronize(c->stream), "kernel execution");
    *n = c->h_pin[0];
    return ES_OK;
}

int es_read_survivor_records(es_ctx* c, es_survivor* out, uint64_t cap, uint64_t* n) {
    if (!c || !n) return fail(ES_ERR_ARG, "null argument");
    uint64_t cnt = 0;
    if (int e = es_survivor_count(c, &cnt)) return e;
    *n = cnt;
    if (cnt > c->surv_cap)
        return fail(ES_ERR_OVERFLOW, "survivor buffer overflow (" + std::to_string(cnt) + " > " +
                                         std::to_string(c->surv_cap) + "); raise max_survivors");
    if (cnt > cap) return fail(ES_ERR_OVERFLOW, "output buffer smaller than the survivor count");
    if (cnt) ES_CUDA(cudaMemcpy(out, c->d_surv, sizeof(es_survivor) * cnt, cudaMemcpyDeviceToHost), "copy");
    return ES_OK;
}

int es_read_survivors(es_ctx* c, uint64_t* idx_out, uint64_t cap, uint64_t* n) {
    if (!c || !n) return fail(ES_ERR_ARG, "null argument");
    uint64_t cnt = 0;
    if (int e = es_survivor_count(c, &cnt)) return e;
    *n = cnt;
    if (cnt > c->surv_cap)
        return fail(ES_ERR_OVERFLOW, "survivor buffer overflow (" + std::to_string(cnt) + " > " +
                                         std::to_string(c->surv_cap) + "); raise max_survivors");
    if (cnt > cap) return fail(ES_ERR_OVERFLOW, "output buffer smaller than the survivor count");
    if (!cnt) return ES_OK;
    std::vector<es_survivor> tmp(cnt);
    ES_CUDA(cudaMemcpy(tmp.data(), c->d_surv, sizeof(es_survivor) * cnt, cudaMemcpyDeviceToHost), "copy");
    for (uint64_t i = 0; i < cnt; ++i) idx_out[i] = tmp[i].idx;
    return ES_OK;
}

int es_stage_counts(es_ctx* c, uint64_t* counts, uint32_t n) {
    if (!c || (n && !counts)) return fail(ES_ERR_ARG, "null argument");
    if (n != c->h_inst.n_filters) return fail(ES_ERR_ARG, "counts length must equal the filter count");
    ES_CUDA(cudaStreamSynchronize(c->stream), "kernel execution");
    if (n) ES_CUDA(cudaMemcpy(counts, c->d_counts, 8ull * n, cudaMemcpyDeviceToHost), "copy");
    return ES_OK;
}

int es_min_survivor(es_ctx* c, int* found, uint64_t* t, uint64_t* s_lo, uint64_t* s_hi) {
    if (!c || !found) return fail(ES_ERR_ARG, "null argument");
    int e = es_launch_min(c->d_surv, c->d_surv_n, c->surv_cap, nullptr, 1, nullptr, c->d_min, c->stream);
    if (e) return cuda_fail((cudaError_t)e, "min launch");
    ES_CUDA(cudaMemcpyAsync(c->h_pin, c->d_min, 32, cudaMemcpyDeviceToHost, c->stream), "copy");
    ES_CUDA(cudaStreamSynchronize(c->stream), "kernel execution");
    if (c->h_pin[0] == 2)
        return fail(ES_ERR_OVERFLOW, "survivor buffer overflow: the minimum over the stored records "
                                     "is not reliable; raise the capacity or scan fewer positions");
    *found = (int)c->h_pin[0];
    if (t) *t = c->h_pin[1];
    if (s_lo) *s_lo = c->h_pin[2];
    if (s_hi) *s_hi = c->h_pin[3];
    return ES_OK;
}

int es_launch_timed(es_ctx* c, uint64_t ostart, uint64_t ocount, float* ms) {
    if (!c) return fail(ES_ERR_ARG, "null context");
    ES_CUDA(cudaEventRecord(c->ev0, c->stream), "event");
    if (int e = es_launch(c, ostart, ocount)) return e;
    ES_CUDA(cudaEventRecord(c->ev1, c->stream), "event");
    ES_CUDA(cudaEventSynchronize(c->ev1), "kernel execution");
    float v = 0.f;
    ES_CUDA(cudaEventElapsedTime(&v, c->ev0, c->ev1), "event");
    if (ms) *ms = v;
    return ES_OK;
}

// ---------------------------------------------------------------------------------------
int es_batch_destroy(es_batch* b) {
    if (!b) return ES_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    cudaFree(b->d_items);
    cudaFree(b->d_items_launch);
    cudaFree(b->d_tconst);
    cudaFree(b->d_counts);
    cudaFree(b->d_surv);
    cudaFree(b->d_surv_n);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return ES_OK;
}

int es_batch_create(es_ctx* const* ctxs, uint32_t n_ctx, const es_batch_item* items,
                    uint32_t n_items, const es_tune* tune_in, es_batch** out) {
    if (!ctxs || !items || !out || n_ctx == 0 || n_items == 0)
        return fail(ES_ERR_ARG, "empty batch");
    *out = nullptr;
    es_tune tune = tune_in ? *tune_in : ctxs[0]->tune;
    if (int e = check_tune(tune)) return e;
    if (int e = device_facts()) return e;
    es_batch* b = new (std::nothrow) es_batch();
    if (!b) return fail(ES_ERR_NOMEM, "host allocation");
    b->tune = tune;
    b->ctxs.assign(ctxs, ctxs + n_ctx);
    for (uint32_t i = 0; i < n_ctx; ++i)
        if (!ctxs[i]) { es_batch_destroy(b); return fail(ES_ERR_ARG, "null context in batch"); }
    // width class of a plan: the kernel instance its inner ring uses
    auto width_class = [](uint32_t W) -> uint32_t { return W <= 2 ? W : (W <= 4 ? 4u : 0u); };
    std::vector<uint32_t> h_tc;
    b->h_items.resize(n_items);
    b->count_off.resize(n_items);
    uint64_t cwords = 0;
    uint32_t max_group = 0;
    for (uint32_t i = 0; i < n_items; ++i) {
        const es_batch_item& s = items[i];
        if (s.ctx_index >= n_ctx) { es_batch_destroy(b); return fail(ES_ERR_ARG, "item ctx_index out of range"); }
        if (s.group >= n_items) { es_batch_destroy(b); return fail(ES_ERR_ARG, "item group must be < n_items"); }
        const es_ctx* c = ctxs[s.ctx_index];
        const EsInst& I = c->h_inst;
        if (s.o_begin > s.o_end || s.o_end > I.n_outer) {
            es_batch_destroy(b);
            return fail(ES_ERR_RANGE, "item outer range outside [0, R/r0)");
        }
        EsItem& it = b->h_items[i];
        memset(&it, 0, sizeof(it));
        it.inst = c->d_inst;
        it.list = nullptr;
        it.t = s.t;
        it.o_begin = s.o_begin;
        it.o_end = s.o_end;
        const uint64_t ncyc = s.o_end > s.o_begin ? cycles_of(I, s.o_begin, s.o_end, &it.c_begin) : 0;
        it.c_end = it.c_begin + ncyc;
        it.n_units = units_of(I, it.c_begin, it.c_end, tune.strip);
        it.group = s.group;
        it.inst_id = s.ctx_index;
        it.caller = i;
        // per-block constants tconst[j] = (t mod q)(M mod q) mod q
        it.tconst = reinterpret_cast<const uint32_t*>((uintptr_t)h_tc.size());  // patched below
        for (uint32_t f = 0; f < I.n_filters; ++f) {
            const uint64_t q = c->q[f];
            const uint64_t mq = (uint64_t)(c->M % q);
            h_tc.push_back((uint32_t)((s.t % q) * mq % q));
        }
        while (h_tc.size() % 4) h_tc.push_back(0);
        b->count_off[i] = cwords;
        cwords += std::max<uint32_t>(I.n_filters, 1);
        max_group = std::max<uint32_t>(max_group, s.group);
    }
    b->n_groups = max_group + 1;
    b->counts_words = cwords;
    // launch order: items grouped by width class (stable), one launch per class; with
    // ES_LAYOUT_AUTO a one- or two-word class splits further into the plans whose inner-stage
    // tables fit shared memory (staged) and the rest
    auto class_key = [&](uint32_t item) -> uint32_t {
        const EsInst& I = ctxs[items[item].ctx_index]->h_inst;
        uint32_t key = 2u * width_class(I.W);
        if (tune.layout == ES_LAYOUT_AUTO && (I.W == 1 || I.W == 2)) {
            const uint32_t Fi = stage_filters(tune.layout, tune.mask_filters, I.n_filters, I.F_built);
            if (launch_layout(ES_LAYOUT_AUTO, I.W, (uint32_t)I.small_bytes, I.n_filters, tune, I.mask_off[Fi]) ==
                ES_LAYOUT_SMEM)
                key += 1u;
        }
        return key;
    };
    std::vector<uint32_t> keys(n_items);
    for (uint32_t i = 0; i < n_items; ++i) keys[i] = class_key(i);
    std::vector<uint32_t> order(n_items);
    for (uint32_t i = 0; i < n_items; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return keys[x] < keys[y]; });
    cudaError_t ce = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreate(&b->ev0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&b->ev1);
    if (ce == cudaSuccess) ce = cudaMalloc(&b->d_items, sizeof(EsItem) * n_items);
    if (ce == cudaSuccess) ce = cudaMalloc(&b->d_items_launch, sizeof(EsItem) * n_items);
    if (ce == cudaSuccess) ce = cudaMalloc(&b->d_tconst, 4ull * std::max<size_t>(h_tc.size(), 4));
    if (ce == cudaSuccess) ce = cudaMalloc(&b->d_counts, 8ull * cwords);
    // scalars: [0] survivor count, [1..4] unit counters of the launches, then group_found[G],
    // group_min[4G], item_next[n_items]
    if (ce == cudaSuccess) ce = cudaMalloc(&b->d_surv_n, 8ull * (1 + kMaxSubs + 5ull * b->n_groups + n_items));
    b->surv_cap = ctxs[0]->surv_cap;
    if (ce == cudaSuccess) ce = cudaMalloc(&b->d_surv, sizeof(es_survivor) * b->surv_cap);
    if (ce != cudaSuccess) { es_batch_destroy(b); return cuda_fail(ce, "batch setup"); }
    b->d_unit = b->d_surv_n + 1;
    b->d_found = b->d_surv_n + 1 + kMaxSubs;
    b->d_min = b->d_found + b->n_groups;
    b->d_item_next = b->d_min + 4ull * b->n_groups;
    b->n_items = n_items;
    for (uint32_t i = 0; i < n_items; ++i) {
        EsItem& it = b->h_items[i];
        it.tconst = b->d_tconst + (uintptr_t)it.tconst;
        it.counts = tune.count_stages ? b->d_counts + b->count_off[i] : nullptr;
    }
    // the launches, one per width class, each over its own unit space
    std::vector<EsItem> launch_items(n_items);
    uint32_t pos = 0;
    while (pos < n_items) {
        const uint32_t cls = width_class(ctxs[items[order[pos]].ctx_index]->h_inst.W);
        uint32_t end = pos;
        uint32_t small_max = 0, nf_max = 1, F = tune.mask_filters, first_ctx = items[order[pos]].ctx_index;
        bool one_ctx = true;
        uint32_t words = ctxs[first_ctx]->h_inst.W;
        uint64_t units = 0;
        while (end < n_items && keys[order[end]] == keys[order[pos]]) {
            const uint32_t ci = items[order[end]].ctx_index;
            const es_ctx* c = ctxs[ci];
            small_max = std::max<uint32_t>(small_max, c->h_inst.small_bytes);
            nf_max = std::max<uint32_t>(nf_max, c->h_inst.n_filters);
            F = std::min(F, stage_filters(tune.layout, tune.mask_filters, c->h_inst.n_filters, c->h_inst.F_built));
            if (ci != first_ctx) one_ctx = false;
            if (c->h_inst.W != words) words = 0;   // the generic instance reads each plan's width
            EsItem it = b->h_items[order[end]];
            it.unit_begin = units;
            units += it.n_units;
            launch_items[end] = it;
            ++end;
        }
        es_batch::Sub sub;
        sub.words = cls == 0 ? 0u : (cls == 4 && words == 0 ? 4u : (words ? words : cls));
        uint32_t mask_words = 0;   // the largest inner-stage word-mask tables among the class's plans
        for (uint32_t j = pos; j < end; ++j)
            mask_words = std::max<uint32_t>(mask_words, ctxs[items[order[j]].ctx_index]->h_inst.mask_off[F]);
        sub.layout = launch_layout(tune.layout, sub.words, small_max, nf_max, tune, mask_words);
        const SmemPlan sp = plan_smem(small_max, nf_max, tune, staged_words(sub.layout, mask_words));
        EsLaunch& L = sub.L;
        memset(&L, 0, sizeof(L));
        L.items = b->d_items_launch + pos;
        L.n_items = end - pos;
        L.threads = tune.threads;
        L.strip = tune.strip;
        L.mask_filters = F;
        L.total_units = units;
        L.nf_max = nf_max;
        L.direct = one_ctx ? 1u : 0u;
        L.unit_counter = b->d_unit + b->subs.size();
        L.item_next = b->d_item_next + pos;
        L.surv = b->d_surv;
        L.surv_n = b->d_surv_n;
        L.surv_cap = b->surv_cap;
        L.group_found = b->d_found;
        L.smem_bytes = sp.bytes;
        L.cnt_off = sp.cnt_off;
        L.queue_off = sp.queue_off;
        L.stage_off = sp.stage_off;
        if (int e = grid_for(sub.layout, tune.count_stages, sub.words, F, tune, sp.bytes,
                             std::max<uint64_t>(units, 1), &sub.grid)) {
            es_batch_destroy(b);
            return e;
        }
        b->subs.push_back(sub);
        pos = end;
    }
    ce = cudaMemcpy(b->d_items, b->h_items.data(), sizeof(EsItem) * n_items, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess)
        ce = cudaMemcpy(b->d_items_launch, launch_items.data(), sizeof(EsItem) * n_items, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess && !h_tc.empty())
        ce = cudaMemcpy(b->d_tconst, h_tc.data(), 4ull * h_tc.size(), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) { es_batch_destroy(b); return cuda_fail(ce, "batch upload"); }
    *out = b;
    return ES_OK;
}

static int batch_enqueue(es_batch* b) {
    ES_CUDA(cudaMemsetAsync(b->d_surv_n, 0, 8ull * (1 + kMaxSubs), b->stream), "memset");   // count + unit counters
    ES_CUDA(cudaMemsetAsync(b->d_found, 0xff, 8ull * b->n_groups, b->stream), "memset");
    ES_CUDA(cudaMemsetAsync(b->d_item_next, 0, 8ull * b->n_items, b->stream), "memset");
    if (b->counts_words)
        ES_CUDA(cudaMemsetAsync(b->d_counts, 0, 8ull * b->counts_words, b->stream), "memset");
    for (const es_batch::Sub& sub : b->subs) {
        if (!sub.L.total_units) continue;
        int e = es_launch_scan(sub.L, (int)sub.layout, (int)b->tune.count_stages, sub.words, sub.grid, b->stream);
        if (e) return cuda_fail((cudaError_t)e, "scan launch");
    }
    // survivors carry the caller's item index: the min-reduction reads the items in that order
    int e = es_launch_min(b->d_surv, b->d_surv_n, b->surv_cap, b->d_items, b->n_groups, b->d_found,
                          b->d_min, b->stream);
    if (e) return cuda_fail((cudaError_t)e, "min launch");
    return ES_OK;
}

int es_batch_run(es_batch* b, int use_graph) {
    if (!b) return fail(ES_ERR_ARG, "null batch");
    ES_CUDA(cudaEventRecord(b->ev0, b->stream), "event");
    if (use_graph) {
        if (!b->exec) {
            ES_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "capture");
            int e = batch_enqueue(b);
            cudaGraph_t g = nullptr;
            cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
            if (e) { if (g) cudaGraphDestroy(g); return e; }
            if (ce != cudaSuccess) return cuda_fail(ce, "end capture");
            b->graph = g;
            ES_CUDA(cudaGraphInstantiate(&b->exec, g, 0), "graph instantiate");
        }
        ES_CUDA(cudaGraphLaunch(b->exec, b->stream), "graph launch");
    } else {
        if (int e = batch_enqueue(b)) return e;
    }
    ES_CUDA(cudaEventRecord(b->ev1, b->stream), "event");
    b->ran = true;
    return ES_OK;
}

int es_batch_sync(es_batch* b, float* ms) {
    if (!b) return fail(ES_ERR_ARG, "null batch");
    ES_CUDA(cudaStreamSynchronize(b->stream), "kernel execution");
    if (ms) {
        float v = 0.f;
        if (b->ran) ES_CUDA(cudaEventElapsedTime(&v, b->ev0, b->ev1), "event");
        *ms = v;
    }
    return ES_OK;
}

int es_batch_group_min(es_batch* b, uint32_t group, int* found, uint64_t* t, uint64_t* s_lo,
                       uint64_t* s_hi) {
    if (!b || !found) return fail(ES_ERR_ARG, "null argument");
    if (group >= b->n_groups) return fail(ES_ERR_ARG, "group out of range");
    if (!b->ran) return fail(ES_ERR_STATE, "batch has not run");
    ES_CUDA(cudaStreamSynchronize(b->stream), "kernel execution");
    unsigned long long v[4];
    ES_CUDA(cudaMemcpy(v, b->d_min + 4ull * group, 32, cudaMemcpyDeviceToHost), "copy");
    *found = (int)v[0];
    if (t) *t = v[1];
    if (s_lo) *s_lo = v[2];
    if (s_hi) *s_hi = v[3];
    if (v[0] == 2)   // records were dropped: the minimum over the stored ones is not reliable
        return fail(ES_ERR_OVERFLOW, "survivor buffer overflow in the batch; the least block of this "
                                     "group holding a good survivor is t = " +
                                     (v[1] == ~0ull ? std::string("none") : std::to_string(v[1])) +
                                     "; rescan the group's blocks one at a time");
    return ES_OK;
}

int es_batch_item_counts(es_batch* b, uint32_t item, uint64_t* counts, uint32_t n) {
    if (!b || (n && !counts)) return fail(ES_ERR_ARG, "null argument");
    if (item >= b->h_items.size()) return fail(ES_ERR_ARG, "item out of range");
    const uint32_t nf = b->ctxs[b->h_items[item].inst_id]->h_inst.n_filters;
    if (n != nf) return fail(ES_ERR_ARG, "counts length must equal the item's filter count");
    if (!b->ran) return fail(ES_ERR_STATE, "batch has not run");
    ES_CUDA(cudaStreamSynchronize(b->stream), "kernel execution");
    if (n) ES_CUDA(cudaMemcpy(counts, b->d_counts + b->count_off[item], 8ull * n, cudaMemcpyDeviceToHost), "copy");
    return ES_OK;
}

int es_batch_survivors(es_batch* b, es_survivor* out, uint64_t cap, uint64_t* n) {
    if (!b || !n) return fail(ES_ERR_ARG, "null argument");
    if (!b->ran) return fail(ES_ERR_STATE, "batch has not run");
    ES_CUDA(cudaStreamSynchronize(b->stream), "kernel execution");
    unsigned long long cnt = 0;
    ES_CUDA(cudaMemcpy(&cnt, b->d_surv_n, 8, cudaMemcpyDeviceToHost), "copy");
    *n = cnt;
    if (cnt > b->surv_cap) return fail(ES_ERR_OVERFLOW, "survivor buffer overflow");
    if (cnt > cap) return fail(ES_ERR_OVERFLOW, "output buffer smaller than the survivor count");
    if (cnt) ES_CUDA(cudaMemcpy(out, b->d_surv, sizeof(es_survivor) * cnt, cudaMemcpyDeviceToHost), "copy");
    return ES_OK;
}

static int int_peak_probe(int mix, double* ops_per_s, double* ms_out) {
    if (int e = device_facts()) return e;
    unsigned long long* sink = nullptr;
    ES_CUDA(cudaMalloc(&sink, 8), "cudaMalloc");
    cudaEvent_t a, z;
    cudaEventCreate(&a);
    cudaEventCreate(&z);
    const int threads = 256, grid = g_dev.sms * 8, iters = 4096;
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(a);
        int e = es_launch_int_peak(sink, grid, threads, iters, mix, nullptr);
        cudaEventRecord(z);
        cudaError_t ce = cudaEventSynchronize(z);
        if (e || ce != cudaSuccess) {
            cudaFree(sink);
            cudaEventDestroy(a);
            cudaEventDestroy(z);
            return cuda_fail(e ? (cudaError_t)e : ce, "int peak kernel");
        }
        float v = 0.f;
        cudaEventElapsedTime(&v, a, z);
        if (rep > 0 && v < best) best = v;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(z);
    cudaFree(sink);
    const double ops = (double)grid * threads * (double)iters * 256.0;
    if (ops_per_s) *ops_per_s = ops / (best * 1e-3);
    if (ms_out) *ms_out = best;
    return ES_OK;
}

int es_int_peak(double* ops_per_s, double* ms_out) { return int_peak_probe(0, ops_per_s, ms_out); }

int es_int_peak_mixed(double* ops_per_s, double* ms_out) { return int_peak_probe(1, ops_per_s, ms_out); }

}  // extern "C"

// ------------------------------------------------------------------------------------------
// es_search_blocks_static: the one entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc at all: code running under an external memory manager
// (a framework that owns every device allocation, a pool with a hard budget), or a service
// that must not allocate after start-up.  For them this is a variant of the block-ordered
// multi-block search launch: blocks t0 .. t0+n_blocks-1 of an existing context, scanned in
// one persistent launch, the first block holding a good survivor ending the search.  The
// caller passes the inputs (the context's plan tables, built earlier) and the outputs (a
// survivor buffer, its count and the 4-word minimum).  The launch's scratch -- work counter,
// search flag, per-block item descriptors and block constants -- lives in the file-scope
// array below, of fixed size ES_STATIC_MAX_BLOCKS blocks x ES_MAX_FILTERS filters (about
// 57 KB); every GPU that loads this library keeps it until the process exits.
namespace {

constexpr size_t kStaticItemsOff = 256;
constexpr size_t kStaticTconstOff = kStaticItemsOff + sizeof(EsItem) * ES_STATIC_MAX_BLOCKS;
constexpr size_t kStaticBytes = kStaticTconstOff + 4ull * ES_STATIC_MAX_BLOCKS * ES_MAX_FILTERS;

// [0,8) work counter, [8,16) least block with a good survivor, items, per-block constants
static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

// Host side: the device address of g_static_scratch per device (the host symbol itself is
// only a stand-in and must never be passed to a kernel), and a host staging area for the
// descriptors (static storage: no heap allocation on the call path).
constexpr int kMaxDevices = 64;
unsigned char* g_static_ptr[kMaxDevices] = {nullptr};
EsItem g_static_items[ES_STATIC_MAX_BLOCKS];
uint32_t g_static_tconst[ES_STATIC_MAX_BLOCKS * ES_MAX_FILTERS];
std::mutex g_static_mu;

}  // namespace

extern "C" int es_search_blocks_static(const es_ctx* c, uint64_t t0, uint32_t n_blocks,
                                       es_survivor* d_out, uint64_t out_cap,
                                       unsigned long long* d_count, unsigned long long* d_min,
                                       void* stream) {
    if (!c || !d_out || !d_count || !d_min || out_cap == 0)
        return fail(ES_ERR_ARG, "null context/output or zero output capacity");
    if (n_blocks == 0 || n_blocks > ES_STATIC_MAX_BLOCKS)
        return fail(ES_ERR_RANGE, "n_blocks must be in [1, " + std::to_string(ES_STATIC_MAX_BLOCKS) +
                                      "] for the static-scratch search");
    if (t0 > UINT64_MAX - n_blocks) return fail(ES_ERR_RANGE, "block range overflows");
    const EsInst& I = c->h_inst;
    if (I.n_filters > ES_MAX_FILTERS) return fail(ES_ERR_RANGE, "too many filters");
    cudaStream_t st = (cudaStream_t)stream;
    // The descriptors below are copied from host staging arrays that the next call overwrites; a
    // captured copy would read them only when the graph runs, so capture is refused.
    cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
    ES_CUDA(cudaStreamIsCapturing(st, &cap_status), "cudaStreamIsCapturing");
    if (cap_status != cudaStreamCaptureStatusNone)
        return fail(ES_ERR_STATE, "es_search_blocks_static cannot be called while its stream is capturing");
    int dev = 0;
    ES_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(ES_ERR_RANGE, "device index out of range");
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[dev]) {
        // once per device, with that device current: the scratch array's device address
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
        g_static_ptr[dev] = static_cast<unsigned char*>(p);
    }
    unsigned char* base = g_static_ptr[dev];
    unsigned long long* d_unit = reinterpret_cast<unsigned long long*>(base);
    unsigned long long* d_found = d_unit + 1;
    EsItem* d_items = reinterpret_cast<EsItem*>(base + kStaticItemsOff);
    uint32_t* d_tc = reinterpret_cast<uint32_t*>(base + kStaticTconstOff);

    const es_tune& tn = c->tune;
    const uint32_t nf = I.n_filters;
    const uint32_t F = stage_filters(tn.layout, tn.mask_filters, nf, I.F_built);
    es_tune tn0 = tn;
    tn0.count_stages = 0;   // the static search never counts
    const uint32_t layout = launch_layout(tn.layout, I.W, I.small_bytes, nf, tn0, I.mask_off[F]);
    const SmemPlan sp = plan_smem((uint32_t)I.small_bytes, nf, tn0, staged_words(layout, I.mask_off[F]));
    uint64_t cbeg = 0;
    const uint64_t ncyc = cycles_of(I, 0, I.n_outer, &cbeg);
    const uint64_t nu = units_of(I, cbeg, cbeg + ncyc, tn.strip);
    for (uint32_t i = 0; i < n_blocks; ++i) {
        const uint64_t t = t0 + i;
        EsItem& it = g_static_items[i];
        memset(&it, 0, sizeof(it));
        it.inst = c->d_inst;
        it.tconst = d_tc + (size_t)i * ES_MAX_FILTERS;
        it.t = t;
        it.o_begin = 0;
        it.o_end = I.n_outer;
        it.c_begin = cbeg;
        it.c_end = cbeg + ncyc;
        it.unit_begin = nu * i;
        it.n_units = nu;
        it.caller = i;
        for (uint32_t f = 0; f < nf; ++f) {
            const uint64_t q = c->q[f];
            g_static_tconst[(size_t)i * ES_MAX_FILTERS + f] = (uint32_t)((t % q) * (uint64_t)(c->M % q) % q);
        }
    }
    ES_CUDA(cudaMemcpyAsync(d_items, g_static_items, sizeof(EsItem) * n_blocks, cudaMemcpyHostToDevice, st),
            "copy items");
    ES_CUDA(cudaMemcpyAsync(d_tc, g_static_tconst, 4ull * ES_MAX_FILTERS * n_blocks, cudaMemcpyHostToDevice, st),
            "copy block constants");
    ES_CUDA(cudaMemsetAsync(d_unit, 0, 8, st), "memset");
    ES_CUDA(cudaMemsetAsync(d_found, 0xff, 8, st), "memset");
    ES_CUDA(cudaMemsetAsync(d_count, 0, 8, st), "memset");

    EsLaunch L;
    memset(&L, 0, sizeof(L));
    L.items = d_items;
    L.n_items = n_blocks;
    L.threads = tn.threads;
    L.strip = tn.strip;
    L.mask_filters = F;
    L.total_units = nu * n_blocks;
    L.nf_max = std::max<uint32_t>(nf, 1);
    L.direct = 1;
    L.unit_counter = d_unit;
    L.surv = d_out;
    L.surv_n = d_count;
    L.surv_cap = out_cap;
    L.group_found = d_found;
    L.smem_bytes = sp.bytes;
    L.cnt_off = sp.cnt_off;
    L.queue_off = sp.queue_off;
    L.stage_off = sp.stage_off;
    if (L.total_units) {
        int grid = 0;
        if (int e = grid_for(layout, 0, I.W, F, tn, sp.bytes, L.total_units, &grid)) return e;
        int e = es_launch_scan(L, (int)layout, 0, I.W, grid, st);
        if (e) return cuda_fail((cudaError_t)e, "scan launch");
    }
    int e = es_launch_min(d_out, d_count, out_cap, d_items, 1, d_found, d_min, st);
    if (e) return cuda_fail((cudaError_t)e, "min launch");
    return ES_OK;
}

/*
 * es_oracle.c -- TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline, never
 * part of the product path).  Plain C restatement of the reference project's CPU path for
 * the CRT-wheel sieve, multi-threaded with pthreads for speed:
 *
 *   for every position idx = oidx * r0 + d0 of the requested outer indices (block t):
 *     digits  d_j of idx in mixed radix, ring 0 fastest        (sieve/gpu_sieve_v9.py:385-390)
 *     s       = (sum_j term_j[d_j]) mod M, term_j[d] = res_j[d] * basis_j mod M
 *                                                              (sieve/gpu_sieve_v9.py:433-437)
 *     n       = t*M + s
 *     filter j passes iff n mod q_j is an admissible residue of p_j, i.e. every base-p digit
 *             of k is <= the matching digit of n              (ref/erdos_ref.py:40-48, 69-81)
 *     the cascade stops at the first failing filter; counts[j] += 1 for each filter passed
 *             (order-dependent; the reference emulation is tests/test_enumeration.py:51-68)
 *   survivors (all filters passed) are reported as idx; n <= k+1 is NOT excluded here, exactly
 *   like the reference kernel (sieve/gpu_sieve_v9.py:323-326) -- the host drops those.
 *
 * Deliberately independent of the engine's design: every position is rebuilt from scratch
 * from its digits (no incremental residues, no sorted inner ring, no carry split, no word
 * masks) and every residue is an exact 128-bit remainder.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

typedef struct {
    uint32_t n_rings;
    const uint32_t* radix;
    const uint32_t* ring_off;
    const u128* terms;
    u128 M;
    uint32_t n_filters;
    const uint32_t* q;
    const uint32_t* tq;           /* (t mod q_j)(M mod q_j) mod q_j */
    const uint8_t* allowed;       /* byte tables, q_j bytes each */
    const uint32_t* tab_off;
    const uint64_t* list;         /* outer indices or NULL */
    uint64_t o_begin, o_end;      /* outer range, or index range into list */
    uint32_t r0;
    /* per-thread outputs */
    uint64_t* counts;
    uint64_t* surv;
    uint64_t surv_cap, n_surv;
} job_t;

static void scan_outer(job_t* J, uint64_t oidx) {
    for (uint32_t d0 = 0; d0 < J->r0; ++d0) {
        const uint64_t idx = oidx * J->r0 + d0;
        uint64_t rem = idx;
        u128 s = 0;
        for (uint32_t j = 0; j < J->n_rings; ++j) {
            const uint64_t d = rem % J->radix[j];
            rem /= J->radix[j];
            s += J->terms[J->ring_off[j] + d];
            if (s >= J->M) s -= J->M;
        }
        uint32_t f = 0;
        for (; f < J->n_filters; ++f) {
            const uint32_t q = J->q[f];
            const uint32_t r = (uint32_t)((s % q + J->tq[f]) % q);
            if (!J->allowed[J->tab_off[f] + r]) break;
            J->counts[f] += 1;
        }
        if (f == J->n_filters) {
            if (J->n_surv < J->surv_cap) J->surv[J->n_surv] = idx;
            J->n_surv += 1;
        }
    }
}

static void* worker(void* arg) {
    job_t* J = (job_t*)arg;
    for (uint64_t i = J->o_begin; i < J->o_end; ++i) scan_outer(J, J->list ? J->list[i] : i);
    return NULL;
}

/*
 * Scan outer indices [o_begin, o_end) (or list[o_begin..o_end) when list != NULL) of block t.
 * terms: 2 * sum(radix) uint64 (lo, hi pairs).  allowed: concatenated byte tables (q_j bytes).
 * counts: n_filters outputs.  surv: up to surv_cap indices (unsorted); *n_surv = total found.
 * Returns 0, or -1 on bad arguments / allocation failure.
 */
int es_oracle_scan(uint32_t n_rings, const uint32_t* radix, const uint64_t* terms_lohi,
                   uint64_t M_lo, uint64_t M_hi, uint32_t n_filters, const uint32_t* q,
                   const uint8_t* allowed, uint64_t t, const uint64_t* list, uint64_t o_begin,
                   uint64_t o_end, int n_threads, uint64_t* counts, uint64_t* surv,
                   uint64_t surv_cap, uint64_t* n_surv) {
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 256) n_threads = 256;
    const u128 M = ((u128)M_hi << 64) | M_lo;
    if (M == 0 || o_begin > o_end) return -1;
    uint64_t nterms = 0;
    uint32_t* ring_off = (uint32_t*)calloc(n_rings + 1, sizeof(uint32_t));
    for (uint32_t j = 0; j < n_rings; ++j) { ring_off[j] = (uint32_t)nterms; nterms += radix[j]; }
    u128* terms = (u128*)malloc(sizeof(u128) * (nterms + 1));
    for (uint64_t i = 0; i < nterms; ++i)
        terms[i] = ((u128)terms_lohi[2 * i + 1] << 64) | terms_lohi[2 * i];
    uint32_t* tab_off = (uint32_t*)calloc(n_filters + 1, sizeof(uint32_t));
    uint32_t* tq = (uint32_t*)calloc(n_filters + 1, sizeof(uint32_t));
    for (uint32_t f = 0; f < n_filters; ++f) {
        tab_off[f + 1] = tab_off[f] + q[f];
        tq[f] = (uint32_t)(((u128)(t % q[f]) * (uint64_t)(M % q[f])) % q[f]);
    }
    const uint32_t r0 = n_rings ? radix[0] : 1;
    static const uint32_t one = 1;
    static const u128 zero = 0;
    job_t* jobs = (job_t*)calloc((size_t)n_threads, sizeof(job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
    const uint64_t n = o_end - o_begin;
    for (int i = 0; i < n_threads; ++i) {
        job_t* J = &jobs[i];
        J->n_rings = n_rings ? n_rings : 1;
        J->radix = n_rings ? radix : &one;
        J->ring_off = ring_off;
        J->terms = n_rings ? terms : &zero;
        J->M = M;
        J->n_filters = n_filters;
        J->q = q;
        J->tq = tq;
        J->allowed = allowed;
        J->tab_off = tab_off;
        J->list = list;
        J->o_begin = o_begin + n * (uint64_t)i / (uint64_t)n_threads;
        J->o_end = o_begin + n * (uint64_t)(i + 1) / (uint64_t)n_threads;
        J->r0 = r0;
        J->counts = (uint64_t*)calloc(n_filters + 1, sizeof(uint64_t));
        J->surv_cap = surv_cap;
        J->surv = (uint64_t*)malloc(sizeof(uint64_t) * (surv_cap + 1));
        pthread_create(&th[i], NULL, worker, J);
    }
    uint64_t tot = 0;
    memset(counts, 0, sizeof(uint64_t) * n_filters);
    for (int i = 0; i < n_threads; ++i) {
        pthread_join(th[i], NULL);
        for (uint32_t f = 0; f < n_filters; ++f) counts[f] += jobs[i].counts[f];
        for (uint64_t s = 0; s < jobs[i].n_surv && s < jobs[i].surv_cap; ++s)
            if (tot + s < surv_cap) surv[tot + s] = jobs[i].surv[s];
        tot += jobs[i].n_surv;
        free(jobs[i].counts);
        free(jobs[i].surv);
    }
    *n_surv = tot;
    free(jobs); free(th); free(terms); free(ring_off); free(tab_off); free(tq);
    return 0;
}

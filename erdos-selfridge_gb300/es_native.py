"""ctypes binding of libes_gb300.so (include/es_gb300.h) plus plan -> descriptor flattening.

The shared library is the only compute path: importing this module fails loudly when the
library is missing, and every call that returns a negative code raises ``EsError`` with the
library's message.  Build the library with ``python erdos-selfridge_gb300/build.py`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("ES_GB300_LIB") or os.path.join(HERE, "libes_gb300.so")

ES_OK = 0
ES_ERR_OVERFLOW = -3
LAYOUT_WORDMASK = 0
LAYOUT_SCALAR = 1
LAYOUT_PAIR = 2       # word masks with the wrapped row beside each phase (inner rings <= 64 slots)
LAYOUT_SMEM = 3       # word masks of the inner-stage filters staged in shared memory (<= 64 slots)
LAYOUT_SMEM_PAIR = 4  # pair tables of the inner-stage filters staged in shared memory (<= 64 slots)
LAYOUT_AUTO = 5       # chosen per launch (per width class in a batch) by the library
MAX_MASK_FILTERS = 8


class EsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"es_gb300 error {code}: {msg}")
        self.code = code


class PlanDesc(C.Structure):
    _fields_ = [("k", C.c_uint32), ("n_rings", C.c_uint32), ("n_filters", C.c_uint32),
                ("flags", C.c_uint32), ("M_lo", C.c_uint64), ("M_hi", C.c_uint64),
                ("radix", C.POINTER(C.c_uint32)), ("term_lo", C.POINTER(C.c_uint64)),
                ("term_hi", C.POINTER(C.c_uint64)), ("filter_q", C.POINTER(C.c_uint32)),
                ("allowed", C.POINTER(C.c_uint32))]


class Tune(C.Structure):
    _fields_ = [("layout", C.c_uint32), ("mask_filters", C.c_uint32), ("threads", C.c_uint32),
                ("strip", C.c_uint32), ("smem_kb", C.c_uint32), ("ctas_per_sm", C.c_uint32),
                ("count_stages", C.c_uint32), ("reserved", C.c_uint32)]


class Survivor(C.Structure):
    _fields_ = [("idx", C.c_uint64), ("s_lo", C.c_uint64), ("s_hi", C.c_uint64),
                ("t", C.c_uint64), ("item", C.c_uint32), ("good", C.c_uint32)]


class BatchItem(C.Structure):
    _fields_ = [("ctx_index", C.c_uint32), ("group", C.c_uint32), ("t", C.c_uint64),
                ("o_begin", C.c_uint64), ("o_end", C.c_uint64)]


SURVIVOR_DTYPE = np.dtype([("idx", "<u8"), ("s_lo", "<u8"), ("s_hi", "<u8"), ("t", "<u8"),
                           ("item", "<u4"), ("good", "<u4")])
assert SURVIVOR_DTYPE.itemsize == C.sizeof(Survivor)

_lib = None


def lib() -> C.CDLL:
    """Load (once) the sm_103a engine library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with erdos-selfridge_gb300/build.py "
                           "(the engine has no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    P, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
    pu64, pu32 = C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)
    sig = {
        "es_last_error": ([], C.c_char_p),
        "es_abi_version": ([], i32),
        "es_device_info": ([C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), pu64], i32),
        "es_device_name": ([C.c_char_p, u32], i32),
        "es_ctx_create": ([C.POINTER(PlanDesc), C.POINTER(Tune), C.POINTER(P)], i32),
        "es_ctx_destroy": ([P], i32),
        "es_ctx_set_tune": ([P, C.POINTER(Tune)], i32),
        "es_ctx_get_tune": ([P, C.POINTER(Tune)], i32),
        "es_ctx_info": ([P, pu64, pu32, pu32, pu64], i32),
        "es_set_capacity": ([P, u64], i32),
        "es_set_block": ([P, pu32, u32, u64], i32),
        "es_reset_survivors": ([P], i32),
        "es_launch": ([P, u64, u64], i32),
        "es_launch_list": ([P, pu64, u64], i32),
        "es_sync": ([P], i32),
        "es_survivor_count": ([P, pu64], i32),
        "es_read_survivors": ([P, pu64, u64, pu64], i32),
        "es_read_survivor_records": ([P, C.POINTER(Survivor), u64, pu64], i32),
        "es_stage_counts": ([P, pu64, u32], i32),
        "es_reset_counts": ([P], i32),
        "es_min_survivor": ([P, C.POINTER(i32), pu64, pu64, pu64], i32),
        "es_launch_timed": ([P, u64, u64, C.POINTER(C.c_float)], i32),
        "es_batch_create": ([C.POINTER(P), u32, C.POINTER(BatchItem), u32, C.POINTER(Tune),
                             C.POINTER(P)], i32),
        "es_batch_run": ([P, i32], i32),
        "es_batch_sync": ([P, C.POINTER(C.c_float)], i32),
        "es_batch_group_min": ([P, u32, C.POINTER(i32), pu64, pu64, pu64], i32),
        "es_batch_item_counts": ([P, u32, pu64, u32], i32),
        "es_batch_survivors": ([P, C.POINTER(Survivor), u64, pu64], i32),
        "es_batch_destroy": ([P], i32),
        "es_int_peak": ([C.POINTER(C.c_double), C.POINTER(C.c_double)], i32),
        "es_int_peak_mixed": ([C.POINTER(C.c_double), C.POINTER(C.c_double)], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def check(code: int) -> int:
    if code < 0:
        raise EsError(code, lib().es_last_error().decode(errors="replace"))
    return code


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def bit_table(q: int, residues) -> np.ndarray:
    """Packed admissible-residue bits: word r>>5, bit r&31 (sieve/gpu_sieve_v11.py layout)."""
    w = np.zeros((q + 31) // 32, dtype=np.uint32)
    r = np.asarray(residues, dtype=np.int64)
    np.bitwise_or.at(w, r >> 5, (np.uint32(1) << (r & 31).astype(np.uint32)))
    return w


class PlanArrays:
    """Flattened plan: ring terms (res * basis_j mod M), filter moduli and bit tables."""

    @classmethod
    def from_arrays(cls, k, radix, term_lo, term_hi, q, allowed, M) -> "PlanArrays":
        """Rebuild from arrays produced elsewhere (e.g. a worker process)."""
        self = object.__new__(cls)
        mask64 = (1 << 64) - 1
        self.radix, self.term_lo, self.term_hi = _u32(radix), _u64(term_lo), _u64(term_hi)
        self.q, self.allowed = _u32(q), _u32(allowed)
        n_rings = 0 if (self.radix.size == 1 and int(self.radix[0]) == 0) else self.radix.size
        n_filters = 0 if (self.q.size == 1 and int(self.q[0]) == 0) else self.q.size
        self.desc = PlanDesc(k=int(k), n_rings=n_rings, n_filters=n_filters, flags=0,
                             M_lo=int(M) & mask64, M_hi=int(M) >> 64,
                             radix=_ptr(self.radix, C.c_uint32), term_lo=_ptr(self.term_lo, C.c_uint64),
                             term_hi=_ptr(self.term_hi, C.c_uint64), filter_q=_ptr(self.q, C.c_uint32),
                             allowed=_ptr(self.allowed, C.c_uint32))
        return self

    def __init__(self, plan):
        M = plan.M
        terms = []
        for j, (q, res) in enumerate(plan.rings):
            b = plan.basis[j]
            terms.extend((a * b) % M for a in res)
        mask64 = (1 << 64) - 1
        self.radix = _u32(plan.radix if plan.radix else [0])
        self.term_lo = _u64([x & mask64 for x in terms] or [0])
        self.term_hi = _u64([x >> 64 for x in terms] or [0])
        self.q = _u32([plan.info[p][0] for p in plan.rest] or [0])
        tabs = [bit_table(plan.info[p][0], plan.info[p][1]) for p in plan.rest]
        self.allowed = _u32(np.concatenate(tabs) if tabs else [0])
        self.desc = PlanDesc(k=plan.k, n_rings=len(plan.radix), n_filters=len(plan.rest), flags=0,
                             M_lo=M & mask64, M_hi=M >> 64,
                             radix=_ptr(self.radix, C.c_uint32), term_lo=_ptr(self.term_lo, C.c_uint64),
                             term_hi=_ptr(self.term_hi, C.c_uint64), filter_q=_ptr(self.q, C.c_uint32),
                             allowed=_ptr(self.allowed, C.c_uint32))


# L1 bytes the phase tables can count on beside the scan's ~51 KB of shared memory (each SM has
# 256 KB for L1 and shared memory together; the CUDA driver's carveout for the scan is 64 KB)
L1_TABLE_BUDGET = 180 * 1024
# Shared-memory bytes the inner-stage phase tables can take: a CTA may opt in to 227 KB, of which
# the scan's small tables and per-warp queues take about 55 KB at 512 threads (the library checks
# the exact figure per launch and falls back to the word-mask layout when the tables do not fit)
SMEM_TABLE_BUDGET = 171 * 1024


def layout_for(r0: int, filter_q, mask_filters: int) -> int:
    """Table layout of the inner-ring stage for an inner ring of r0 slots whose first filters have
    moduli filter_q.  Word-mask tables that fit in shared memory are staged there (a random
    4- or 8-byte gather from shared memory costs a few bank wavefronts instead of one L1 sector
    per lane: 1.17x at k = 300).  Otherwise pair tables cost one load per filter and word instead
    of two, but twice the bytes: they win unless the word-mask tables fit L1 and the pair tables
    do not (k = 390 gains about 1.3x from pairs).  Neither choice changes which candidates pass.
    The library applies the same rule per launch to LAYOUT_AUTO (launch_layout in
    csrc/es_abi.cu), with the exact shared-memory figure of the launch."""
    W = -(-max(1, int(r0)) // 32)
    if W > 2:
        return LAYOUT_WORDMASK
    qs = [int(q) for q in list(filter_q)[:min(int(mask_filters), MAX_MASK_FILTERS)]]
    single = 4 * sum(-(-(q * W) // 4) * 4 for q in qs)
    if single <= SMEM_TABLE_BUDGET:
        return LAYOUT_SMEM
    if single <= L1_TABLE_BUDGET < 2 * single:
        return LAYOUT_WORDMASK
    return LAYOUT_PAIR


def layout_for_plan(plan, mask_filters: int) -> int:
    return layout_for(plan.radix[0] if plan.radix else 1, [plan.info[p][0] for p in plan.rest], mask_filters)


def make_tune(layout=LAYOUT_WORDMASK, mask_filters=4, threads=512, strip=8, smem_kb=0,
              ctas_per_sm=4, count_stages=1) -> Tune:
    return Tune(layout=int(layout), mask_filters=int(mask_filters), threads=int(threads),
                strip=int(strip), smem_kb=int(smem_kb), ctas_per_sm=int(ctas_per_sm),
                count_stages=int(count_stages), reserved=0)


def tune_dict(t: Tune) -> dict:
    return {f: int(getattr(t, f)) for f, _ in Tune._fields_ if f != "reserved"}


def tconst_for(plan, t: int) -> np.ndarray:
    """tconst[j] = (t mod q_j)(M mod q_j) mod q_j (harness/run_k.py:102-104)."""
    out = np.zeros(max(1, len(plan.rest)), dtype=np.uint32)
    for j, p in enumerate(plan.rest):
        q = plan.info[p][0]
        out[j] = ((t % q) * (plan.M % q)) % q
    return out


class Context:
    """One plan resident on the device (es_ctx)."""

    def __init__(self, plan, tune: Tune | None = None, capacity: int | None = None, arrays=None):
        L = lib()
        self.plan = plan
        self.arrays = arrays if arrays is not None else PlanArrays(plan)
        self.tune = tune if tune is not None else make_tune()
        h = C.c_void_p()
        check(L.es_ctx_create(C.byref(self.arrays.desc), C.byref(self.tune), C.byref(h)))
        self.h = h
        n_outer, r0, nf, tb = C.c_uint64(), C.c_uint32(), C.c_uint32(), C.c_uint64()
        check(L.es_ctx_info(h, C.byref(n_outer), C.byref(r0), C.byref(nf), C.byref(tb)))
        self.n_outer, self.r0, self.n_filters, self.table_bytes = n_outer.value, r0.value, nf.value, tb.value
        self.capacity = 1 << 20
        if capacity is not None:
            self.set_capacity(capacity)
        self.t = 0

    @classmethod
    def from_arrays(cls, arrays: PlanArrays, tune: Tune | None = None, n_filters: int | None = None) -> "Context":
        """A context built from flattened arrays only (no Plan object; set_block needs tconst)."""
        return cls(None, tune, None, arrays)

    def close(self):
        if getattr(self, "h", None):
            lib().es_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tune(self, tune: Tune):
        check(lib().es_ctx_set_tune(self.h, C.byref(tune)))
        self.tune = tune

    def set_capacity(self, cap: int):
        check(lib().es_set_capacity(self.h, int(cap)))
        self.capacity = int(cap)

    def set_block(self, t: int, tconst: np.ndarray | None = None):
        tc = _u32(tconst_for(self.plan, t) if tconst is None else tconst)
        check(lib().es_set_block(self.h, _ptr(tc, C.c_uint32), self.n_filters, int(t) & ((1 << 64) - 1)))
        self.t = int(t)

    def reset(self):
        check(lib().es_reset_survivors(self.h))

    def reset_counts(self):
        check(lib().es_reset_counts(self.h))

    def launch(self, ostart: int, ocount: int):
        check(lib().es_launch(self.h, int(ostart), int(ocount)))

    def launch_list(self, outer):
        a = _u64(outer)
        check(lib().es_launch_list(self.h, _ptr(a, C.c_uint64), a.size))

    def launch_timed(self, ostart: int, ocount: int) -> float:
        ms = C.c_float()
        check(lib().es_launch_timed(self.h, int(ostart), int(ocount), C.byref(ms)))
        return ms.value

    def sync(self):
        check(lib().es_sync(self.h))

    def count(self) -> int:
        n = C.c_uint64()
        check(lib().es_survivor_count(self.h, C.byref(n)))
        return n.value

    def survivors(self, n: int | None = None) -> np.ndarray:
        """Survivor position indices.  With `n` (a count the caller already read) the first n of
        them, read without counting twice when there are no more than n."""
        if n is not None:
            out = np.zeros(max(n, 1), dtype=np.uint64)
            got = C.c_uint64()
            if lib().es_read_survivors(self.h, _ptr(out, C.c_uint64), out.size, C.byref(got)) == 0:
                return out[:min(got.value, n)]
            return self.survivors()[:n]   # more than n, or an overflow (raised there)
        n = self.count()
        out = np.zeros(max(n, 1), dtype=np.uint64)
        got = C.c_uint64()
        check(lib().es_read_survivors(self.h, _ptr(out, C.c_uint64), out.size, C.byref(got)))
        return out[:got.value]

    def records(self) -> np.ndarray:
        n = self.count()
        out = np.zeros(max(n, 1), dtype=SURVIVOR_DTYPE)
        got = C.c_uint64()
        check(lib().es_read_survivor_records(self.h, out.ctypes.data_as(C.POINTER(Survivor)),
                                             out.size, C.byref(got)))
        return out[:got.value]

    def stage_counts(self) -> np.ndarray:
        out = np.zeros(max(self.n_filters, 1), dtype=np.uint64)
        check(lib().es_stage_counts(self.h, _ptr(out, C.c_uint64), self.n_filters))
        return out[:self.n_filters]

    def min_survivor(self):
        """(t, s) of the least good survivor since the last reset, or None."""
        f, t, lo, hi = C.c_int(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(lib().es_min_survivor(self.h, C.byref(f), C.byref(t), C.byref(lo), C.byref(hi)))
        if not f.value:
            return None
        return t.value, (hi.value << 64) | lo.value


class Batch:
    """Persistent work-stealing launch over many (context, block, outer range) items."""

    def __init__(self, ctxs: list[Context], items: list[tuple], tune: Tune | None = None):
        L = lib()
        self.ctxs = ctxs
        arr = (C.c_void_p * len(ctxs))(*[c.h.value for c in ctxs])
        its = (BatchItem * len(items))()
        for i, (ci, group, t, ob, oe) in enumerate(items):
            its[i] = BatchItem(ctx_index=ci, group=group, t=t, o_begin=ob, o_end=oe)
        self.items = items
        self.tune = tune if tune is not None else ctxs[0].tune
        h = C.c_void_p()
        check(L.es_batch_create(arr, len(ctxs), its, len(items), C.byref(self.tune), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().es_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, use_graph: bool = True):
        check(lib().es_batch_run(self.h, 1 if use_graph else 0))

    def sync(self) -> float:
        ms = C.c_float()
        check(lib().es_batch_sync(self.h, C.byref(ms)))
        return ms.value

    def group_min(self, group: int):
        f, t, lo, hi = C.c_int(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(lib().es_batch_group_min(self.h, group, C.byref(f), C.byref(t), C.byref(lo), C.byref(hi)))
        return (t.value, (hi.value << 64) | lo.value) if f.value else None

    def item_counts(self, item: int) -> np.ndarray:
        nf = self.ctxs[self.items[item][0]].n_filters
        out = np.zeros(max(nf, 1), dtype=np.uint64)
        check(lib().es_batch_item_counts(self.h, item, _ptr(out, C.c_uint64), nf))
        return out[:nf]

    def survivors(self) -> np.ndarray:
        cap = self.ctxs[0].capacity
        out = np.zeros(cap, dtype=SURVIVOR_DTYPE)
        got = C.c_uint64()
        check(lib().es_batch_survivors(self.h, out.ctypes.data_as(C.POINTER(Survivor)), cap, C.byref(got)))
        return out[:got.value]


def int_peak(mixed: bool = False) -> tuple[float, float]:
    """(int32 ops/s, ms) of an integer microbenchmark on the current device: the ALU pipe alone
    (IADD3 + LOP3), or with ``mixed`` the ALU and FMA pipes together (LOP3 + IMAD)."""
    ops, ms = C.c_double(), C.c_double()
    fn = lib().es_int_peak_mixed if mixed else lib().es_int_peak
    check(fn(C.byref(ops), C.byref(ms)))
    return ops.value, ms.value


def device_info() -> dict:
    s, a, b, o = C.c_int(), C.c_int(), C.c_int(), C.c_uint64()
    check(lib().es_device_info(C.byref(s), C.byref(a), C.byref(b), C.byref(o)))
    name = C.create_string_buffer(256)
    check(lib().es_device_name(name, 256))
    return {"sm_count": s.value, "cc": (a.value, b.value), "smem_optin": o.value,
            "name": name.value.decode(errors="replace")}

"""CPU: the C-ABI library loads, exports every symbol include/es_gb300.h declares, rejects bad
input without a device, and the Python flattening of a plan matches the reference arrays."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "es_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(es_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    import es_native
    lib = C.CDLL(es_native.LIB_PATH)
    names = _declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert lib.es_abi_version() == 1


def test_binding_covers_the_header():
    """The Python bindings (es_native: engine; es_learned: MLP; es_mitm: meet-in-the-middle)
    cover every entry point except the one the no-allocation test binds itself."""
    import es_learned
    import es_mitm
    import es_native
    es_native.lib()
    src = open(es_native.__file__).read() + open(es_learned.__file__).read() + open(es_mitm.__file__).read()
    missing = [n for n in _declared() if n not in src and n != "es_search_blocks_static"]
    assert not missing, missing


def test_create_without_device_fails_loudly():
    """No GPU here: context creation must return an error code with a message, never crash."""
    import es_gb300
    import es_native as N
    try:
        N.device_info()
        pytest.skip("a device is present")
    except N.EsError:
        pass
    with pytest.raises(N.EsError) as e:
        N.Context(es_gb300.Plan(40))
    assert e.value.code < 0


def test_null_arguments_rejected():
    import es_native as N
    L = N.lib()
    assert L.es_ctx_create(None, None, None) == -1
    assert b"null" in L.es_last_error()
    assert L.es_launch(None, 0, 1) == -1
    assert L.es_batch_run(None, 1) == -1


def test_plan_arrays_match_reference_tables():
    import es_gb300
    import es_native as N
    for k in (40, 300):
        P = es_gb300.Plan(k)
        A = N.PlanArrays(P)
        terms = [(a * b) % P.M for (_, res), b in zip(P.rings, P.basis) for a in res]
        got = [(int(h) << 64) | int(l) for l, h in zip(A.term_lo, A.term_hi)]
        assert got == terms and all(t < P.M for t in terms)
        assert list(A.radix) == P.radix
        off = 0
        for p, q in zip(P.rest, A.q):
            res = P.info[p][1]
            w = A.allowed[off:off + (q + 31) // 32]
            bits = [r for r in range(q) if (int(w[r >> 5]) >> (r & 31)) & 1]
            assert bits == res
            off += (q + 31) // 32
        assert off == A.allowed.size
        assert A.desc.M_lo == P.M & ((1 << 64) - 1) and A.desc.M_hi == P.M >> 64


def test_tconst_matches_driver_formula():
    import es_gb300
    import es_native as N
    P = es_gb300.Plan(390)
    for t in (0, 1, 7, 2**33 + 5):
        tc = N.tconst_for(P, t)
        for j, p in enumerate(P.rest):
            q = P.info[p][0]
            assert tc[j] == ((t % q) * (P.M % q)) % q   # harness/run_k.py:102-104

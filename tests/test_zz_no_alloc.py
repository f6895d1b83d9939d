"""GPU test of es_search_blocks_static, the entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc: here the test plays that caller, holding
the output buffers itself (allocated through torch) and passing them in.  The result of two
calls in a row must equal the block-ordered search of the allocating batch path (es_batch_*)
on the same blocks: the same least good survivor, and the same survivor records for every
block up to and including the one that holds it (later blocks may be cut short by the early
exit in either path).  This file is collected last so that a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_BLOCKS = 64   # ES_STATIC_MAX_BLOCKS in include/es_gb300.h


def _entry(N):
    fn = N.lib().es_search_blocks_static
    fn.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p,
                   C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def _records(buf, n):
    import es_native as N
    raw = buf[: n * N.SURVIVOR_DTYPE.itemsize].cpu().numpy()
    return np.frombuffer(raw.tobytes(), dtype=N.SURVIVOR_DTYPE)


def _key(recs, t_max):
    return sorted((int(r["t"]), int(r["idx"]), int(r["s_lo"]), int(r["s_hi"]), int(r["good"]))
                  for r in recs if int(r["t"]) <= t_max)


@pytest.mark.parametrize("k,t0,nb,count_stages,layout", [(60, 0, 16, 0, 0), (97, 0, 8, 0, 0), (70, 3, 20, 0, 0),
                                                         (30, 0, 12, 0, 0), (57, 0, 10, 1, 0), (97, 0, 8, 0, 3),
                                                         (97, 0, 8, 0, 4), (300, 0, 2, 0, 5)])
def test_static_search_matches_batch(native, bfile, k, t0, nb, count_stages, layout):
    """Two calls in a row against the allocating batch path, and the least n against g(k) of the
    b-file (every block before g(k)'s holds no good survivor).  A context built for counting
    launches works too (the static search never counts), and so does one whose launches stage
    the phase tables in shared memory (word masks, layout 3, or pair tables, layout 4), and one whose
    layout the library picks per launch (layout 5; at k = 300 the staged word masks)."""
    import torch
    import es_gb300
    N = native
    fn = _entry(N)
    plan = es_gb300.Plan(k)
    ctx = N.Context(plan, N.make_tune(count_stages=count_stages, layout=layout))
    # reference result: the allocating batch path, one group over the same blocks
    b = N.Batch([ctx], [(0, 0, t0 + i, 0, ctx.n_outer) for i in range(nb)], ctx.tune)
    b.run(use_graph=False)
    b.sync()
    want_min = b.group_min(0)
    assert want_min is not None
    want = _key(b.survivors(), want_min[0])
    b.close()

    cap = 1 << 16
    rec_size = N.SURVIVOR_DTYPE.itemsize
    d_out = torch.zeros(cap * rec_size, dtype=torch.uint8, device="cuda")
    d_count = torch.zeros(1, dtype=torch.int64, device="cuda")
    d_min = torch.zeros(4, dtype=torch.int64, device="cuda")
    for _ in range(2):   # two calls in a row share the one scratch array
        rc = fn(ctx.h, t0, nb, d_out.data_ptr(), cap, d_count.data_ptr(), d_min.data_ptr(), None)
        assert rc == 0, N.lib().es_last_error().decode()
        torch.cuda.synchronize()
        n = int(d_count.item())
        assert 0 < n <= cap
        mn = [int(x) & ((1 << 64) - 1) for x in d_min.cpu().tolist()]
        assert mn[0] == 1
        got_min = (mn[1], (mn[3] << 64) | mn[2])
        assert got_min == want_min
        assert got_min[0] * plan.M + got_min[1] > k + 1
        assert _key(_records(d_out, n), got_min[0]) == want
        if t0 == 0:
            assert got_min[0] * plan.M + got_min[1] == bfile[k]


def test_static_search_overflow_is_flagged(native):
    """More survivors than the caller's buffer holds: the count still says how many there were,
    found = 2 flags the overflow, and d_min[1] is the least block holding a good survivor (the
    block of g(k), which the allocating path reports too)."""
    import torch
    import es_gb300
    N = native
    fn = _entry(N)
    k, nb = 30, 12                       # g(30) lies in block 9; blocks 0..9 hold 3 survivors
    plan = es_gb300.Plan(k)
    ctx = N.Context(plan, N.make_tune(count_stages=0))
    cap = 1
    d_out = torch.zeros(cap * N.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_count = torch.zeros(1, dtype=torch.int64, device="cuda")
    d_min = torch.zeros(4, dtype=torch.int64, device="cuda")
    rc = fn(ctx.h, 0, nb, d_out.data_ptr(), cap, d_count.data_ptr(), d_min.data_ptr(), None)
    assert rc == 0, N.lib().es_last_error().decode()
    torch.cuda.synchronize()
    assert int(d_count.item()) > cap
    mn = [int(x) & ((1 << 64) - 1) for x in d_min.cpu().tolist()]
    assert mn[0] == 2 and mn[1] == 9 and mn[2] == 0 and mn[3] == 0


def test_static_search_rejects_oversize(native):
    import torch
    import es_gb300
    N = native
    fn = _entry(N)
    ctx = N.Context(es_gb300.Plan(40), N.make_tune(count_stages=0))
    d_out = torch.zeros(1024 * N.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_count = torch.zeros(1, dtype=torch.int64, device="cuda")
    d_min = torch.zeros(4, dtype=torch.int64, device="cuda")
    rc = fn(ctx.h, 0, MAX_BLOCKS + 1, d_out.data_ptr(), 1024, d_count.data_ptr(), d_min.data_ptr(), None)
    assert rc == -4   # ES_ERR_RANGE
    assert b"n_blocks" in N.lib().es_last_error()


def test_static_search_refuses_stream_capture(native):
    """A call made while its stream is capturing a CUDA graph returns ES_ERR_STATE and enqueues
    nothing (its descriptor copies come from host staging arrays the next call reuses)."""
    import torch
    import es_gb300
    N = native
    fn = _entry(N)
    ctx = N.Context(es_gb300.Plan(40), N.make_tune(count_stages=0))
    d_out = torch.zeros(1024 * N.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_count = torch.zeros(1, dtype=torch.int64, device="cuda")
    d_min = torch.zeros(4, dtype=torch.int64, device="cuda")
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        rc = fn(ctx.h, 0, 4, d_out.data_ptr(), 1024, d_count.data_ptr(), d_min.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
        d_count.add_(0)   # something for the graph to hold
    assert rc == -6   # ES_ERR_STATE
    assert b"capturing" in N.lib().es_last_error()

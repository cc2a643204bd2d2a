"""Serving with continuous batching (g3l_server_*, g3l_submit/g3l_poll).

The contract: a request's results are the same whether it runs alone or while other
requests arrive, run and leave around it -- bit-identical here, since every
integral's trajectory depends only on its own regions -- and equal to g3l_eval's.
"""
import threading
import time

import numpy as np
import pytest

import g3lhalo_gb300 as G
from g3lhalo_gb300 import workloads as W
from g3lhalo_gb300.tables import make_tables

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    T = make_tables(Nz=64, Nm=128, Nk=256)
    c = G.Context(T, clamp_k=True)
    c.set_hod(0, W.hod_default())
    c.set_hod(1, W.hod_second())
    hods = W.hod_sweep(8, seed=12345)
    for k in range(4):
        c.set_hod(2 + k, hods[k])
    return c


def _request(tri, slot=0, kind=G.NNMAP, max_eval=100_000):
    trip = W.triplets_all()
    return [(kind, t, slot, slot, tuple(trip[i]), 1e-4, max_eval) for i in tri for t in (1, 2, 3)]


def _same(a, b):
    return (np.array_equal(a["val"], b["val"]) and np.array_equal(a["err"], b["err"])
            and np.array_equal(a["neval"], b["neval"]))


@pytest.mark.parametrize("precision", [G.MIXED, G.FP64])
def test_result_is_the_same_alone_and_in_the_mix(ctx, precision):
    A = _request(range(0, 220, 37), slot=0)
    ref = ctx.eval(A, precision)
    srv = G.Server(ctx, precision, max_items_per_term=256, pool_regions=1 << 21,
                   rounds_per_launch=2)
    try:
        alone, _ = srv.poll(srv.submit(A))
        assert _same(alone, ref)
        # A arrives while a larger request is already running; more arrive after it
        big = srv.submit(_request(range(1, 220, 5), slot=2, max_eval=300_000))
        while srv.info()["running_integrals"] == 0:
            time.sleep(0.001)
        ta = srv.submit(A)
        later = [srv.submit(_request(range(k, 220, 50), slot=3 + k % 2, kind=k % 2))
                 for k in range(4)]
        mixed, _ = srv.poll(ta)
        assert _same(mixed, ref)
        rb, _ = srv.poll(big)
        assert np.all(rb["status"] == 0)
        for t in later:
            r, lat = srv.poll(t)
            assert np.all(r["status"] == 0) and lat > 0
        assert srv.info()["launches"] > 1
    finally:
        srv.close()


def test_admission_waits_for_pool_memory(ctx):
    # a pool that holds one request at a time: the second waits, then runs
    A = _request(range(0, 220, 55), slot=0, max_eval=60_000)
    ref = ctx.eval(A, G.MIXED)
    caps = sum(3 + (60_000 + n) // (2 * n) for n in (93, 149, 241)) * 4
    srv = G.Server(ctx, G.MIXED, max_items_per_term=64, pool_regions=caps + 10)
    try:
        t1, t2 = srv.submit(A), srv.submit(A)
        info = srv.info()
        assert info["queued"] + info["admitted"] >= 1
        r1, _ = srv.poll(t1)
        r2, _ = srv.poll(t2)
        assert _same(r1, ref) and _same(r2, ref)
        assert srv.info()["free_regions"] == caps + 10
    finally:
        srv.close()


def test_oversized_request_is_rejected(ctx):
    srv = G.Server(ctx, G.MIXED, max_items_per_term=2, pool_regions=1 << 16)
    try:
        with pytest.raises(G.G3LError):
            srv.submit(_request(range(3)))  # 3 integrals of one term > 2 slots
        with pytest.raises(G.G3LError):
            srv.submit(_request([0], max_eval=100_000_000))  # beyond the pool
    finally:
        srv.close()


def test_cancel(ctx):
    srv = G.Server(ctx, G.MIXED, max_items_per_term=512, pool_regions=1 << 21)
    try:
        t = srv.submit(_request(range(0, 220, 2), slot=2, max_eval=1_000_000))
        srv.cancel(t)
        r, _ = srv.poll(t, check=False)
        assert np.all((r["status"] == 0) | (r["status"] == 6))
        # the server keeps serving
        A = _request([17, 99], slot=0)
        got, _ = srv.poll(srv.submit(A))
        assert _same(got, ctx.eval(A, G.MIXED))
        assert srv.info()["running_integrals"] == 0
    finally:
        srv.close()


def test_submissions_from_several_threads(ctx):
    srv = G.Server(ctx, G.MIXED, max_items_per_term=256, pool_regions=1 << 21)
    reqs = [_request(range(k, 220, 40), slot=k % 3) for k in range(6)]
    refs = [ctx.eval(q, G.MIXED) for q in reqs]
    out = [None] * len(reqs)

    def client(k):
        out[k] = srv.poll(srv.submit(reqs[k]))[0]

    try:
        th = [threading.Thread(target=client, args=(k,)) for k in range(len(reqs))]
        for x in th:
            x.start()
        for x in th:
            x.join()
        for k in range(len(reqs)):
            assert _same(out[k], refs[k])
    finally:
        srv.close()


def test_context_submit_and_poll(ctx):
    import ctypes as C
    from g3lhalo_gb300 import api as A
    specs = _request([5, 150], slot=1)
    ref = ctx.eval(specs, G.FP64)
    items, n = ctx.make_items(specs)
    t = C.c_int64()
    assert A.lib().g3l_submit(ctx.h, items, n, G.FP64, C.byref(t)) == 0
    out = (A.Result * n)()
    assert A.lib().g3l_poll(ctx.h, t.value, out, 1) == 0
    assert _same(A.results_to_numpy(out, n), ref)


def test_randomized_stream_with_cancellations(ctx):
    """48 random requests (kind, terms, slot pair, rtol and budget drawn per request)
    from two threads, every fifth cancelled in flight: every integral that finished --
    including those of cancelled requests -- equals g3l_eval bit for bit, the rest report
    G3L_ERR_CANCELLED, and the server ends idle."""
    rng = np.random.default_rng(2026)
    trip = W.triplets_all()
    reqs = []
    for _ in range(48):
        idx = rng.choice(220, int(rng.integers(1, 10)), replace=False)
        kind = int(rng.integers(0, 2))
        s1 = int(rng.integers(0, 6))
        s2 = s1 if kind == G.NMAPMAP or rng.random() < 0.5 else int(rng.integers(0, 6))
        rtol = (1e-3, 1e-4, 1e-5)[int(rng.integers(0, 3))]
        me = int(rng.choice([5_000, 50_000, 200_000]))
        terms = [t for t in (1, 2, 3) if rng.random() < 0.7] or [2]
        reqs.append([(kind, t, s1, s2, tuple(trip[i]), rtol, me) for i in idx for t in terms])
    srv = G.Server(ctx, G.MIXED, max_items_per_term=256, pool_regions=1 << 21,
                   rounds_per_launch=3)
    try:
        tickets, lock = {}, threading.Lock()

        def submit(lo, hi, seed):
            g = np.random.default_rng(seed)
            for i in range(lo, hi):
                t = srv.submit(reqs[i])
                with lock:
                    tickets[i] = t
                time.sleep(float(g.exponential(0.003)))

        th = [threading.Thread(target=submit, args=(0, 24, 1)),
              threading.Thread(target=submit, args=(24, 48, 2))]
        for x in th:
            x.start()
        time.sleep(0.03)
        cancelled = set()
        for i in range(0, 48, 5):
            with lock:
                t = tickets.get(i)
            if t is not None:
                srv.cancel(t)
                cancelled.add(i)
        for x in th:
            x.join()
        for i in range(48):
            r, _ = srv.poll(tickets[i], check=False)
            ok = r["status"] == 0
            if i in cancelled:
                assert np.all(ok | (r["status"] == 6))
            else:
                assert np.all(ok)
            ref = ctx.eval(reqs[i], G.MIXED)
            assert np.array_equal(r["val"][ok], ref["val"][ok])
            assert np.array_equal(r["neval"][ok], ref["neval"][ok])
        assert srv.info()["running_integrals"] == 0
    finally:
        srv.close()


def test_cancel_after_completion_keeps_the_results(ctx):
    srv = G.Server(ctx, G.MIXED, max_items_per_term=64, pool_regions=1 << 20)
    try:
        A = _request([5], slot=0, max_eval=5_000)
        t = srv.submit(A)
        for _ in range(400):  # bounded wait for completion
            if srv.info()["completed"] >= 1:
                break
            time.sleep(0.005)
        srv.cancel(t)          # finished, not yet polled: a no-op
        got, _ = srv.poll(t)
        assert np.all(got["status"] == 0) and _same(got, ctx.eval(A, G.MIXED))
        with pytest.raises(G.G3LError):
            srv.cancel(t)      # already polled
    finally:
        srv.close()

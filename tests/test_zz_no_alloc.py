"""g3l_eval_static (fixed device scratch, no allocation) against g3l_eval.

The file name sorts last so that the entry point is exercised after every other
test has used the library on the same device; it also passes alone in a fresh
process (its first call performs the per-device scratch set-up).
"""
import numpy as np
import pytest

import g3lhalo_gb300 as G
from g3lhalo_gb300 import api as A
from g3lhalo_gb300 import workloads as W
from g3lhalo_gb300.tables import make_tables

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12   # same kernels and inputs as g3l_eval: identical in practice
MIXED_RTOL = 1e-4   # the per-term contract of the mixed-precision form


def _eval_static(ctx, specs, precision):
    items, n = ctx.make_items(specs)
    out = (A.Result * n)()
    st = A.lib().g3l_eval_static(ctx.h, items, n, precision, out)
    return st, A.results_to_numpy(out, n)


@pytest.fixture(scope="module")
def ctx():
    T = make_tables(Nz=64, Nm=128, Nk=256)
    c = G.Context(T, clamp_k=True)
    c.set_hod(0, W.hod_default())
    c.set_hod(1, W.hod_second())
    return c


def _specs():
    trip = W.triplets_all()
    specs = [(G.NNMAP, t, 0, 1, tuple(trip[i]), 1e-4, 200_000) for i in (3, 90, 171) for t in (1, 2, 3)]
    specs += [(G.NMAPMAP, t, 0, 0, tuple(trip[i]), 1e-4, 200_000) for i in (40, 200) for t in (1, 2, 3)]
    return specs


@pytest.mark.parametrize("precision,rtol", [(G.FP64, FP64_RTOL), (G.MIXED, MIXED_RTOL)])
def test_static_entry_matches_eval_on_two_calls(ctx, precision, rtol):
    specs = _specs()
    ref = ctx.eval(specs, precision)
    for _ in range(2):
        st, r = _eval_static(ctx, specs, precision)
        assert st == 0, A.lib().g3l_last_error()
        assert np.all(r["status"] == 0)
        assert np.array_equal(r["neval"], ref["neval"])
        rel = np.abs(r["val"] - ref["val"]) / np.abs(ref["val"])
        assert rel.max() < rtol, rel.max()
        np.testing.assert_allclose(r["result"], ref["result"], rtol=rtol)


def test_static_entry_rejects_oversized_batches(ctx):
    trip = W.triplets_all()
    # too many integrals
    many = [(G.NNMAP, 1, 0, 1, tuple(trip[0]), 1e-4, 1000)] * 1025
    st, _ = _eval_static(ctx, many, G.FP64)
    assert st == 1 and b"1024" in A.lib().g3l_last_error()
    # region pools beyond the fixed scratch
    big = [(G.NNMAP, 3, 0, 1, tuple(trip[0]), 1e-4, 100_000_000)] * 10
    st, _ = _eval_static(ctx, big, G.FP64)
    assert st == 1 and b"bytes of scratch" in A.lib().g3l_last_error()


def test_static_entry_stats_and_threads_on_one_device(ctx):
    """The call's statistics are filled like g3l_eval's; two threads calling at once on
    one device (two contexts sharing its scratch) get their sequential results, because
    the library serialises calls on a device."""
    import threading
    specs = _specs()
    st, r = _eval_static(ctx, specs, G.MIXED)
    assert st == 0
    s = ctx.stats()
    assert s["points_evaluated"] == int(r["neval"].sum())
    assert sum(s["group_points"]) == s["points_evaluated"]
    assert s["escalated_full"] <= s["escalated"]
    T2 = make_tables(Nz=64, Nm=128, Nk=256)
    c2 = G.Context(T2, clamp_k=True)
    c2.set_hod(0, W.hod_second())
    c2.set_hod(1, W.hod_default())
    specs2 = [(k, t, 0, 1 if k == G.NNMAP else 0, th, rt, me) for (k, t, _, _, th, rt, me) in specs]
    seq = [_eval_static(ctx, specs, G.MIXED)[1], _eval_static(c2, specs2, G.MIXED)[1]]
    got = [None, None]

    def run(k, c, sp):
        for _ in range(3):
            got[k] = _eval_static(c, sp, G.MIXED)

    th = [threading.Thread(target=run, args=(0, ctx, specs)),
          threading.Thread(target=run, args=(1, c2, specs2))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for k in range(2):
        assert got[k][0] == 0
        assert np.array_equal(got[k][1]["val"], seq[k]["val"])
        assert np.array_equal(got[k][1]["neval"], seq[k]["neval"])
    c2.close()

"""Stopping a g3l_eval call in flight: g3l_eval_cancel from another thread, and the
deadline option.

The batch mixes short integrals (a small evaluation cap: they finish in a few rounds)
with long ones (a cap of 2e8 at rtol 1e-12: dozens of rounds and about a second of
device time).  A stopped call must return promptly with the long integrals cancelled
(or past their deadline), the short ones exactly as an uninterrupted call gives them,
and a context that evaluates correctly afterwards.
"""
import threading
import time

import numpy as np
import pytest

import g3lhalo_gb300 as G
from g3lhalo_gb300 import workloads as W
from g3lhalo_gb300.tables import make_tables

pytestmark = pytest.mark.gpu

LONG_CAP = 200_000_000


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(make_tables(Nz=64, Nm=128, Nk=256), clamp_k=True)
    c.set_hod(0, W.hod_default())
    c.set_hod(1, W.hod_second())
    return c


def _batch(short_cap=20_000):
    trip = W.triplets_all()
    short = [(G.NNMAP, t, 0, 1, tuple(trip[i]), 1e-4, short_cap) for i in (5, 60) for t in (1, 2, 3)]
    long_ = [(G.NNMAP, 2, 0, 1, tuple(trip[i]), 1e-12, LONG_CAP) for i in range(0, 220, 5)]
    return short, long_


def _timed(ctx, specs, precision=G.MIXED):
    t0 = time.perf_counter()
    r = ctx.eval(specs, precision)
    return r, time.perf_counter() - t0


def test_cancel_from_another_thread(ctx):
    short, long_ = _batch()
    ref_short = ctx.eval(short, G.MIXED)
    full, t_full = _timed(ctx, short + long_)
    assert np.all(full["status"] == 0)
    assert t_full > 0.4, "the long integrals must run long enough to be cancelled"
    out = {}

    def run():
        out["r"], out["t"] = _timed(ctx, short + long_)

    th = threading.Thread(target=run)
    th.start()
    time.sleep(0.15 * t_full)
    ctx.cancel_eval()
    th.join()
    r = out["r"]
    ns = len(short)
    # the long integrals stopped part-way, the call well before its full time
    assert np.all(r["status"][ns:] == 6), r["status"]
    assert np.all(r["neval"][ns:] < LONG_CAP)
    assert np.all(np.isfinite(r["val"][ns:]))
    assert out["t"] < 0.7 * t_full, (out["t"], t_full)
    # integrals that had finished keep their results, bit for bit
    assert np.all(r["status"][:ns] == 0)
    assert np.array_equal(r["val"][:ns], ref_short["val"])
    assert np.array_equal(r["neval"][:ns], ref_short["neval"])
    # the context is usable afterwards, and a cancel with no call running does nothing
    ctx.cancel_eval()
    again = ctx.eval(short, G.MIXED)
    assert np.all(again["status"] == 0)
    assert np.array_equal(again["val"], ref_short["val"])


@pytest.mark.parametrize("use_graph", [1, 0])
def test_deadline(ctx, use_graph):
    # short integrals of a few rounds: they finish while the long ones' rounds are still
    # cheap, well before the deadline (FP64 rounds of the long integrals double in cost)
    short, long_ = _batch(short_cap=3_000)
    ref_short = ctx.eval(short, G.FP64)
    ctx.set_options(use_graph=use_graph, deadline_ms=300.0)
    try:
        r, t = _timed(ctx, short + long_, G.FP64)
    finally:
        ctx.set_options(use_graph=1, deadline_ms=0.0)
    ns = len(short)
    assert np.all(r["status"][ns:] == 10), r["status"]
    assert np.all(r["status"][:ns] == 0)
    assert np.array_equal(r["val"][:ns], ref_short["val"])
    # the FP64 form of the long integrals takes far longer than the deadline; the call
    # ends within a few rounds of it
    assert t < 5.0, t
    again = ctx.eval(short, G.FP64)
    assert np.array_equal(again["val"], ref_short["val"])


def test_deadline_option_validation(ctx):
    with pytest.raises(G.G3LError):
        ctx.set_options(deadline_ms=-1.0)
    with pytest.raises(G.G3LError):
        ctx.set_options(deadline_ms=float("nan"))
    assert ctx.options().deadline_ms == 0.0

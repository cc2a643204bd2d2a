"""Satellite-variance rescaling (the reference's SCALING build) on the device.

g3l_set_scaling gives a HOD slot a rescaling s per mass bin; the same-population pair
count of NNMap 1h and 2h becomes (N_s + s^2 - 1) N_s (src/HOD.cu:78-87,
src/NNMap_Model.cu:563,808).  The reference's SCALING build reads scaling1 for both
types, so to reproduce it both slots get scaling1.

Tolerances as in test_gpu_parity: the FP64 form within 1e-9 of the reference with
identical evaluation counts; mixed precision within the 1e-4 contract of every term.
"""
import os

import numpy as np
import pytest

import g3lhalo_gb300 as G
import pyoracle as P
from g3lhalo_gb300 import workloads as W
from g3lhalo_gb300.tables import make_tables

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-9
TERM_RTOL = 1e-4
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def scal():
    return dict(np.load(os.path.join(HERE, "golden", "ref_scaling_n64.npz")))


@pytest.fixture(scope="module")
def sctx(golden, golden_tables, scal):
    c = G.Context(golden_tables, clamp_k=False)
    c.set_hod(0, golden["hod1"])
    c.set_hod(1, golden["hod2"])
    c.set_scaling(0, scal["scaling1"])
    c.set_scaling(1, scal["scaling1"])
    return c


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), 1e-300)


def _specs(rows, thetas, slot_of):
    return [(G.NNMAP, int(term), *slot_of(int(t1), int(t2)), tuple(thetas[int(it)]), 1e-4,
             int(me)) for it, term, t1, t2, me, v, e, n in rows]


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED])
def test_scaling_matches_reference_build(sctx, golden, scal, precision):
    tol = FP64_RTOL if precision == G.FP64 else TERM_RTOL
    for key, slot_of in (("sc_terms", lambda a, b: (a - 1, b - 1)),
                         ("sc_same_terms", lambda a, b: (0, 0))):
        rows = scal[key]
        r = sctx.eval(_specs(rows, golden["thetas"], slot_of), precision)
        for k, (it, term, t1, t2, me, v, e, n) in enumerate(rows):
            assert r["status"][k] == 0
            assert int(r["neval"][k]) == int(n), (key, k, r["neval"][k], n)
            assert _rel(r["val"][k], v) < tol, (key, k, r["val"][k], v)
            if precision == G.FP64:
                assert _rel(r["err"][k], e) < 1e-6, (key, k, r["err"][k], e)


def test_scaling_stock_methods_prefactor(sctx, golden, scal):
    """NNMap_1h/2h(type 1, 1) with the stock budgets against the SCALING build."""
    th = tuple(golden["thetas"][1])
    specs = [(G.NNMAP, int(t), 0, 0, th, 1e-3, 5_000_000) for t, _ in scal["sc_stock"]]
    for prec, tol in ((G.FP64, 1e-6), (G.MIXED, TERM_RTOL)):
        r = sctx.eval(specs, prec)
        assert np.all(_rel(r["result"], scal["sc_stock"][:, 1]) < tol), (prec, r["result"])


def test_unit_scaling_is_bitwise_no_scaling(golden, golden_tables):
    """s = 1 everywhere gives the unscaled engine's results bit for bit."""
    c = G.Context(golden_tables, clamp_k=False)
    c.set_hod(0, golden["hod1"])
    th = golden["thetas"]
    specs = [(G.NNMAP, t, 0, 0, tuple(th[i]), 1e-4, 30_000) for i in (0, 2) for t in (1, 2)]
    for prec in (G.FP64, G.MIXED):
        a = c.eval(specs, prec)
        c.set_scaling(0, np.ones(golden_tables.Nm))
        b = c.eval(specs, prec)
        c.set_scaling(0, None)
        assert np.array_equal(a["val"], b["val"]) and np.array_equal(a["err"], b["err"])
        assert np.array_equal(a["neval"], b["neval"])


def test_per_slot_scaling_on_rectangular_tables_matches_oracle():
    """Different rescalings on different slots in one launch (128 m x 64 z x 256 k)."""
    T = make_tables(Nz=64, Nm=128, Nk=256)
    h = W.hod_sweep(8, seed=4242)
    j = np.arange(T.Nm)
    sA = 1.0 + 0.3 * np.cos(0.11 * j)
    sB = 0.8 + 0.005 * j
    c = G.Context(T, clamp_k=True)
    trip = W.triplets_all()
    specs, want = [], []
    for slot, (hod, s) in enumerate(((h[1], sA), (h[5], sB), (h[5], None))):
        c.set_hod(slot, hod)
        c.set_scaling(slot, s)
        O = P.Oracle(T, hod, None, clamp_k=True, scaling=None if s is None else (s, s))
        for ti, t in ((17, 1), (120, 2), (200, 1)):
            specs.append((G.NNMAP, t, slot, slot, tuple(trip[ti]), 1e-4, 30_000))
            want.append(O.term(0, t, trip[ti], 1, 1, maxEval=30_000, rtol=1e-4))
    a = c.eval(specs, G.FP64)
    b = c.eval(specs, G.MIXED)
    for k, (v, e, n, res) in enumerate(want):
        assert int(a["neval"][k]) == n and _rel(a["val"][k], v) < FP64_RTOL, (k, a["val"][k], v)
        assert int(b["neval"][k]) == n and _rel(b["val"][k], v) < TERM_RTOL, (k, b["val"][k], v)
    # the scaled slots differ from the unscaled one on the same HOD
    assert abs(a["val"][3] - a["val"][6]) > 1e-3 * abs(a["val"][6])


def test_scaled_slot_through_the_server(sctx, golden):
    th = golden["thetas"]
    specs = [(G.NNMAP, t, 1, 1, tuple(th[i]), 1e-4, 50_000) for i in (1, 3) for t in (1, 2)]
    want = sctx.eval(specs, G.MIXED)
    srv = G.Server(sctx, G.MIXED, max_items_per_term=64, pool_regions=1 << 20)
    try:
        got, _ = srv.poll(srv.submit(specs))
    finally:
        srv.close()
    assert np.array_equal(got["val"], want["val"])
    assert np.array_equal(got["neval"], want["neval"])


def test_set_scaling_rejects_invalid_input(sctx, golden_tables):
    bad = np.ones(golden_tables.Nm)
    bad[3] = np.nan
    with pytest.raises(G.G3LError):
        sctx.set_scaling(2, bad)
    with pytest.raises(G.G3LError):
        sctx.set_scaling(-1, None)
    with pytest.raises(G.G3LError):
        sctx.set_scaling(G.lib().g3l_max_hod_slots(), None)
    with pytest.raises(ValueError):
        sctx.set_scaling(2, np.ones(golden_tables.Nm + 1))


def test_python_model_scaling_constructor(golden, golden_tables, scal):
    """api.NNMapModel(scaling=...) puts scaling1 on both slots, as the reference's SCALING
    build reads it, and reproduces that build's stock NNMap_1h / NNMap_2h (type 1, 1)."""
    from g3lhalo_gb300 import api as A
    m = A.NNMapModel(golden_tables, golden["hod1"], golden["hod2"], precision=G.FP64,
                     clamp_k=False, scaling=(scal["scaling1"], scal["scaling2"]))
    th = golden["thetas"][1]
    for term, want in scal["sc_stock"]:
        got = m.term(int(term), *th, type1=1, type2=1)
        assert _rel(got, want) < 1e-6, (term, got, want)

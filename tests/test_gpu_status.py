"""Per-integral statuses: the engine ends an integral with a status instead of
exiting (the reference exits on any CUDA error, src/cuda_helpers.h:11-19, and ignores
hcubature's status), and the other integrals of the call are unaffected."""
import numpy as np
import pytest

import g3lhalo_gb300 as G
from g3lhalo_gb300 import workloads as W
from g3lhalo_gb300.tables import make_tables

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(make_tables(Nz=64, Nm=128, Nk=256), clamp_k=True)
    c.set_hod(0, W.hod_default())
    return c


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED])
def test_pool_exhaustion_ends_with_status_4(ctx, precision):
    th = tuple(W.triplets_all()[40])
    keep = ctx.options().unlimited_pool
    ctx.set_options(unlimited_pool=64)
    try:
        r = ctx.eval([(G.NNMAP, 1, 0, 0, th, 1e-12, 0),          # unlimited: hits the pool
                      (G.NNMAP, 2, 0, 0, th, 1e-4, 20_000)], precision)
    finally:
        ctx.set_options(unlimited_pool=keep)
    assert r["status"][0] == 4 and np.isfinite(r["val"][0]) and r["neval"][0] > 0
    assert r["status"][1] == 0
    ref = ctx.eval([(G.NNMAP, 2, 0, 0, th, 1e-4, 20_000)], precision)
    assert r["val"][1] == ref["val"][0]


def test_round_cap_ends_with_status_7(ctx):
    th = tuple(W.triplets_all()[90])
    keep = ctx.options().max_rounds
    ctx.set_options(max_rounds=3)
    try:
        r = ctx.eval([(G.NNMAP, 3, 0, 0, th, 1e-12, 1_000_000)], G.MIXED)
    finally:
        ctx.set_options(max_rounds=keep)
    assert r["status"][0] == 7 and r["rounds"][0] == 3 and np.isfinite(r["val"][0])


def test_invalid_items_are_rejected_before_any_work(ctx):
    th = tuple(W.triplets_all()[0])
    for bad in [(7, 1, 0, 0, th, 1e-4, 1000),            # kind
                (G.NNMAP, 4, 0, 0, th, 1e-4, 1000),       # term
                (G.NNMAP, 1, 5, 5, th, 1e-4, 1000),       # unset HOD slot
                (G.NNMAP, 1, 0, 0, th, -1.0, 1000)]:      # rtol
        with pytest.raises(G.G3LError) as e:
            ctx.eval([bad], G.MIXED)
        assert e.value.status == 1


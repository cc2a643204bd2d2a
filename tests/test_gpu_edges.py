"""Edge cases of the cubature contract, against the oracle (FP64 form to 1e-9, mixed
precision to 1e-4, identical evaluation counts in both).

- An empty batch is a no-op.
- A budget below one rule still evaluates the root region once and stops there: the
  reference's loop tests the budget only after the first rule
  (src/hcubature.cpp:931-940).
- Ragged budgets: the batch pop stops at the first region that reaches the budget,
  so the count overshoots maxEval by up to one pair of rules (src/hcubature.cpp:971-985).
- rtol = 0 never converges and runs to the budget.
- Non-finite or non-positive aperture radii are rejected before any work.
"""
import numpy as np
import pytest

import g3lhalo_gb300 as G
import pyoracle as P
from g3lhalo_gb300 import workloads as W
from g3lhalo_gb300.tables import make_tables

pytestmark = pytest.mark.gpu

NPTS = {1: 93, 2: 149, 3: 241}  # Genz-Malik points in 5, 6, 7 dimensions


@pytest.fixture(scope="module")
def setup():
    T = make_tables(Nz=64, Nm=128, Nk=256)
    h1, h2 = W.hod_default(), W.hod_second()
    c = G.Context(T, clamp_k=True)
    c.set_hod(0, h1)
    c.set_hod(1, h2)
    O = P.Oracle(T, h1, h2, clamp_k=True)
    return c, O


def _check(c, O, kind, term, th, rtol, me):
    for prec, tol in ((G.FP64, 1e-9), (G.MIXED, 1e-4)):
        r = c.eval([(kind, term, 0, 1 if kind == G.NNMAP else 0, tuple(th), rtol, me)], prec)
        v, e, n, _ = O.term(kind, term, th, 1, 2, maxEval=me, rtol=rtol)
        assert r["status"][0] == 0
        assert int(r["neval"][0]) == n, (prec, term, me, r["neval"][0], n)
        assert abs(r["val"][0] - v) <= tol * abs(v), (prec, term, me, r["val"][0], v)
    return n


def test_empty_batch(setup):
    c, _ = setup
    for prec in (G.FP64, G.MIXED):
        assert len(c.eval([], prec)) == 0


@pytest.mark.parametrize("term", [1, 2, 3])
def test_budget_below_one_rule_is_the_root_rule(setup, term):
    c, O = setup
    th = W.triplets_all()[33]
    for kind in (G.NNMAP, G.NMAPMAP):
        assert _check(c, O, kind, term, th, 1e-4, 1) == NPTS[term]


@pytest.mark.parametrize("me", [149, 150, 298, 299, 447, 1001, 4321, 20_000])
def test_ragged_budgets(setup, me):
    c, O = setup
    n = _check(c, O, G.NNMAP, 2, W.triplets_all()[150], 1e-4, me)
    assert n >= min(me, NPTS[2]) and n < max(me, NPTS[2]) + 2 * NPTS[2]


def test_zero_rtol_runs_to_the_budget(setup):
    c, O = setup
    n = _check(c, O, G.NMAPMAP, 1, W.triplets_all()[70], 0.0, 12_000)
    assert 12_000 <= n < 12_000 + 2 * NPTS[1]


@pytest.mark.parametrize("bad", [np.nan, np.inf, 0.0, -1e-3])
def test_bad_aperture_radius_is_rejected(setup, bad):
    c, _ = setup
    th = list(W.triplets_all()[5])
    th[1] = bad
    with pytest.raises(G.G3LError) as e:
        c.eval([(G.NNMAP, 1, 0, 1, tuple(th), 1e-4, 1000)], G.MIXED)
    assert e.value.status == 1

"""GPU parity of the mixed-precision form (FP32 integrand, FP64-class decisions).

Contract: every term within 1e-4 relative of the FP64 result of the same
algorithm (the reference's own hcubature_v trajectory, src/hcubature.cpp:1059-1067),
with the same number of integrand evaluations.  Split and selection decisions
whose FP32 inputs are not decisive under the error bounds are re-taken in FP64,
so the region sets, and therefore the evaluation counts, are the reference's.
"""
import numpy as np
import pytest

import g3lhalo_gb300 as G
import pyoracle as P
from g3lhalo_gb300 import workloads as W
from g3lhalo_gb300.tables import make_tables

pytestmark = pytest.mark.gpu

TERM_RTOL = 1e-4     # every term, mixed vs FP64 (and vs the reference build)
REGION_RTOL = 2e-5   # one Genz-Malik region: value, relative to |value|


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), 1e-300)


@pytest.fixture(scope="module")
def rect():
    """The benchmark tables: 64 z x 128 m x 256 k, k clamp on."""
    T = make_tables(Nz=64, Nm=128, Nk=256)
    c = G.Context(T, clamp_k=True)
    c.set_hod(0, W.hod_default())
    c.set_hod(1, W.hod_second())
    return T, c


def _bench_specs(kind, step=9, max_eval=1_000_000):
    trip = W.triplets_all()
    return [(kind, t, 0, 0, tuple(trip[i]), 1e-4, max_eval)
            for i in range(0, len(trip), step) for t in (1, 2, 3)]


@pytest.mark.parametrize("kind", [G.NNMAP, G.NMAPMAP])
def test_mixed_matches_fp64_on_benchmark_triplets(rect, kind):
    """Every 9th of the 220 benchmark triplets, all three terms, maxEval 1e6."""
    _, c = rect
    specs = _bench_specs(kind)
    a = c.eval(specs, G.FP64)
    b = c.eval(specs, G.MIXED)
    assert np.all(b["status"] == 0)
    assert np.array_equal(a["neval"], b["neval"])
    rel = _rel(b["val"], a["val"])
    assert rel.max() < TERM_RTOL, (int(np.argmax(rel)), rel.max())
    assert np.all(_rel(b["result"], a["result"]) < TERM_RTOL)


@pytest.mark.parametrize("kind", [G.NNMAP, G.NMAPMAP])
def test_reevaluation_caches_match_the_batched_kernel(rect, kind, monkeypatch):
    """The device-wide FP64 re-evaluation passes compute u_NFW, the aperture filter of
    l3, P_lin, the bispectrum, r_200 and the NFW normalisation once per projection of the
    rule's points (or per (mass, z) pair) and share them; the batched kernel k_reeval64
    evaluates every point on its own.  Sending every entry through the batched kernel
    (G3L_REEVAL_CAP=0, read when a context allocates its workspace) changes no value,
    error or evaluation count: the cached values are bit-identical."""
    T, c = rect
    specs = _bench_specs(kind, step=22)
    a = c.eval(specs, G.MIXED)
    esc = c.stats()["escalated"]
    assert esc > 0
    monkeypatch.setenv("G3L_REEVAL_CAP", "0")
    c2 = G.Context(T, clamp_k=True)
    c2.set_hod(0, W.hod_default())
    c2.set_hod(1, W.hod_second())
    b = c2.eval(specs, G.MIXED)
    assert c2.stats()["escalated"] == esc
    for k in ("val", "err", "neval", "status"):
        assert np.array_equal(a[k], b[k]), k


def test_mixed_two_populations_and_sweep_hods(rect):
    """Distinct lens populations, and HODs drawn from the fitter's sweep."""
    T, _ = rect
    c = G.Context(T, clamp_k=True)
    hods = W.hod_sweep(64, seed=12345)
    trip = W.triplets_all()
    for h1, h2 in ((hods[7], hods[20]), (hods[30], hods[30])):
        c.set_hod(0, h1)
        c.set_hod(1, h2)
        specs = [(G.NNMAP, t, 0, 1, tuple(trip[i]), 1e-4, 400_000)
                 for i in range(3, 220, 23) for t in (1, 2, 3)]
        specs += [(G.NMAPMAP, t, 1, 1, tuple(trip[i]), 1e-4, 400_000)
                  for i in range(5, 220, 31) for t in (1, 2, 3)]
        a = c.eval(specs, G.FP64)
        b = c.eval(specs, G.MIXED)
        assert np.array_equal(a["neval"], b["neval"])
        rel = _rel(b["val"], a["val"])
        assert rel.max() < TERM_RTOL, (int(np.argmax(rel)), rel.max())


@pytest.fixture(scope="module")
def gctx(golden, golden_tables):
    c = G.Context(golden_tables, clamp_k=False)
    c.set_hod(0, golden["hod1"])
    c.set_hod(1, golden["hod2"])
    c.set_hod(2, golden["hod2"])
    return c


@pytest.mark.parametrize("rows,kind,slots", [
    ("nn_terms", G.NNMAP, lambda a, b: (a - 1, b - 1)),
    ("nn_same_terms", G.NNMAP, lambda a, b: (0, 0)),
    ("nm_terms", G.NMAPMAP, lambda a, b: (2, 2)),
])
def test_mixed_matches_reference_build(gctx, golden, rows, kind, slots):
    """Against the values and evaluation counts of the reference's own CPU build
    (the reference's unclamped P_lin read included)."""
    specs = []
    for it, term, t1, t2, me, v, e, n in golden[rows]:
        h1, h2 = slots(int(t1), int(t2))
        specs.append((kind, int(term), h1, h2, tuple(golden["thetas"][int(it)]), 1e-4, int(me)))
    r = gctx.eval(specs, G.MIXED)
    for k, (it, term, t1, t2, me, v, e, n) in enumerate(golden[rows]):
        assert r["status"][k] == 0
        assert int(r["neval"][k]) == int(n), (k, r["neval"][k], n)
        assert _rel(r["val"][k], v) < TERM_RTOL, (k, r["val"][k], v)


def test_mixed_region_rule_matches_oracle(rect):
    """One Genz-Malik rule application (value and error) on regions at several depths."""
    T, c = rect
    O = P.Oracle(T, W.hod_default(), W.hod_second(), clamp_k=True)
    trip = W.triplets_all()
    rng = np.random.default_rng(7)
    for kind, term, ti in ((0, 1, 12), (0, 2, 77), (0, 3, 150), (1, 1, 30), (1, 2, 99), (1, 3, 200)):
        dim = term + 4
        lo, hi = O.bounds(term)
        lo, hi = np.asarray(lo), np.asarray(hi)
        hw0 = 0.5 * (hi - lo)
        rootvol = float(np.prod(2 * hw0))
        spec = (kind, term, 0, 1, tuple(trip[ti]), 1e-4, 100000)
        # regions below 1e-20 of the whole integral may underflow the FP32 range
        vroot, _, _ = O.region(kind, term, trip[ti], lo + hw0, hw0, rootvol, 1, 2)
        floor = 1e-20 * abs(vroot)
        for depth in (0, 2, 4):
            lev = rng.integers(0, depth + 1, size=dim)
            cells = rng.integers(0, 2 ** lev)
            center = lo + (2 * cells + 1) * hw0 * 2.0 ** (-lev)
            _, (v32, e32, _) = c.debug_region(spec, center, lev, G.MIXED)
            v, e, _ = O.region(kind, term, trip[ti], center, hw0 * 2.0 ** (-lev),
                               rootvol * 2.0 ** (-int(lev.sum())), 1, 2)
            assert abs(v32 - v) <= REGION_RTOL * abs(v) + floor, (kind, term, depth, v32, v)
            assert abs(e32 - e) <= REGION_RTOL * abs(v) + floor, (kind, term, depth, e32, e)


def test_mixed_batch_invariance_and_determinism(rect):
    """A mixed-precision result does not depend on the rest of the batch and is
    bit-identical between runs (no floating-point atomics in any sum)."""
    _, c = rect
    specs = _bench_specs(G.NNMAP, step=20, max_eval=300_000)
    a = c.eval(specs, G.MIXED)
    b = c.eval(specs, G.MIXED)
    assert np.array_equal(a["val"], b["val"]) and np.array_equal(a["err"], b["err"])
    for k in (0, 4, 8, len(specs) - 1):
        one = c.eval([specs[k]], G.MIXED)
        assert one["val"][0] == a["val"][k] and one["neval"][0] == a["neval"][k]


def test_mixed_statistics(rect):
    _, c = rect
    c.eval(_bench_specs(G.NNMAP, step=40), G.MIXED)
    st = c.stats()
    assert st["rounds"] > 0 and st["kernel_launches"] > 0
    assert st["points_evaluated"] > 0 and st["regions_evaluated"] > 0
    assert st["escalated"] > 0   # FP64 re-evaluations happen on these integrals
    assert st["device_ms"] > 0


def test_autotune_picks_a_variant_per_term_and_keeps_parity(rect):
    """g3l_autotune times the three register-budget variants of the rule kernels on a
    batch and keeps the fastest per kind x term; the results stay within the contract."""
    T, _ = rect
    c = G.Context(T, clamp_k=True)
    c.set_hod(0, W.hod_default())
    specs = _bench_specs(G.NNMAP, step=22, max_eval=200_000)
    variants, ms = c.autotune(specs)
    assert all(v in (0, 1, 2) for v in variants)
    assert np.all(ms[:3] > 0)                      # NNMap groups timed for every variant
    assert list(c.options().evalmx_variant) == variants
    assert c.options().use_graph == 1              # the tuner restores the graph path
    a = c.eval(specs, G.FP64)
    b = c.eval(specs, G.MIXED)
    assert np.array_equal(a["neval"], b["neval"])
    assert _rel(b["val"], a["val"]).max() < TERM_RTOL


@pytest.mark.parametrize("rtol", [1e-2, 1e-3, 1e-5])
def test_mixed_matches_fp64_at_other_tolerances(rect, rtol):
    """The serving stream's tolerances: every term within 1e-4 of the FP64 form and the
    same evaluation counts, both kinds (rtol sets how many regions each round pops, so
    each tolerance is its own trajectory)."""
    T, _ = rect
    c = G.Context(T, clamp_k=True)
    hods = W.hod_sweep(16, seed=99)
    c.set_hod(0, hods[0])
    c.set_hod(1, hods[1])
    trip = W.triplets_all()
    for kind in (G.NNMAP, G.NMAPMAP):
        specs = [(kind, t, 0, 1 if kind == G.NNMAP else 0, tuple(trip[i]), rtol, 300_000)
                 for i in range(0, 220, 22) for t in (1, 2, 3)]
        a = c.eval(specs, G.FP64)
        b = c.eval(specs, G.MIXED)
        assert np.array_equal(a["neval"], b["neval"])
        assert _rel(b["val"], a["val"]).max() < TERM_RTOL


def _region_set(c, index, dim):
    p = c.debug_pool(index)
    n = p["n"]
    cen = p["centers"][:dim * n].reshape(dim, n).T
    lev = p["levels"][:dim * n].reshape(dim, n).T
    return {tuple(cen[j]) + tuple(lev[j]) for j in range(n)}


def test_gladwell_count_near_its_threshold_follows_fp64(rect):
    """A 3-halo term whose value nearly cancels (V = 2 against an error of 110 in round
    16, rtol 1e-3): the Gladwell count -- how many regions leave the error within
    rtol |V| -- sits within the FP32 noise of the sums it compares.  The mixed form
    re-takes that decision after FP64 re-evaluation (unc_thr), so it cuts the same
    regions as the FP64 form; unguarded, it cut one region more in round 16 and ended
    7.3e-5 away (the same evaluation count: the budget cap evens the total out)."""
    T, _ = rect
    c = G.Context(T, clamp_k=True)
    c.set_hod(0, W.hod_sweep(64, seed=12345)[46])
    th = (0.00014545, 0.00046177496601754924, 0.0006786865952253847)
    spec = (G.NNMAP, 3, 0, 0, th, 1e-3, 1_000_000)
    a = c.eval([spec], G.FP64)
    sa = _region_set(c, 0, 7)
    b = c.eval([spec], G.MIXED)
    sb = _region_set(c, 0, 7)
    assert c.stats()["thr_checks"] > 0
    c.close()
    assert a["neval"][0] == b["neval"][0]
    assert sa == sb, (len(sa - sb), len(sb - sa))
    assert _rel(b["val"], a["val"])[0] < 1e-5

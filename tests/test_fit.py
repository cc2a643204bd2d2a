"""The HOD fitting client (g3lhalo_gb300/fit.py).

CPU: the Nelder-Mead minimiser and the parameter mapping.  GPU: a fit of one HOD
parameter to synthetic <N N M_ap> data made with a known parameter vector recovers it,
with every simplex evaluated through the continuous-batching server."""
import numpy as np
import pytest

from g3lhalo_gb300 import fit as F


def test_nelder_mead_minimises_a_quadratic_valley():
    def fmany(xs):
        return [float((x[0] - 1.0) ** 2 + 10.0 * (x[1] + 2.0) ** 2) for x in xs]
    x, f, hist = F.nelder_mead(fmany, [0.0, 0.0], [0.5, 0.5], iters=200)
    assert np.allclose(x, [1.0, -2.0], atol=1e-4) and f < 1e-8
    assert all(b <= a for a, b in zip(hist, hist[1:]))  # the best vertex never worsens


def test_parameter_mapping_round_trips():
    p1 = F.params_from_log10(12.0, 0.2, 13.5, 1.0)
    p2 = F.params_from_log10(12.8, 0.3, 14.0, 0.9)
    p = np.array([p1[0], p2[0], p1[1], p2[1], p1[2], p2[2], p1[3], p2[3], p1[4], p2[4],
                  p1[5], p2[5]])
    h1, h2 = F.hods_from_params(p)
    assert np.isclose(np.log10(h1[2]), 12.0) and np.isclose(np.log10(h2[4]), 14.0)
    assert np.isclose(h1[3], p1[3]) and np.isclose(h2[5], 0.9)


@pytest.mark.gpu
def test_fit_recovers_the_threshold_mass():
    import g3lhalo_gb300 as G
    from g3lhalo_gb300 import workloads as W
    from g3lhalo_gb300.tables import make_tables
    T = make_tables(Nz=64, Nm=128, Nk=256)
    ctx = G.Context(T)
    srv = G.Server(ctx, G.MIXED, max_items_per_term=512, pool_regions=1 << 22)
    try:
        trip = W.triplets_all()
        thetas = np.array([trip[i] for i in (0, 60, 120, 180, 219)])
        p1 = F.params_from_log10(12.0, 0.2, 13.5, 1.0)
        p2 = F.params_from_log10(12.8, 0.3, 14.0, 0.9)
        truth = np.array([p1[0], p2[0], p1[1], p2[1], p1[2], p2[2], p1[3], p2[3], p1[4],
                          p2[4], p1[5], p2[5]])
        free = [4]  # log10 Mth of population 1
        chi = F.ChiSquared(srv, ctx, thetas, np.zeros(45), np.eye(45), truth, free,
                           lo=[11.0], hi=[13.5], max_eval=20_000)
        data = chi.model_many([truth[free]])[0]
        chi.data = data
        chi.icov = np.diag(1.0 / (0.01 * np.abs(data)) ** 2)  # 1% errors
        x, f, hist = F.nelder_mead(chi.many, [12.3], [0.1], iters=40, tol=1e-12)
        assert abs(x[0] - 12.0) < 0.01, (x, f)
        assert f < 1e-2 * hist[0]
        assert chi.calls > 10
    finally:
        srv.close()

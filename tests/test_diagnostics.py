"""The FP32 error-model diagnostic (g3lhalo_gb300.diagnostics): rule weights and the
effective eps of a region's decision quantities, on constructed values (CPU)."""
import numpy as np
import pytest

from g3lhalo_gb300 import diagnostics as dg


@pytest.mark.parametrize("dim", [5, 6, 7])
def test_rule_weights_integrate_constants(dim):
    r7, r5 = dg.rule_weights(dim)
    n = 1 + 4 * dim + 2 * dim * (dim - 1) + (1 << dim)
    assert r7.shape == (n,) and r5.shape == (n,)
    # both rules integrate 1 exactly over the unit-volume region
    assert abs(r7.sum() - 1.0) < 1e-14
    assert abs(r5.sum() - 1.0) < 1e-14
    # the 5th-degree rule has no corner points
    assert np.all(r5[1 + 4 * dim + 2 * dim * (dim - 1):] == 0)


def _values(dim, seed=3):
    rng = np.random.default_rng(seed)
    n = 1 + 4 * dim + 2 * dim * (dim - 1) + (1 << dim)
    return rng.uniform(0.5, 2.0, n).astype(np.float32)


def test_exact_values_have_zero_effective_eps():
    v32 = _values(6)
    e = dg.effective_eps(v32, v32.astype(np.float64) * 4.0, 6, tau=0.0, scale=4.0)
    assert e == {"val": 0.0, "err": 0.0, "diff": 0.0}


def test_one_perturbed_point():
    dim, delta, s = 6, 3e-5, 2.5
    v32 = _values(dim)
    v64 = v32.astype(np.float64) * s
    p = 1 + 4 * 2  # the first axis point of dimension 2
    v64[p] *= 1 + delta
    e = dg.effective_eps(v32, v64, dim, tau=0.0, scale=s)
    a = np.abs(v32.astype(np.float64))
    r7, r5 = dg.rule_weights(dim)
    err_p = delta * a[p]
    assert e["val"] == pytest.approx(abs(r7[p]) * err_p / np.sum(np.abs(r7) * a), rel=1e-9)
    assert e["err"] == pytest.approx(abs(r7[p] - r5[p]) * err_p / np.sum(np.abs(r7 - r5) * a),
                                     rel=1e-9)
    b = 1 + 4 * 2
    U = a[b] + a[b + 1] + dg.RATIO * (a[b + 2] + a[b + 3]) + (2 - 2 * dg.RATIO) * a[0]
    assert e["diff"] == pytest.approx(err_p / U, rel=1e-9)


def test_scale_defaults_to_the_median_ratio():
    dim = 5
    v32 = _values(dim)
    v64 = v32.astype(np.float64) * 7.0
    v64[0] *= 1 + 1e-4  # one outlier does not move the median
    e = dg.effective_eps(v32, v64, dim, tau=0.0)
    assert e["diff"] > 0 and e["val"] > 0
    e2 = dg.effective_eps(v32, v64, dim, tau=0.0, scale=7.0)
    assert e["val"] == pytest.approx(e2["val"], rel=1e-9)

"""The table precomputation on the device (g3l_precompute_tables).

Against the reference's own doPrecomputations pipeline (tests/golden/ref_precompute.npz,
written by tests/golden/make_golden.py --precompute from its Cosmology, Powerspectrum and
HMF classes) and against the oracle restatement (oracle/precompute.c) on other inputs.
Tolerance: the device runs the reference's refinement with the same operations, so the
tables differ only by the device libm's last-ulp differences (measured: <= 5e-14
relative, the mass function the largest); 1e-11 is required of every entry.
"""
import os

import numpy as np
import pytest

import g3lhalo_gb300 as G
import pyoracle as P
from g3lhalo_gb300 import api as A

pytestmark = pytest.mark.gpu

RTOL = 1e-11
KEYS = ("g", "w", "dwdz", "P_lin", "conc", "hmf", "b_h")
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(HERE, "golden", "ref_precompute.npz")))


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), 1e-300)


@pytest.mark.parametrize("ci", [0, 1])
def test_device_tables_match_the_reference(gold, ci):
    zmin, zmax, mmin, mmax, kmin, kmax, N = gold[f"c{ci}_in"]
    r = G.precompute_tables(gold[f"c{ci}_cosmo"], gold["nz_z"], gold["nz_v"], zmin, zmax, mmin,
                            mmax, kmin, kmax, int(N))
    for k in KEYS:
        assert _rel(r[k], gold[f"c{ci}_{k}"]).max() < RTOL, k
    assert _rel(r["amplitude"], gold[f"c{ci}_amplitude"][0]) < RTOL
    assert r["integrals"] == 1 + int(N) + len(gold["nz_z"]) + int(N) * (2 * int(N) + 256)


def test_device_tables_match_the_oracle_at_other_inputs():
    cosmo = (0.27, 0.73, 0.05, 0.9, 72.0, 0.95)
    z = np.linspace(0.0, 2.5, 41)
    nz = np.exp(-0.5 * ((z - 0.9) / 0.3) ** 2)
    args = (0.05, 1.2, 1e11, 1e16, 0.005, 500.0, 20)
    r = G.precompute_tables(cosmo, z, nz, *args)
    o = P.precompute(cosmo, z, nz, *args)
    for k in KEYS:
        assert _rel(r[k], o[k]).max() < RTOL, k


def test_precomputed_tables_feed_the_model(gold):
    """From a cosmology to <N N M_ap>: device tables, then the FP64 model against the
    oracle on the same tables (values to 1e-9, identical evaluation counts)."""
    zmin, zmax, mmin, mmax, kmin, kmax, N = gold["c0_in"]
    N = int(N)
    zs = zmin + np.arange(N) * ((zmax - zmin) / N)
    pl = np.exp(-0.5 * ((zs - 0.5) / 0.15) ** 2)
    T = A.precomputed_tables(gold["c0_cosmo"], gold["nz_z"], gold["nz_v"], zmin, zmax, mmin, mmax,
                             kmin, kmax, N, pl)
    h = [0.9, 1.0, 3e12, 0.3, 3e13, 1.0]
    c = G.Context(T, clamp_k=True)
    c.set_hod(0, h)
    O = P.Oracle(T, h, None, clamp_k=True)
    th = np.array([1.0, 2.0, 4.0]) * 2.909e-4
    specs = [(G.NNMAP, t, 0, 0, tuple(th), 1e-4, 30_000) for t in (1, 2, 3)]
    r = c.eval(specs, G.FP64)
    for k, t in enumerate((1, 2, 3)):
        v, e, n, _ = O.term(0, t, th, 1, 1, maxEval=30_000, rtol=1e-4)
        assert int(r["neval"][k]) == n and _rel(r["val"][k], v) < 1e-9, (t, r["val"][k], v)


def test_invalid_precompute_input_is_reported():
    z = np.linspace(0, 2, 10)
    with pytest.raises(G.G3LError):
        G.precompute_tables((0.3, 0.7, 0.045, 0.8, 70.0, 0.96), z, z, 0.1, 2.0, 1e10, 1e17,
                            0.01, 1000.0, 0)
    with pytest.raises(G.G3LError):
        G.precompute_tables((np.nan, 0.7, 0.045, 0.8, 70.0, 0.96), z, z, 0.1, 2.0, 1e10, 1e17,
                            0.01, 1000.0, 8)


def test_overflow_pass_gives_the_same_tables(gold, monkeypatch):
    """Integrals that outgrow the first pass's region capacity run again with a larger
    one from their root region; forcing most of them through that pass (a 64-region
    first pass) changes no table entry."""
    zmin, zmax, mmin, mmax, kmin, kmax, N = gold["c1_in"]
    args = (gold["c1_cosmo"], gold["nz_z"], gold["nz_v"], zmin, zmax, mmin, mmax, kmin, kmax,
            int(N))
    a = G.precompute_tables(*args)
    monkeypatch.setenv("G3L_PC_FIRST_CAP", "64")
    b = G.precompute_tables(*args)
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), k
    assert a["points"] == b["points"]

"""The reference's ASCII inputs (g3l_read_*, g3lhalo_gb300/reference_files.py).

Against the reference's own readers (g3lhalo::Function, Function2D, Params, Cosmology
compiled from its sources by oracle/build_ref.sh), bit for bit, on files that exercise
their rules: linear interpolation with a default outside [x_first, x_last) (the last
file point itself included), reading that stops at the first non-number, log bins,
2-D tables taken in file order, comments and key order in parameter files.  Then a
round trip of the golden tables through files in the reference's formats.  Host only.
"""
import os

import numpy as np
import pytest

import g3lhalo_gb300 as G
from g3lhalo_gb300 import reference_files as RF

try:
    import pyoracle as P
    HAVE_REF = P.build_ref() is not None
except Exception:  # pragma: no cover - reference build absent
    HAVE_REF = False

needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference CPU build unavailable")


def _ref_function(path, N, lo, hi, default=0.0, log_bins=False):
    out = np.empty(N)
    assert P.ref_lib().ref_function_read(str(path).encode(), default, N, lo, hi,
                                         1 if log_bins else 0, P._ptr(out)) == 0
    return out


def _ref_function2d(path, N, a, b, c, d, default=0.0):
    out = np.empty(N * N)
    assert P.ref_lib().ref_function2d_read(str(path).encode(), default, N, a, b, c, d,
                                           P._ptr(out)) == 0
    return out.reshape(N, N)


def _write(path, rows, fmt="%.17g", tail=""):
    with open(path, "w") as f:
        for r in rows:
            f.write(" ".join(fmt % v for v in r) + "\n")
        f.write(tail)
    return path


@needs_ref
def test_function_read_matches_reference(tmp_path):
    rng = np.random.default_rng(11)
    x = np.sort(rng.uniform(0.1, 1.5, 40))
    y = rng.normal(size=40)
    f1 = _write(tmp_path / "a.dat", zip(x, y))
    # exact bin points: the last one hits x_last and reads the default
    xb = 0.001 + np.arange(32) * ((2.0 - 0.001) / 32)
    f2 = _write(tmp_path / "b.dat", zip(xb, np.cos(xb)), fmt="  %.9e ")
    f3 = _write(tmp_path / "c.dat", zip(x, y), tail="# trailing words stop the read\n1 2\n")
    for f in (f1, f2, f3):
        for N, lo, hi in ((32, 0.001, 2.0), (64, 0.2, 1.2), (7, -1.0, 3.0)):
            for default in (0.0, -2.5):
                got = RF.read_function(f, N, lo, hi, default=default)
                assert np.array_equal(got, _ref_function(f, N, lo, hi, default)), (f, N)
        got = RF.read_function(f, 50, 0.05, 1.9, log_bins=True)
        assert np.array_equal(got, _ref_function(f, 50, 0.05, 1.9, log_bins=True))
    assert RF.read_function(f2, 32, 0.001, 2.0, default=7.0)[-1] != np.cos(xb[-1])


@needs_ref
def test_function2d_read_matches_reference(tmp_path):
    rng = np.random.default_rng(12)
    N = 16
    z = 0.001 + np.arange(N) * (1.999 / N)
    m = 1e10 * (1e7 ** (np.arange(N) / N))
    rows = [(zi, mj, rng.lognormal()) for zi in z for mj in m]
    f1 = _write(tmp_path / "h.dat", rows, fmt="%.6g")
    f2 = _write(tmp_path / "h2.dat", rows + rows[:5])  # extra rows are ignored
    for f in (f1, f2):
        for args in ((N, 0.001, 2.0, 1e10, 1e17), (N, 0.5, 1.0, 1e12, 1e14)):
            got = RF.read_function2d(f, *args, default=0.5)
            assert np.array_equal(got, _ref_function2d(f, *args, default=0.5))
    got = RF.read_function2d(f1, 8, 0.001, 2.0, 1e10, 1e17)
    assert np.array_equal(got, _ref_function2d(f1, 8, 0.001, 2.0, 1e10, 1e17))


@needs_ref
def test_parameter_files_match_reference(tmp_path):
    hod = tmp_path / "hod.param"
    hod.write_text("# HOD\n\nbeta 0.9\nM_min 3.1e12\nsigma 0.25\nM' 2.2e13\nalpha 0.85\n"
                   "f 1.1\n")
    cos = tmp_path / "cosmo.param"
    cos.write_text("# cosmology\nH0 67.74\nOmega_m 0.3089\nOmega_Lambda 0.6911\n"
                   "Omega_b 0.0486\nsigma8 0.8159\nns 0.9667\n")
    want = np.empty(6)
    P.ref_lib().ref_params_read(str(hod).encode(), P._ptr(want))
    assert np.array_equal(RF.read_hod_params(hod), want)
    P.ref_lib().ref_cosmology_read(str(cos).encode(), P._ptr(want))
    c = RF.read_cosmology(cos)
    assert np.array_equal(c.as_array(), want)


def test_triplets(tmp_path):
    t = np.array([[0.5, 1.0, 2.0], [4.0, 4.0, 8.0], [1e-1, 2.5e0, 16.0]])
    f = _write(tmp_path / "thetas.dat", t, fmt="%.10g")
    assert np.array_equal(RF.read_triplets(f), t)
    assert RF.read_triplets(_write(tmp_path / "empty.dat", [])).shape == (0, 3)


def test_reader_errors_are_reported_not_fatal(tmp_path):
    missing = tmp_path / "missing.dat"
    empty = _write(tmp_path / "empty.dat", [])
    short2d = _write(tmp_path / "short.dat", [(0.1, 1e12, 1.0)] * 10)
    bad = tmp_path / "bad.param"
    bad.write_text("M_min 1e12\nsigma 0.2\nM' 1e13\nbeta 1\nalpha 1\nf 1\ngamma 2\n")
    partial = tmp_path / "partial.param"
    partial.write_text("M_min 1e12\nsigma 0.2\n")
    for call in (lambda: RF.read_function(missing, 8, 0, 1),
                 lambda: RF.read_function(empty, 8, 0, 1),
                 lambda: RF.read_function2d(short2d, 8, 0.0, 2.0, 1e10, 1e17),
                 lambda: RF.read_hod_params(bad),
                 lambda: RF.read_hod_params(partial),
                 lambda: RF.read_cosmology(missing),
                 lambda: RF.read_triplets(missing)):
        with pytest.raises(G.G3LError):
            call()


def test_golden_tables_round_trip_through_reference_formats(tmp_path, golden, golden_tables):
    """The golden N = 64 tables written in the reference's file formats and read back
    as the driver reads them give the same arrays, bit for bit."""
    T = golden_tables
    N = T.Nz
    zs = T.zmin + np.arange(N + 1) * ((T.zmax - T.zmin) / N)  # one point past the last bin
    ms = T.mmin * (T.mmax / T.mmin) ** (np.arange(N) / N)
    ks = T.kmin * (T.kmax / T.kmin) ** (np.arange(N) / N)
    files = {}
    for k in ("g", "p_lens1", "p_lens2", "w", "dwdz"):
        v = getattr(T, k)
        files[k] = _write(tmp_path / (k + ".dat"), zip(zs, np.append(v, v[-1])))
    for k, grid in (("hmf", ms), ("b_h", ms), ("conc", ms), ("P_lin", ks)):
        v = np.asarray(getattr(T, k)).reshape(N, N)
        files[k] = _write(tmp_path / (k + ".dat"),
                          [(zs[i], grid[j], v[i, j]) for i in range(N) for j in range(N)])
    c = golden["cosmo"]
    cos = tmp_path / "cosmo.param"
    cos.write_text("Omega_m %r\nOmega_Lambda %r\nOmega_b %r\nsigma8 %r\nH0 %r\nns %r\n"
                   % tuple(float(x) for x in c))
    R = RF.tables_from_files(cos, T.zmin, T.zmax, T.kmin, T.kmax, T.mmin, T.mmax, N,
                             files["g"], files["p_lens1"], files["p_lens2"], files["w"],
                             files["dwdz"], files["hmf"], files["P_lin"], files["b_h"],
                             files["conc"])
    for k, v in T.arrays().items():
        assert np.array_equal(np.asarray(getattr(R, k)).ravel(), np.asarray(v).ravel()), k
    assert np.array_equal(R.cosmo.as_array(), c)

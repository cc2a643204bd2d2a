import os
import platform
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_n64.npz")
# The golden vectors were produced on x86-64; other hosts may differ from glibc's
# x86 libm in the last bit of a transcendental, so equality is relaxed there.
EXACT_HOST = platform.machine() in ("x86_64", "AMD64")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return load_golden()


def load_golden():
    return dict(np.load(GOLDEN))


def tables_from_golden(g):
    """The N=64 tables the golden vectors were computed on."""
    from g3lhalo_gb300.tables import Cosmology, Tables
    meta = g["tab_meta"]
    c = g["cosmo"]
    cos = Cosmology(Om=c[0], OL=c[1], Ob=c[2], s8=c[3], h=c[4] / 100.0, ns=c[5])
    return Tables(Nz=int(meta[0]), Nm=int(meta[1]), Nk=int(meta[2]), zmin=meta[3], zmax=meta[4],
                  mmin=meta[5], mmax=meta[6], kmin=meta[7], kmax=meta[8], cosmo=cos,
                  g=g["tab_g"], p_lens1=g["tab_p_lens1"], p_lens2=g["tab_p_lens2"], w=g["tab_w"],
                  dwdz=g["tab_dwdz"], hmf=g["tab_hmf"], P_lin=g["tab_P_lin"], b_h=g["tab_b_h"],
                  conc=g["tab_conc"])


@pytest.fixture(scope="session")
def golden_tables(golden):
    return tables_from_golden(golden)


def assert_close(a, b, rtol_exact=0.0, rtol_other=1e-9):
    rtol = rtol_exact if EXACT_HOST else rtol_other
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if rtol == 0.0:
        assert np.array_equal(a, b, equal_nan=True), (a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=rtol, atol=0)

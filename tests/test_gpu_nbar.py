"""n_bar(z) on the device (g3l_set_hod / g3l_set_hods) against the host restatement of
the reference's updateDensities integral (g3l_host_densities, pinned to the reference
build by test_host_library.py) and against itself.

The device evaluates the same expressions with the device's libm, whose pow, erf and
log may differ from the host's in the last bit, so the bar is relative 1e-12 (the golden
parity tests in test_gpu_parity.py use the device n_bar and keep their 1e-9 / identical
evaluation-count bars).
"""
import numpy as np
import pytest

import g3lhalo_gb300 as G
from g3lhalo_gb300 import workloads as W
from g3lhalo_gb300.tables import make_tables

pytestmark = pytest.mark.gpu

NBAR_RTOL = 1e-12


@pytest.fixture(scope="module")
def tables():
    return make_tables(Nz=64, Nm=128, Nk=256)


def test_device_nbar_matches_host_across_the_sweep_box(tables):
    c = G.Context(tables, clamp_k=True)
    hods = np.vstack([W.hod_default(), W.hod_second(), W.hod_sweep(30, seed=99)])
    c.set_hods(np.arange(len(hods)), hods)
    for k, h in enumerate(hods):
        _, dev = c.densities(k)
        _, host = G.host_densities(tables, h)
        np.testing.assert_allclose(dev, host, rtol=NBAR_RTOL, atol=0)
    c.close()


def test_batched_and_single_updates_agree_bit_for_bit(tables):
    """The block-factor table is shared by the z bins and vectors of a launch; who fills
    an entry must not matter."""
    hods = W.hod_sweep(12, seed=5)
    a = G.Context(tables, clamp_k=True)
    b = G.Context(tables, clamp_k=True)
    a.set_hods(np.arange(12), hods)
    for k in range(12):
        b.set_hod(k, hods[k])
    for k in range(12):
        assert np.array_equal(a.densities(k)[1], b.densities(k)[1])
    # the same slot updated again gives the same densities, and a change shows
    b.set_hod(3, hods[3])
    assert np.array_equal(a.densities(3)[1], b.densities(3)[1])
    b.set_hod(3, hods[4])
    assert np.array_equal(a.densities(4)[1], b.densities(3)[1])
    a.close()
    b.close()


def test_set_hods_rejects_bad_input(tables):
    c = G.Context(tables, clamp_k=True)
    bad = W.hod_default().copy()
    bad[2] = -1.0
    with pytest.raises(G.G3LError):
        c.set_hods([0, 1], np.vstack([W.hod_default(), bad]))
    with pytest.raises(G.G3LError):
        c.set_hods([0, 5000], np.vstack([W.hod_default(), W.hod_default()]))
    c.close()

"""Mixed precision against the FP64 form across the fit-sweep box (SURVEY config 3).

32 HOD vectors drawn like the batched fit sweep (log Mth in [11, 13.5], sigma in
[0.1, 0.6], log M1 in [12.5, 14.5], slope in [0.6, 1.4], f in [0.5, 1.5]) x every tenth
of the 220 benchmark triplets x the 1-, 2- and 3-halo terms, at the benchmark's
maxEval 1e6 and rtol 1e-4, each precision in one call (the reference's calculateAll
loop over HOD vectors, src/NNMap_Model.cu:382-415).  Every mixed term must be within
1e-4 relative of the FP64 term with the same evaluation count.
"""
import numpy as np
import pytest

import g3lhalo_gb300 as G
from g3lhalo_gb300 import workloads as W
from g3lhalo_gb300.tables import make_tables

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1e-4  # the per-term contract of the mixed-precision form
N_HOD = 32


@pytest.mark.parametrize("kind", [G.NNMAP, G.NMAPMAP])
def test_sweep_box_mixed_matches_fp64(kind):
    c = G.Context(make_tables(Nz=64, Nm=128, Nk=256), clamp_k=True)
    hods = W.hod_sweep(N_HOD, seed=2024 + kind)
    for k, h in enumerate(hods):
        c.set_hod(k, h)
    trip = W.triplets_all()[::10]
    n_hod = N_HOD if kind == G.NNMAP else N_HOD // 4
    specs = [(kind, t, k, k, tuple(th), 1e-4, 1_000_000)
             for k in range(n_hod) for th in trip for t in (1, 2, 3)]
    rm = c.eval(specs, G.MIXED)
    r64 = c.eval(specs, G.FP64)
    c.close()
    assert np.all(rm["status"] == 0) and np.all(r64["status"] == 0)
    assert np.array_equal(rm["neval"], r64["neval"])
    rel = np.abs(rm["val"] - r64["val"]) / np.abs(r64["val"])
    worst = int(np.argmax(rel))
    assert rel.max() < MIXED_RTOL, (rel.max(), specs[worst])

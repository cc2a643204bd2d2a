"""CPU-side checks of libg3lgpu.so: exported symbols, host densities and the host
cubature entry point (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import g3lhalo_gb300 as G
from g3lhalo_gb300 import api
from conftest import ROOT, assert_close


def test_exports_every_declared_symbol():
    lib = C.CDLL(G.library_path() if os.path.exists(G.library_path()) else api._build.build())
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(g3l_[a-z0-9_]+)\s*\(", src))
    names -= {"g3l_integrand_v"}
    assert len(names) >= 15
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_host_densities_match_reference(golden, golden_tables):
    rho, n1 = G.host_densities(golden_tables, golden["hod1"])
    _, n2 = G.host_densities(golden_tables, golden["hod2"])
    assert_close(rho, golden["nn_rho_bar"])
    assert_close(n1, golden["nn_nbar1"])
    assert_close(n2, golden["nn_nbar2"])


def test_host_hcubature_matches_reference_engine(golden):
    import make_golden as MG
    for ci, dim, me, rtol, v, e, n in golden["engine"]:
        name = MG.ENGINE_CASES[int(ci)][0]
        d = int(dim)
        val, err = G.hcubature_v(MG.FUNCS[name], d, np.zeros(d), np.ones(d), int(me), rtol)
        assert_close([val, err], [v, e], rtol_other=1e-9)


def test_invalid_arguments_are_reported_not_fatal(golden_tables):
    bad = dict(golden_tables.__dict__)
    from g3lhalo_gb300.tables import Tables
    t = Tables(**bad)
    t.hmf = t.hmf.copy()
    t.hmf[3, 4] = np.nan
    with pytest.raises(G.G3LError) as ei:
        G.Context(t)
    assert ei.value.status in (1, 8)  # INVALID on a GPU host, NO_DEVICE without one


def test_header_is_c_and_a_c_program_links(tmp_path):
    """include/g3l_gpu.h is plain C (C11, pedantic) and a C program links the library."""
    import subprocess
    src = tmp_path / "use.c"
    src.write_text('#include "g3l_gpu.h"\n'
                   'int main(void) {\n'
                   '    g3l_tables t = {0}; g3l_integral it = {0}; g3l_result r = {0};\n'
                   '    (void)t; (void)it; (void)r;\n'
                   '    return g3l_abi_version() == G3L_ABI_VERSION ? 0 : 1;\n'
                   '}\n')
    lib = G.library_path()
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror",
                        "-I" + os.path.join(ROOT, "include"), str(src), "-o",
                        str(tmp_path / "use"), "-L" + os.path.dirname(lib), "-lg3lgpu",
                        "-Wl,-rpath," + os.path.dirname(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("table", ["g", "p_lens1", "w", "dwdz", "hmf", "b_h", "conc", "P_lin"])
def test_nonfinite_tables_are_rejected_at_creation(table):
    """A NaN or infinity in any table is refused before any device work (the reference
    would carry it into every result); no GPU is needed to see it."""
    from g3lhalo_gb300.tables import make_tables
    for bad in (np.nan, np.inf):
        T = make_tables(Nz=8, Nm=8, Nk=8)
        a = np.array(getattr(T, table), dtype=np.float64)
        a.flat[a.size // 2] = bad
        setattr(T, table, a)
        with pytest.raises(G.G3LError) as e:
            G.Context(T)
        assert e.value.status == 1

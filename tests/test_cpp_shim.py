"""The C++ model shim (include/g3lhalo_model.hpp): the reference's NNMap_Model /
NMapMap_Model interface over the C ABI.

CPU: the driver compiles and links against libg3lgpu.so, and the header also compiles
against the reference's own class headers where those sources are present.
GPU: the per-term methods reproduce the reference build's own stock results
(NNMap_1h/2h/3h at maxEval 5e6, NMapMap_1h), and calculateAll equals g3l_eval of the
same integrals.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import g3lhalo_gb300 as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle  # noqa: E402  (the checker's helpers: where the reference sources lie)

REF_SRC = pyoracle.ref_src()


def _build_driver(tmp_path):
    lib = G.library_path()
    exe = str(tmp_path / "shim_driver")
    cmd = ["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), "-I" + CPP,
           os.path.join(CPP, "shim_driver.cpp"), "-o", exe, "-L" + os.path.dirname(lib),
           "-lg3lgpu", "-Wl,-rpath," + os.path.dirname(lib),
           "-Wl,--allow-shlib-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_driver_builds_against_the_library(tmp_path):
    _build_driver(tmp_path)


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not mounted")
def test_header_compiles_with_the_reference_classes(tmp_path):
    src = tmp_path / "with_ref.cu"
    src.write_text('#include "Cosmology.h"\n#include "HOD.h"\n#include "g3lhalo_model.hpp"\n'
                   "double f(g3lhalo::NNMap_Model &m) { return m.NNMap(1e-3, 1e-3, 1e-3, 1, 2); }\n"
                   "double h(g3lhalo::NMapMap_Model &m) { return m.NMapMap(1e-3, 1e-3, 1e-3); }\n"
                   "g3lhalo::NNMap_Model *s(g3lhalo::Cosmology *c, double *t, g3lhalo::HOD *a,\n"
                   "                        g3lhalo::HOD *b) {  // the SCALING constructor\n"
                   "    return new g3lhalo::NNMap_Model(c, 0.1, 2., 0.1, 1e3, 1e10, 1e17, 8, t, t, t,\n"
                   "                                    t, t, t, t, t, t, t, t, a, b, 0., 0.); }\n")
    r = subprocess.run(["nvcc", "-std=c++17", "-c", "-I" + REF_SRC,
                        "-I" + os.path.join(ROOT, "include"), str(src), "-o",
                        str(tmp_path / "with_ref.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _write_input(path, g, scaling=None):
    meta = g["tab_meta"]
    with open(path, "wb") as f:
        f.write(np.array([int(meta[0])], dtype=np.int32).tobytes())
        f.write(np.array([meta[3], meta[4], meta[7], meta[8], meta[5], meta[6]]).tobytes())
        f.write(np.asarray(g["cosmo"], dtype=np.float64).tobytes())
        f.write(np.asarray(g["hod1"], dtype=np.float64).tobytes())
        f.write(np.asarray(g["hod2"], dtype=np.float64).tobytes())
        for k in ("tab_g", "tab_p_lens1", "tab_p_lens2", "tab_w", "tab_dwdz"):
            f.write(np.ascontiguousarray(g[k], dtype=np.float64).tobytes())
        for k in ("tab_hmf", "tab_P_lin", "tab_b_h", "tab_conc"):
            f.write(np.ascontiguousarray(g[k], dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(g["thetas"], dtype=np.float64).tobytes())
        if scaling is not None:
            for a in scaling:
                f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())


def _run(exe, path, mixed, scaled=False):
    r = subprocess.run([exe, str(path), "1" if mixed else "0", "1" if scaled else "0"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stderr)
    out = {}
    for line in r.stdout.splitlines():
        k, v = line.split()
        out.setdefault(k, []).append(float(v))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("mixed,rtol", [(False, 1e-9), (True, 1e-4)])
def test_shim_reproduces_the_reference_methods(tmp_path, golden, golden_tables, mixed, rtol):
    exe = _build_driver(tmp_path)
    path = tmp_path / "in.bin"
    _write_input(path, golden)
    out = _run(exe, path, mixed)
    assert out["status"] == [0, 0]
    stock = dict((int(t), v) for t, v in golden["nn_stock"])
    for t in (1, 2, 3):
        got = out["NNMap_%dh" % t][0]
        assert abs(got - stock[t]) <= rtol * abs(stock[t]), (t, got, stock[t])
    assert abs(out["NNMap"][0] - sum(stock.values())) <= rtol * abs(sum(stock.values()))
    nm = golden["nm_stock"][0][1]
    assert abs(out["NMapMap_1h"][0] - nm) <= rtol * abs(nm)
    # calculateAll: N1N2, N1N1, N2N2 blocks over thetas[0:2], one launch
    c = G.Context(golden_tables, clamp_k=False)
    c.set_hod(0, golden["hod1"])
    c.set_hod(1, golden["hod2"])
    th = golden["thetas"]
    specs = [(G.NNMAP, t, a, b, tuple(th[i]), 1e-4 if t == 3 else 1e-3, 5_000_000)
             for a, b in ((0, 1), (0, 0), (1, 1)) for i in range(2) for t in (1, 2, 3)]
    r = c.eval(specs, G.MIXED if mixed else G.FP64)
    want = r["result"].reshape(-1, 3).sum(axis=1)
    got = np.array([out["calculateAll_%d" % k][0] for k in range(6)])
    np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("mixed,rtol", [(False, 1e-9), (True, 1e-4)])
def test_shim_scaling_constructor_reproduces_the_scaling_build(tmp_path, golden, mixed, rtol):
    """The SCALING constructor against the reference's SCALING build (same-population
    NNMap_1h / NNMap_2h at the stock budgets)."""
    scal = dict(np.load(os.path.join(ROOT, "tests", "golden", "ref_scaling_n64.npz")))
    exe = _build_driver(tmp_path)
    path = tmp_path / "in_scaled.bin"
    _write_input(path, golden, (scal["scaling1"], scal["scaling2"]))
    out = _run(exe, path, mixed, scaled=True)
    assert out["status"] == [0]
    for t, want in scal["sc_stock"]:
        got = out["S_NNMap_%dh" % int(t)][0]
        assert abs(got - want) <= rtol * abs(want), (t, got, want)


# A prelude forced into the reference's own driver sources: it defines the include
# guards of the reference's NNMap_Model.h / NMapMap_Model.h, so the drivers' first
# #include becomes a no-op, and brings in the shim after Cosmology.h and HOD.h.
PRELUDE = ('#define G3LHALO_NNMAP_MODEL_H\n#define G3LHALO_NMAPMAP_MODEL_H\n'
           '#include "Cosmology.h"\n#include "HOD.h"\n#include "g3lhalo_model.hpp"\n')


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not mounted")
@pytest.mark.parametrize("driver,defs", [("calculateNNMap", []), ("calculateNMapMap", []),
                                         ("calculateNNMap_twoPop", []),
                                         ("calculateNNMap_twoPop", ["-DSCALING=1"])])
def test_reference_drivers_link_against_the_library(tmp_path, driver, defs):
    """The reference's executables, compiled unmodified from their sources with the shim
    in place of its model classes, link against libg3lgpu.so (src/calculateNNMap.cu,
    src/calculateNNMap_twoPop.cu with and without SCALING, src/calculateNMapMap.cu)."""
    import pyoracle as P
    P.build_ref()  # the reference's own Cosmology, HOD, Params, Function objects
    obj = os.path.join(ROOT, "oracle", "_ref", "obj")
    lib = G.library_path()
    (tmp_path / "prelude.h").write_text(PRELUDE)
    run = lambda cmd: subprocess.run(cmd, capture_output=True, text=True)  # noqa: E731
    r = run(["g++", "-std=c++17", "-O1", "-fopenmp", "-fPIC", "-I" + REF_SRC, "-c",
             os.path.join(REF_SRC, "helpers.cpp"), "-o", str(tmp_path / "helpers.o")])
    assert r.returncode == 0, r.stderr
    r = run(["nvcc", "-std=c++17", "-O1", "-rdc=true", "-Xcompiler", "-fopenmp"] + defs +
            ["-include", str(tmp_path / "prelude.h"), "-I" + os.path.join(ROOT, "include"),
             "-I" + REF_SRC, "-c", os.path.join(REF_SRC, driver + ".cu"), "-o",
             str(tmp_path / "driver.o")])
    assert r.returncode == 0, r.stderr
    objs = [os.path.join(obj, f + ".o") for f in ("Cosmology", "Params", "Function",
                                                  "Function2D", "hcubature", "HOD",
                                                  "generalFunctions")]
    r = run(["nvcc", "-rdc=true", "-Xcompiler", "-fopenmp", str(tmp_path / "driver.o"),
             str(tmp_path / "helpers.o")] + objs + ["-L" + os.path.dirname(lib), "-lg3lgpu",
                                                    "-o", str(tmp_path / (driver + ".x"))])
    assert r.returncode == 0, r.stderr

"""The FP64 re-take of an unsettled split computes only what the centre and the
contending dimensions' axis points read (coordinate slots, u_NFW combinations, k3 and
auxiliary projections, (mass, z) pairs).  tests/cpp/reeval_cover.cu checks, on the host
with the device header's own index functions, that every value a needed point reads is
computed, for every kind, term and mask of contenders (CPU; needs nvcc)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "g3lhalo_gb300", "csrc")


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not on PATH")
def test_split_retake_reads_only_computed_values(tmp_path):
    exe = str(tmp_path / "reeval_cover")
    r = subprocess.run(["nvcc", "-std=c++17", "-I", CSRC, "-o", exe,
                        os.path.join(HERE, "cpp", "reeval_cover.cu")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok ")
    assert int(r.stdout.split()[1]) > 80000  # every kind x term x mask x needed point

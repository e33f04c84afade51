"""The facet-patch basis change of the patch kernel (csrc/xg_patch.cuh),
checked on the host: node images, hierarchical interpolation and the
reconstruction of every function of the neighbour for random affine maps, all
dimensions and orders.  Compiles tests/native/patch_basis_check.cu with nvcc
(host code only; no GPU needed)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_patch_basis_change_is_exact(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "patch_basis_check")
    subprocess.check_call([nvcc, "-x", "cu", "-std=c++17", "-O1",
                           "-I", os.path.join(ROOT, "ngsxfem_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "native", "patch_basis_check.cu"), "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

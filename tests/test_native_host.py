"""Host checks of the exact reformulations in the element kernels, compiled
with nvcc as host code (no GPU needed):

* tests/native/moment_tables_check.cu: the integer term tables of the cut
  element moment kernels (csrc/xg_moments.cuh) reproduce every integrand of
  the term menu at random barycentric points (D = 2, 3; K = 1..3; packed and
  full entry orders);
* tests/native/patch_basis_check.cu: the facet-patch basis change
  (csrc/xg_patch.cuh) reproduces every function of the neighbour for random
  affine maps."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _run(tmp_path, name):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / name)
    subprocess.check_call([nvcc, "-x", "cu", "-std=c++17", "-O1",
                           "-I", os.path.join(ROOT, "ngsxfem_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "native", name + ".cu"), "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_moment_tables_reproduce_the_integrands(tmp_path):
    _run(tmp_path, "moment_tables_check")


def test_patch_basis_change_is_exact(tmp_path):
    _run(tmp_path, "patch_basis_check")


def test_edge_and_face_numbering_beyond_2_21_vertices(tmp_path):
    """xg_mesh_create numbers faces by full sorted vertex triples: vertex
    numbers up to 2^24 keep every face distinct and the lexicographic order."""
    _run(tmp_path, "topology_check")

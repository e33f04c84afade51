"""Build recipe of libxg.so (sm_103a only), in-tree under ngsxfem_gb300/_build.

    python -m ngsxfem_gb300.build          # builds if sources changed
    python -m ngsxfem_gb300.build --force

xg_geom.cu, xg_quad.cu and xg_mlset.cu are compiled with -fmad=false: they hold
the marking and rule-export kernels whose cut points, volumes and weights
follow the CPU statement operation by operation.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libxg.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
UNITS = [
    ("xg_host.cpp", []),
    ("xg_geom.cu", ["-fmad=false"]),
    ("xg_asm.cu", []),
    ("xg_st.cu", []),
    ("xg_iso.cu", ["-fmad=false"]),
    ("xg_learn.cu", []),
    ("xg_lf.cu", []),
    ("xg_quad.cu", ["-fmad=false"]),
    ("xg_quad_int.cu", []),
    ("xg_mlset.cu", ["-fmad=false"]),
    ("xg_isomesh.cu", ["-fmad=false"]),
    ("xg_rows.cu", []),
    ("xg_mlp_tc.cu", []),
    ("xg_skel.cu", []),
    ("xg_subdiv.cu", []),
    ("xg_mlform.cu", []),
    ("xg_bform.cu", []),
    ("xg_cform.cu", []),
    ("xg_qform.cu", []),
]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libxg needs the CUDA toolkit to build")


def _sources():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "xg.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _sources())


def build(force=False, verbose=False, extra_flags=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nv = nvcc()
    procs = []
    objs = []
    for src, flags in UNITS:
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        cmd = [nv, "-c", os.path.join(CSRC, src), "-o", obj] + COMMON + ARCH + list(flags) + list(extra_flags)
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append(" ".join(cmd) + "\n" + text)
        elif verbose and text.strip():
            print(text)
    if failed:
        raise RuntimeError("libxg build failed:\n" + "\n".join(failed))
    tmp = LIB + ".tmp"
    cmd = [nv, "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC", "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)

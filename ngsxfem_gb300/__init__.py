"""ngsxfem_gb300: GB300-native (sm_103a) cut-element assembly.

The compute path is libxg.so (C ABI in include/xg.h); this package holds the
Python mirror of ngsxfem's interface for that path (ngsxfem_gb300.xfem) and
the structured mesh generators used as inputs.  Importing the package does not
load the library; the first call into it does, and fails loudly if libxg.so is
missing.
"""
from .meshes import Mesh, MakeStructured2DMesh, MakeStructured3DMesh  # noqa: F401

__all__ = ["Mesh", "MakeStructured2DMesh", "MakeStructured3DMesh"]

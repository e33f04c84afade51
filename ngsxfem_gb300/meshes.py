"""Structured simplex meshes (the inputs ngsolve.meshes.MakeStructured2DMesh /
MakeStructured3DMesh provide to ngsxfem's tests and demos).

NGSolve's generators are not available, so the split pattern is this project's
own and is stated here:

* 2D: each quad (p00, p10, p11, p01) is split along the p00-p11 diagonal into
  the triangles (p00, p10, p11) and (p00, p11, p01).
* 3D: each cube is split into the 6 Kuhn (Freudenthal) tetrahedra
  [v000, v000+e_a, v000+e_a+e_b, v111] for the 6 permutations (a, b, c) of the
  axes, which is conforming across cubes.

Vertices are numbered with x fastest.  Arrays are numpy: coords (nv, dim)
float64, elements (ne, dim+1) int32.
"""
import itertools

import numpy as np


class Mesh:
    """A simplex mesh held on the host: vertex coordinates and element vertices."""

    def __init__(self, coords, elements):
        self.coords = np.ascontiguousarray(coords, dtype=np.float64)
        self.elements = np.ascontiguousarray(elements, dtype=np.int32)
        self.dim = self.coords.shape[1]
        if self.elements.shape[1] != self.dim + 1:
            raise ValueError("only simplex meshes (trig / tet) are supported")
        self._device = None

    @property
    def nv(self):
        return self.coords.shape[0]

    @property
    def ne(self):
        return self.elements.shape[0]

    def GetNE(self):
        return self.ne

    def GetNV(self):
        return self.nv


def MakeStructured2DMesh(nx=10, ny=10, xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0):
    xs = np.linspace(xmin, xmax, nx + 1)
    ys = np.linspace(ymin, ymax, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    i = i.ravel()
    j = j.ravel()
    p00 = i + (nx + 1) * j
    p10 = p00 + 1
    p01 = p00 + (nx + 1)
    p11 = p01 + 1
    t1 = np.stack([p00, p10, p11], axis=1)
    t2 = np.stack([p00, p11, p01], axis=1)
    el = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return Mesh(coords, el)


def MakeStructured3DMesh(nx=4, ny=None, nz=None, box=((0.0, 1.0), (0.0, 1.0), (0.0, 1.0))):
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    xs = np.linspace(box[0][0], box[0][1], nx + 1)
    ys = np.linspace(box[1][0], box[1][1], ny + 1)
    zs = np.linspace(box[2][0], box[2][1], nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    base = (i + (nx + 1) * (j + (ny + 1) * k)).ravel()
    step = [1, nx + 1, (nx + 1) * (ny + 1)]
    v111 = base + sum(step)
    tets = []
    for perm in itertools.permutations(range(3)):
        a, b, _ = perm
        tets.append(np.stack([base, base + step[a], base + step[a] + step[b], v111], axis=1))
    el = np.stack(tets, axis=1).reshape(-1, 4)
    return Mesh(coords, el)

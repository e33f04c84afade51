"""Structured simplex meshes (the inputs ngsolve.meshes.MakeStructured2DMesh /
MakeStructured3DMesh provide to ngsxfem's tests and demos).

NGSolve's generators are not available, so the split pattern is this project's
own and is stated here:

* 2D: each quad (p00, p10, p11, p01) is split along the p00-p11 diagonal into
  the triangles (p00, p10, p11) and (p00, p11, p01).
* 3D: each cube is split into the 6 Kuhn (Freudenthal) tetrahedra
  [v000, v000+e_a, v000+e_a+e_b, v111] for the 6 permutations (a, b, c) of the
  axes, which is conforming across cubes.

With quads=True / hexes=True the cells are kept whole: a quadrilateral lists
its vertices (p00, p10, p11, p01), a hexahedron the same square at z0, then
at z1 (the corner order of cutint/straightcutrule.hpp:76-90).

Vertices are numbered with x fastest.  Arrays are numpy: coords (nv, dim)
float64, elements (ne, dim+1) int32 for simplices, (ne, 2^dim) for
quadrilaterals and hexahedra.
"""
import itertools

import numpy as np


class Mesh:
    """A mesh held on the host: vertex coordinates and element vertices, either
    simplices (trig / tet) or tensor cells (quad / hex)."""

    def __init__(self, coords, elements):
        self.coords = np.ascontiguousarray(coords, dtype=np.float64)
        self.elements = np.ascontiguousarray(elements, dtype=np.int32)
        self.dim = self.coords.shape[1]
        nve = self.elements.shape[1]
        if nve == self.dim + 1:
            self.tensor = False
        elif nve == 2 ** self.dim and self.dim in (2, 3):
            self.tensor = True
        else:
            raise ValueError("elements must be simplices (dim+1 vertices) or quads / hexes (2^dim vertices)")
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

    def boundary_elements(self):
        """The BND elements of a simplex mesh: the facets that belong to one
        element, each with its vertices ascending, in lexicographic order of
        those vertex tuples (the order libxg numbers its facets and BND
        elements in).  int32 array (nbnd, dim)."""
        if self.tensor:
            raise NotImplementedError("boundary elements of quadrilateral / hexahedral meshes")
        if getattr(self, "_bnd", None) is None:
            d = self.dim
            f = np.concatenate([np.delete(self.elements, s, axis=1) for s in range(d + 1)])
            f = np.sort(f, axis=1)
            u, cnt = np.unique(f, axis=0, return_counts=True)
            self._bnd = np.ascontiguousarray(u[cnt == 1], dtype=np.int32)
        return self._bnd

    def Boundaries(self, pattern):
        """Region of the BND elements on the named sides of the mesh's bounding
        box (a regular expression over the names, as NGSolve's
        mesh.Boundaries): in 2D bottom (y = ymin), right (x = xmax), top
        (y = ymax), left (x = xmin); in 3D left / right (x), front / back (y),
        bottom / top (z), the names of netgen's unit_square and unit_cube.  A
        BND element is on a side if all its vertices are."""
        import re
        names = (("left", 0, 0), ("right", 0, 1), ("bottom", 1, 0), ("top", 1, 1)) if self.dim == 2 else (
            ("left", 0, 0), ("right", 0, 1), ("front", 1, 0), ("back", 1, 1), ("bottom", 2, 0), ("top", 2, 1))
        bnd = self.boundary_elements()
        lo, hi = self.coords.min(axis=0), self.coords.max(axis=0)
        rx = re.compile(pattern)
        mask = np.zeros(len(bnd), dtype=bool)
        for name, axis, side in names:
            if rx.fullmatch(name):
                val = hi[axis] if side else lo[axis]
                mask |= np.all(self.coords[bnd, axis] == val, axis=1)
        return Region(self, mask)


class Region:
    """A set of BND elements of a mesh (mesh.Boundaries(...)): a boolean mask in
    the order of Mesh.boundary_elements."""

    def __init__(self, mesh, mask):
        self.mesh, self.mask = mesh, np.asarray(mask, dtype=bool)

    def Mask(self):
        return self.mask

    def __or__(self, o):
        return Region(self.mesh, self.mask | o.mask)

    def __and__(self, o):
        return Region(self.mesh, self.mask & o.mask)

    def __invert__(self):
        return Region(self.mesh, ~self.mask)


def MakeStructured2DMesh(nx=10, ny=10, xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0, quads=False):
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
    if quads:
        return Mesh(coords, np.stack([p00, p10, p11, p01], axis=1))
    t1 = np.stack([p00, p10, p11], axis=1)
    t2 = np.stack([p00, p11, p01], axis=1)
    el = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return Mesh(coords, el)


def MakeStructured3DMesh(nx=4, ny=None, nz=None, box=((0.0, 1.0), (0.0, 1.0), (0.0, 1.0)), hexes=False):
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
    if hexes:
        sx, sy, sz = step
        sq = [base, base + sx, base + sx + sy, base + sy]
        return Mesh(coords, np.stack(sq + [v + sz for v in sq], axis=1))
    tets = []
    for perm in itertools.permutations(range(3)):
        a, b, _ = perm
        tets.append(np.stack([base, base + step[a], base + step[a] + step[b], v111], axis=1))
    el = np.stack(tets, axis=1).reshape(-1, 4)
    return Mesh(coords, el)


def concatenate(meshes):
    """One mesh holding several independent meshes (vertex numbers offset), so a
    batch of meshes is assembled by one step; each component keeps its own
    dofs, rows and columns (the matrix is block diagonal)."""
    coords = np.concatenate([m.coords for m in meshes])
    off = np.cumsum([0] + [m.nv for m in meshes[:-1]])
    el = np.concatenate([m.elements + o for m, o in zip(meshes, off)])
    out = Mesh(coords, el)
    out.component_vertex_offsets = off
    out.component_element_counts = np.array([m.ne for m in meshes])
    return out


def replicated_circle_2d(copies, n=40, r=0.5):
    """`copies` replicas of [-1,1]^2 with n x n x 2 triangles and the level set
    sqrt(x^2+y^2) - r at the vertices (the 2D circle configuration)."""
    base = MakeStructured2DMesh(n, n, -1.0, 1.0, -1.0, 1.0)
    vals = np.sqrt(base.coords[:, 0] ** 2 + base.coords[:, 1] ** 2) - r
    m = concatenate([base] * copies)
    return m, np.tile(vals, copies)


def batched_ellipsoids(count=512, min_tets=1e3, max_tets=2e5, seed=20261203):
    """Independent unit-cube Kuhn meshes with log-uniform target sizes (the mesh
    with 6 n^3 tets closest to the target, n >= 6), each with a rotated ellipsoid
    level set (centre U[0.3,0.7]^3, semi-axes U[0.1,0.4], rotation = Q of a QR
    factorisation of a Gaussian 3x3 with sign-fixed diagonal) and an H1 order
    drawn from {1,2,3}.  Returns a list of (n, order, centre, semi-axes, rotation);
    `ellipsoid_values` turns one entry into vertex values."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        size = np.exp(rng.uniform(np.log(min_tets), np.log(max_tets)))
        n = max(6, int(round((size / 6.0) ** (1.0 / 3.0))))
        centre = rng.uniform(0.3, 0.7, 3)
        axes = rng.uniform(0.1, 0.4, 3)
        q, r = np.linalg.qr(rng.standard_normal((3, 3)))
        q = q * np.sign(np.diag(r))
        order = int(rng.integers(1, 4))
        out.append((n, order, centre, axes, q))
    return out


def ellipsoid_values(coords, centre, axes, rot):
    y = (coords - centre) @ rot
    return np.sqrt(((y / axes) ** 2).sum(axis=1)) - 1.0

"""Python surface of the cut-element path, shaped like ngsxfem's `xfem` module
(python/__init__.py, xfem/python_xfem.cpp, cutint/python_cutint.cpp) so that a
script written like demos/fictdom.py:95-133 keeps its structure:

    ci = CutInfo(mesh, lsetp1)
    hasneg = ci.GetElementsOfType(HASNEG)
    ba_facets = GetFacetsWithNeighborTypes(mesh, a=hasneg, b=ci.GetElementsOfType(IF))
    u, v = V.TnT()
    a = BilinearForm(V)
    a += grad(u) * grad(v) * dCut(lsetp1, NEG, definedonelements=hasneg)
    a += gamma / h**2 * (u - u.Other()) * (v - v.Other()) * dFacetPatch(definedonelements=ba_facets)
    a.Assemble()

Every operation runs on the GPU through libxg (include/xg.h); device memory is
held in torch tensors.  Integrands are parsed into the term menu of the C ABI
(mass, Laplace, Nitsche normal-derivative terms, convection, ghost-penalty
patch mass, and on interior facets the jump / average skeleton terms and
normal-derivative jumps of discontinuous-Galerkin forms, demos/fictdom_dg.py);
anything outside the menu raises.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .meshes import Mesh, MakeStructured2DMesh, MakeStructured3DMesh  # noqa: F401

NEG, POS, IF = 0, 1, 2
WHOLE = 3  # skeleton terms over the whole facet (dx(skeleton=True))
# direction policy of the quadrilateral / hexahedral cut rules
# (python/python_ngsxfem.cpp:35-37: FIRST_ALLOWED, FIND_OPTIMAL, ALWAYS_NONE)
FIRST, OPTIMAL, FALLBACK = 0, 1, 2
CDOM_NO, CDOM_NEG, CDOM_POS, CDOM_UNCUT, CDOM_IF, CDOM_HASNEG, CDOM_HASPOS, CDOM_ANY = range(8)
UNCUT, HASNEG, HASPOS, ANY = CDOM_UNCUT, CDOM_HASNEG, CDOM_HASPOS, CDOM_ANY
VOL, BND = "VOL", "BND"

TERM_MASS, TERM_LAPLACE, TERM_NGRADU_V, TERM_U_NGRADV, TERM_CONV, TERM_GHOST_MASS, TERM_DT_U_V = range(7)
TERM_SKEL_JUMP, TERM_SKEL_FLUX, TERM_SKEL_FLUX_T, TERM_SKEL_DN1, TERM_SKEL_DN2, TERM_SKEL_DN3 = range(7, 13)
TERM_NGRADU_NGRADV = 13
PREC_FP64, PREC_MIXED = 0, 1
XG_LTERM_SOURCE, XG_LTERM_SOURCE_GF, XG_LTERM_SOURCE_BND = 0, 1, 2


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev():
    if not torch.cuda.is_available():
        raise RuntimeError("ngsxfem_gb300 needs a CUDA device (GB300, sm_103a); there is no CPU path")
    return torch.device("cuda", torch.cuda.current_device())


# ----------------------------------------------------------------------------
# mesh / space / grid functions
# ----------------------------------------------------------------------------
class DeviceMesh:
    """libxg mesh handle (topology built once, resident on the device)."""

    def __init__(self, mesh):
        _dev()
        self.mesh = mesh
        h = ctypes.c_void_p()
        create = "xg_mesh_create_tensor" if getattr(mesh, "tensor", False) else "xg_mesh_create"
        _lib.call(create, mesh.dim, mesh.nv, mesh.coords.ctypes.data_as(ctypes.c_void_p), mesh.ne,
                  mesh.elements.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h))
        self.h = h
        info = np.zeros(6, dtype=np.int64)
        _lib.call("xg_mesh_info", self.h, info.ctypes.data_as(ctypes.c_void_p))
        self.dim, self.nv, self.ne, self.nedges, self.nfaces, self.nfacets = (int(x) for x in info)

    def facet_elements(self):
        out = np.zeros((self.nfacets, 2), dtype=np.int32)
        _lib.call("xg_mesh_facet_elements", self.h, out.ctypes.data_as(ctypes.c_void_p))
        return out

    def check(self):
        torch.cuda.synchronize()
        _lib.check(_lib.load().xg_mesh_check(self.h), "device (mesh)")

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib.load().xg_mesh_destroy(self.h)
            self.h = None


def device_mesh(mesh):
    if getattr(mesh, "_device", None) is None:
        mesh._device = DeviceMesh(mesh)
    return mesh._device


class BitArray:
    """Bit set on the device: bit i of 64-bit word i//64 (int64 storage)."""

    def __init__(self, n, words=None):
        self.n = int(n)
        nw = (self.n + 63) // 64
        self.words = words if words is not None else torch.zeros(nw, dtype=torch.int64, device=_dev())

    def __len__(self):
        return self.n

    def numpy(self):
        w = self.words.cpu().numpy().view(np.uint64)
        bits = np.unpackbits(w.view(np.uint8), bitorder="little")
        return bits[: self.n].astype(bool)

    def NumSet(self):
        return int(self.numpy().sum())

    def __getitem__(self, i):
        return bool((int(self.words[i // 64].item()) >> (i % 64)) & 1)

    def _mask(self):
        extra = self.words.numel() * 64 - self.n
        m = torch.full_like(self.words, -1)
        if extra:
            m[-1] = (1 << (64 - extra)) - 1
        return m

    def __or__(self, o):
        return BitArray(self.n, self.words | o.words)

    def __and__(self, o):
        return BitArray(self.n, self.words & o.words)

    def __invert__(self):
        return BitArray(self.n, (~self.words) & self._mask())

    @staticmethod
    def from_bool(mask):
        """Packs a device bool tensor into a BitArray on the same device."""
        n = int(mask.numel())
        pad = (-n) % 64
        m = torch.cat([mask.reshape(-1).to(torch.int64), torch.zeros(pad, dtype=torch.int64, device=mask.device)])
        weights = torch.ones(64, dtype=torch.int64, device=mask.device) << torch.arange(64, device=mask.device)
        # distinct bits: the sum is the OR (bit 63 wraps to the sign bit)
        return BitArray(n, (m.reshape(-1, 64) * weights).sum(dim=1))

    def bool_tensor(self):
        """The bits as a device bool tensor of length n."""
        i = torch.arange(self.n, device=self.words.device)
        return ((self.words[i >> 6] >> (i & 63)) & 1).bool()

    @staticmethod
    def from_numpy(bits):
        bits = np.asarray(bits, dtype=bool)
        n = bits.size
        packed = np.packbits(bits, bitorder="little")
        pad = (-packed.size) % 8
        packed = np.concatenate([packed, np.zeros(pad, np.uint8)]).view(np.int64)
        return BitArray(n, torch.from_numpy(packed.copy()).to(_dev()))


class H1:
    """H1 space of order 1..3 on a simplex mesh (libxg dof numbering); on a
    quadrilateral / hexahedral mesh order 1 only (the vertex values of a
    bilinear / trilinear level set), which the cut rules and Integrate use."""

    def __init__(self, mesh, order=1, dgjumps=False, **kwargs):
        self.mesh = mesh
        self.order = int(order)
        self.dm = device_mesh(mesh)
        if getattr(mesh, "tensor", False):
            if self.order != 1:
                raise ValueError("H1 on quadrilateral / hexahedral meshes: order 1 only")
            self.h = None
            self.ndof, self.ndof_el = mesh.nv, mesh.elements.shape[1]
            return
        h = ctypes.c_void_p()
        _lib.call("xg_space_create", self.dm.h, self.order, ctypes.byref(h))
        self.h = h
        info = np.zeros(3, dtype=np.int64)
        _lib.call("xg_space_info", self.h, info.ctypes.data_as(ctypes.c_void_p))
        self.ndof, self.ndof_el = int(info[0]), int(info[1])

    def element_dofs(self):
        if self.h is None:
            return self.mesh.elements.copy()
        out = np.zeros((self.mesh.ne, self.ndof_el), dtype=np.int32)
        _lib.call("xg_space_element_dofs", self.h, out.ctypes.data_as(ctypes.c_void_p))
        return out

    def TrialFunction(self):
        return _Expr.atom(("u", False))

    def TestFunction(self):
        return _Expr.atom(("v", False))

    def TnT(self):
        return self.TrialFunction(), self.TestFunction()

    def FreeDofs(self, coupling=False):
        """All dofs, or those of the active elements of a Restrict(...) view
        (no Dirichlet dofs: boundary conditions are imposed weakly)."""
        active = getattr(self, "_active_elements", None)
        if active is None:
            return BitArray.from_bool(torch.ones(self.ndof, dtype=torch.bool, device=_dev()))
        return GetDofsOfElements(self, active)

    def _element_dofs_device(self):
        if getattr(self, "_el_dofs_dev", None) is None:
            self._el_dofs_dev = torch.from_numpy(self.element_dofs().astype(np.int64)).to(_dev())
        return self._el_dofs_dev

    def __del__(self):
        # a Restrict(...) view shares the handle of the space it was made from
        if getattr(self, "h", None) and getattr(self, "_owner", True) and _lib._lib is not None:
            _lib.load().xg_space_destroy(self.h)
            self.h = None


class L2(H1):
    """Discontinuous space L2(mesh, order, dgjumps=True) of order 1..3 on a
    simplex mesh: the H1 element basis with element-local dofs,
    dof(e, i) = e * ndof_per_element + i (xg_space_create_l2)."""

    def __init__(self, mesh, order=1, dgjumps=True, **kwargs):
        self.mesh = mesh
        self.order = int(order)
        self.dm = device_mesh(mesh)
        if getattr(mesh, "tensor", False):
            raise NotImplementedError("L2 spaces are built on simplex meshes")
        h = ctypes.c_void_p()
        _lib.call("xg_space_create_l2", self.dm.h, self.order, ctypes.byref(h))
        self.h = h
        info = np.zeros(3, dtype=np.int64)
        _lib.call("xg_space_info", self.h, info.ctypes.data_as(ctypes.c_void_p))
        self.ndof, self.ndof_el = int(info[0]), int(info[1])


class ScalarTimeFE:
    """Nodal time finite element on [0, 1] with Gauss-Lobatto nodes
    (spacetime/python_spacetime.cpp:156, SpaceTimeFE.cpp:263-281): order 1
    nodes {0, 1}, order 2 nodes {0, 1/2, 1}."""

    def __init__(self, order=0, skip_first_nodes=False, only_first_nodes=False, **kwargs):
        if skip_first_nodes or only_first_nodes or kwargs.get("skip_first_node") or kwargs.get("only_first_node"):
            raise NotImplementedError("restricted time elements are not part of the GPU path")
        self.order = int(order)

    def __mul__(self, fes):
        return SpaceTimeFESpace(fes, self)

    __rmul__ = __mul__


class SpaceTimeFESpace:
    """Tensor product of an H1 space (order 1..2) and a ScalarTimeFE (order
    1..2); dof (time dof i, space dof j) -> i * ndof_space + j."""

    def __init__(self, spacefes, timefe, dirichlet=None, **kwargs):
        self.base, self.tfe = spacefes, timefe
        self.mesh = spacefes.mesh
        self.order, self.order_time = spacefes.order, timefe.order
        self.dm = device_mesh(self.mesh)
        h = ctypes.c_void_p()
        _lib.call("xg_space_create_st", self.dm.h, self.order, self.order_time, ctypes.byref(h))
        self.h = h
        info = np.zeros(6, dtype=np.int64)
        _lib.call("xg_space_info_st", self.h, info.ctypes.data_as(ctypes.c_void_p))
        self.ndof, self.ndof_el, _, _, self.ndof_space, self.ndof_el_space = (int(v) for v in info)

    def TrialFunction(self):
        return _Expr.atom(("u", False))

    def TestFunction(self):
        return _Expr.atom(("v", False))

    def TnT(self):
        return self.TrialFunction(), self.TestFunction()

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib.load().xg_space_destroy(self.h)
            self.h = None


def _time_nodes(k):
    return [0.0] if k == 0 else ([0.0, 1.0] if k == 1 else [0.0, 0.5, 1.0])


def SpaceTimeInterpolateToP1(spacetime_cf, time=None, spacetime_gf=None, t0=0.0, dt=1.0, eps_perturbation=1e-14):
    """Nodal in time, P1 in space (spacetime/python_spacetime.cpp:438): the
    callable spacetime_cf(x, y[, z], t) at the vertices and the time nodes
    t = t0 + dt * tau_i of the GridFunction's space-time P1 space, with
    InterpolateToP1's |v| < eps -> eps perturbation on the device."""
    gf = spacetime_gf
    V = gf.space
    if not isinstance(V, SpaceTimeFESpace) or V.order != 1:
        raise TypeError("spacetime_gf must be a GridFunction of a P1 x P_k space-time space")
    mesh = V.mesh
    coords = [mesh.coords[:, k] for k in range(mesh.dim)]
    vals = np.concatenate([np.asarray(spacetime_cf(*coords, t0 + dt * tau), dtype=np.float64)
                           for tau in _time_nodes(V.order_time)])
    gf.vec.copy_(torch.from_numpy(np.ascontiguousarray(vals)))
    _lib.call("xg_interpolate_p1_perturb", _vp(gf.vec), gf.vec.numel(), eps_perturbation, _stream())
    return gf


def dtref(func):
    """Time derivative on the reference time interval (python/__init__.py:129)."""
    if isinstance(func, _Expr) and len(func.monos) == 1 and func.monos[0].scal == (("u", False),):
        return _Expr([_Mono(c=func.monos[0].c, scal=(("dtu", False),))])
    raise TypeError("dtref() of the space-time trial function only")


class TimeVector:
    """Convection field b(t) = b + bc cos(omega t) + bs sin(omega t) with
    t = t0 + dt * tau on the slab (the time-dependent CoefficientFunction of
    the space-time demo, reduced to what the GPU kernels evaluate)."""

    def __init__(self, b=(0.0, 0.0, 0.0), bc=(0.0, 0.0, 0.0), bs=(0.0, 0.0, 0.0), omega=0.0, t0=0.0, dt=1.0):
        pad = lambda v: tuple(float(a) for a in v) + (0.0,) * (3 - len(v))  # noqa: E731
        self.key = (pad(b), pad(bc), pad(bs), float(omega), float(t0), float(dt))

    def _expr(self):
        return _Expr([_Mono(vec=("tb", self.key))])


class GridFunction:
    def __init__(self, space):
        self.space = space
        self.vec = torch.zeros(space.ndof, dtype=torch.float64, device=_dev())

    def Set(self, f):
        """Interpolation of f(x, y[, z]) (vectorised over numpy arrays) into the
        H1 / L2 space of order 1..3: the function's values at the canonical
        nodes of every element (vertices; edge midpoints for order 2; edge
        points at 1/3, 2/3 and face centroids for order 3) give the
        hierarchical coefficients (the relations of csrc/xg_patch.cuh
        nodal_to_hier), with the cubic edge functions oriented by global vertex
        numbers.  Exact for polynomials of the space's degree."""
        V = self.space
        mesh, k = V.mesh, V.order
        if isinstance(V, SpaceTimeFESpace) or getattr(mesh, "tensor", False):
            raise NotImplementedError("Set on simplex H1 / L2 spaces")
        D = mesh.dim
        X = mesh.coords[mesh.elements]                      # ne x (D+1) x D
        ev = lambda P: np.asarray(f(*[P[..., c] for c in range(D)]), dtype=np.float64)  # noqa: E731
        cols = [ev(X[:, i]) for i in range(D + 1)]
        edges = [(0, 1), (0, 2), (1, 2)] if D == 2 else [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
        alpha = {}
        if k >= 2:
            gv = mesh.elements
            for j, (a, b) in enumerate(edges):
                pa, pb = cols[a], cols[b]
                if k == 2:
                    al = 4 * ev(0.5 * (X[:, a] + X[:, b])) - 2 * (pa + pb)
                    cols.append(al)
                else:
                    q1 = ev(X[:, a] / 3 + 2 * X[:, b] / 3) - (pa + 2 * pb) / 3
                    q2 = ev(2 * X[:, a] / 3 + X[:, b] / 3) - (2 * pa + pb) / 3
                    al = 2.25 * (q1 + q2)
                    sign = np.where(gv[:, a] < gv[:, b], 1.0, -1.0)
                    cols += [al, 6.75 * (q2 - q1) * sign]
                alpha[(a, b)] = al
        if k == 3:
            faces = [(0, 1, 2)] if D == 2 else [(0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)]
            for a, b, c in faces:
                cen = ev((X[:, a] + X[:, b] + X[:, c]) / 3)
                e = alpha[(a, b)] + alpha[(a, c)] + alpha[(b, c)]
                cols.append(27 * (cen - (cols[a] + cols[b] + cols[c]) / 3 - e / 9))
        loc = np.stack(cols, 1)
        out = np.zeros(V.ndof)
        out[V.element_dofs()] = loc
        self.vec.copy_(torch.from_numpy(out))
        return self

    def _atom(self):
        return _Expr([_Mono(scal=(("gf", self),))])

    def __mul__(self, o):
        if isinstance(o, (_Expr, int, float, _Measure, GridFunction, _Monomial)):
            return self._atom() * o
        return NotImplemented

    def __rmul__(self, o):
        if isinstance(o, (_Expr, int, float, GridFunction, _Monomial)):
            return _Expr.wrap(o) * self._atom()
        return NotImplemented

    # coefficient-function arithmetic (integrands of Integrate and forms)
    def __add__(self, o):
        return self._atom() + o

    __radd__ = __add__

    def __sub__(self, o):
        return self._atom() - o

    def __rsub__(self, o):
        return _Expr.wrap(o) - self._atom()

    def __neg__(self):
        return -self._atom()

    def __pow__(self, p):
        return self._atom() ** p


def GetDofsOfElements(space, a, heapsize=None):
    """The dofs of the elements in the BitArray a (the reference's
    GetDofsOfElements), marked on the device from the space's element-dof
    table."""
    el = space._element_dofs_device()
    if a.n != el.shape[0]:
        raise ValueError("the BitArray must have one bit per element of the space's mesh")
    mask = torch.zeros(space.ndof, dtype=torch.bool, device=_dev())
    mask[el[a.bool_tensor()].reshape(-1)] = True
    return BitArray.from_bool(mask)


def Restrict(space, active_elements):
    """A view of the space whose FreeDofs() are the dofs of the active
    elements (the reference's Restrict(fes, ba)).  The dof numbering stays
    the space's: the assembled matrix holds the rows of the active elements
    only, and FreeDofs() selects them for a solver."""
    if not isinstance(space, H1) or getattr(space, "h", None) is None:
        raise NotImplementedError("Restrict / Compress of spatial H1 / L2 spaces on simplex meshes")
    view = object.__new__(type(space))
    view.__dict__.update(space.__dict__)
    view._base, view._owner, view._active_elements = space, False, active_elements
    return view


def Compress(space, active_dofs):
    """Compress(fes, GetDofsOfElements(fes, ba)): the space with FreeDofs() =
    active_dofs (numbering kept, as Restrict)."""
    view = Restrict(space, None)
    view.FreeDofs = lambda coupling=False: active_dofs
    return view


def InterpolateToP1(f, gf, eps_perturbation=1e-14):
    """Vertex values of f (callable on coordinate arrays, or an array of vertex
    values) into the P1 GridFunction gf, with ngsxfem's |v| < eps -> eps
    perturbation (utils/p1interpol.cpp:104-107) applied on the device."""
    mesh = gf.space.mesh
    if callable(f):
        vals = np.asarray(f(*[mesh.coords[:, k] for k in range(mesh.dim)]), dtype=np.float64)
    else:
        vals = np.asarray(f, dtype=np.float64)
    gf.vec[: mesh.nv].copy_(torch.from_numpy(np.ascontiguousarray(vals)))
    _lib.call("xg_interpolate_p1_perturb", _vp(gf.vec), mesh.nv, eps_perturbation, _stream())
    return gf


def _lset_vec(levelset):
    if isinstance(levelset, GridFunction):
        if isinstance(levelset.space, SpaceTimeFESpace):
            if levelset.space.order != 1:
                raise ValueError("space-time level sets are P1 in space")
            return levelset.vec
        if levelset.space.order != 1:
            raise ValueError("the straight-cut path needs a P1 level set (CF2GFForStraightCutRule)")
        return levelset.vec
    if isinstance(levelset, torch.Tensor):
        return levelset
    raise TypeError("level set must be a P1 GridFunction or a device tensor of vertex values")


# ----------------------------------------------------------------------------
# marking
# ----------------------------------------------------------------------------
class CutInfo:
    """CutInformation (xfem/cutinfo.cpp:61-284): element domain types, cut ratios
    and the combined-domain bitsets of a P1 level set on the VOL and BND
    elements (BND elements: the boundary facets in facet order), the
    cut-neighbouring nodes and the domain type of every node."""

    def __init__(self, mesh, levelset=None, subdivlvl=0, time_order=-1, heapsize=None):
        self.mesh = mesh
        self.dm = device_mesh(mesh)
        ne = mesh.ne
        dev = _dev()
        nb = np.zeros(1, dtype=np.int64)
        _lib.call("xg_mesh_boundary", self.dm.h, nb.ctypes.data_as(ctypes.c_void_p), None)
        self.nbnd = int(nb[0])
        self.dom = torch.zeros(ne, dtype=torch.uint8, device=dev)
        self.cut_ratio = torch.zeros(ne, dtype=torch.float64, device=dev)
        self.bits = torch.zeros((8, (ne + 63) // 64), dtype=torch.int64, device=dev)
        self.dom_bnd = torch.zeros(max(self.nbnd, 1), dtype=torch.uint8, device=dev)
        self.cut_ratio_bnd = torch.zeros(max(self.nbnd, 1), dtype=torch.float64, device=dev)
        self.bits_bnd = torch.zeros((8, (self.nbnd + 63) // 64 or 1), dtype=torch.int64, device=dev)
        dm = self.dm
        w = lambda n: torch.zeros(max((n + 63) // 64, 1), dtype=torch.int64, device=dev)  # noqa: E731
        self.cut_nb_nodes = {"vertex": w(dm.nv), "edge": w(dm.nedges), "face": w(dm.nfaces), "element": w(ne)}
        self.dom_of_node = {"vertex": torch.zeros(dm.nv, dtype=torch.uint8, device=dev),
                            "edge": torch.zeros(dm.nedges, dtype=torch.uint8, device=dev),
                            "face": torch.zeros(max(dm.nfaces, 1), dtype=torch.uint8, device=dev),
                            "cell": torch.zeros(ne, dtype=torch.uint8, device=dev)}
        self.levelset = None
        if levelset is not None:
            self.Update(levelset, subdivlvl, time_order)

    def Update(self, levelset, subdivlvl=0, time_order=-1, heapsize=None):
        if subdivlvl != 0 or time_order > 0:
            raise NotImplementedError("CutInfo on the GPU supports P1 level sets (subdivlvl=0, time_order<=0)")
        self.levelset = levelset
        lv = _lset_vec(levelset)
        if isinstance(levelset, GridFunction) and isinstance(levelset.space, SpaceTimeFESpace):
            # space-time prisms (time_order = 0): CutInformation::Update with the
            # space-time cut rule of orders 0/0
            _lib.call("xg_cutinfo_update_st", self.dm.h, _vp(lv), levelset.space.order_time, _vp(self.dom),
                      _vp(self.cut_ratio), _vp(self.bits), _stream())
            return
        _lib.call("xg_cutinfo_update", self.dm.h, _vp(lv), _vp(self.dom), _vp(self.cut_ratio), _vp(self.bits),
                  _stream())
        if getattr(self.mesh, "tensor", False):
            return  # quadrilaterals / hexahedra: the element part only
        if self.nbnd:
            _lib.call("xg_cutinfo_update_bnd", self.dm.h, _vp(lv), _vp(self.dom_bnd), _vp(self.cut_ratio_bnd),
                      _vp(self.bits_bnd), _stream())
        nb, dn = self.cut_nb_nodes, self.dom_of_node
        three = self.mesh.dim == 3
        _lib.call("xg_cutinfo_nodes", self.dm.h, _vp(self.dom), _vp(self.cut_ratio), _vp(nb["vertex"]),
                  _vp(nb["edge"]), _vp(nb["face"]) if three else None, _vp(nb["element"]), _vp(dn["vertex"]),
                  _vp(dn["edge"]), _vp(dn["face"]) if three else None, _vp(dn["cell"]), _stream())

    @staticmethod
    def _cdt(domain_type):
        return {NEG: CDOM_NEG, POS: CDOM_POS, IF: CDOM_IF}.get(domain_type, domain_type) \
            if isinstance(domain_type, int) and domain_type < 3 else domain_type

    def GetElementsOfType(self, domain_type=IF, VorB=VOL):
        cdt = self._cdt(domain_type)
        if VorB == BND:
            return BitArray(self.nbnd, self.bits_bnd[cdt].clone())
        return BitArray(self.mesh.ne, self.bits[cdt].clone())

    def GetCutRatios(self, VorB=VOL):
        return self.cut_ratio_bnd[: self.nbnd] if VorB == BND else self.cut_ratio

    def GetElementsWithThresholdContribution(self, domain_type=NEG, threshold=1.0, VorB=VOL):
        if domain_type not in (NEG, POS):
            raise ValueError("Unknown/Invalid type for dt: Only POS, NEG are implemented a.t.m.")
        ratio = self.GetCutRatios(VorB)
        n = self.nbnd if VorB == BND else self.mesh.ne
        out = BitArray(n)
        _lib.call("xg_elements_with_threshold", _vp(ratio), n, domain_type, float(threshold), _vp(out.words),
                  _stream())
        return out

    def GetCutNeighboringNodes(self, node_type="vertex"):
        """Nodes of cut elements (cut_neighboring_node of CutInformation)."""
        if getattr(self.mesh, "tensor", False):
            raise NotImplementedError("node markers are built for simplex meshes")
        n = {"vertex": self.dm.nv, "edge": self.dm.nedges, "face": self.dm.nfaces, "element": self.mesh.ne}[node_type]
        return BitArray(n, self.cut_nb_nodes[node_type].clone())

    def GetDomainOfNodes(self, node_type="vertex"):
        """Domain type (NEG/POS) of every node (dom_of_node of CutInformation)."""
        if getattr(self.mesh, "tensor", False):
            raise NotImplementedError("node markers are built for simplex meshes")
        n = {"vertex": self.dm.nv, "edge": self.dm.nedges, "face": self.dm.nfaces, "cell": self.mesh.ne}[node_type]
        return self.dom_of_node[node_type][:n]

    def Mesh(self):
        return self.mesh


def GetFacetsWithNeighborTypes(mesh, a, bnd_val_a=True, bnd_val_b=True, use_and=True, b=None, heapsize=None):
    dm = device_mesh(mesh)
    b = a if b is None else b
    out = BitArray(dm.nfacets)
    _lib.call("xg_facets_with_neighbor_types", dm.h, _vp(a.words), _vp(b.words), int(bnd_val_a), int(bnd_val_b),
              int(use_and), _vp(out.words), _stream())
    return out


def GetElementsWithNeighborFacets(mesh, a, heapsize=None):
    dm = device_mesh(mesh)
    out = BitArray(mesh.ne)
    _lib.call("xg_elements_with_neighbor_facets", dm.h, _vp(a.words), _vp(out.words), _stream())
    return out


# ----------------------------------------------------------------------------
# integrands
# ----------------------------------------------------------------------------
class _Mono:
    """c * h^hpow * (scalar atoms) * (dot products) * (at most one free vector)."""
    __slots__ = ("c", "hpow", "scal", "dots", "vec")

    def __init__(self, c=1.0, hpow=0, scal=(), dots=(), vec=None):
        self.c, self.hpow, self.scal, self.dots, self.vec = c, hpow, tuple(scal), tuple(dots), vec

    def mul(self, o):
        vec, dots = None, self.dots + o.dots
        if self.vec is not None and o.vec is not None:
            dots = dots + (tuple(sorted((self.vec, o.vec), key=repr)),)
        else:
            vec = self.vec if self.vec is not None else o.vec
        return _Mono(self.c * o.c, self.hpow + o.hpow, tuple(sorted(self.scal + o.scal, key=repr)), dots, vec)


class _Expr:
    def __init__(self, monos):
        self.monos = monos

    @staticmethod
    def atom(a, vector=False):
        return _Expr([_Mono(vec=a)] if vector else [_Mono(scal=(a,))])

    @staticmethod
    def wrap(x):
        if isinstance(x, _Expr):
            return x
        if isinstance(x, (int, float)):
            return _Expr([_Mono(c=float(x))])
        if isinstance(x, GridFunction):
            return x._atom()
        if isinstance(x, TimeVector):
            return x._expr()
        if isinstance(x, _Monomial):
            return _Expr([_Mono(scal=(("xyz", x.e),))])
        if isinstance(x, (tuple, list)):
            if all(isinstance(v, (int, float)) for v in x):
                return _Expr([_Mono(vec=("b", tuple(float(v) for v in x)))])
            # a vector with coefficient-field components, e.g.
            # CoefficientFunction((gf_x, gf_y)): the sum of its components
            # times the unit vectors (the constant components as one vector)
            const = [float(v) if isinstance(v, (int, float)) else 0.0 for v in x]
            monos = [_Mono(vec=("b", tuple(const)))] if any(const) else []
            for i, v in enumerate(x):
                if isinstance(v, (int, float)):
                    continue
                unit = tuple(1.0 if j == i else 0.0 for j in range(len(x)))
                for m in _Expr.wrap(v).monos:
                    if m.vec is not None or m.dots or any(a[0] not in ("gf", "xyz") for a in m.scal):
                        raise TypeError("vector components: numbers, GridFunctions, x, y, z and their products")
                    monos.append(_Mono(m.c, m.hpow, m.scal, (), ("b", unit)))
            return _Expr(monos)
        raise TypeError("unsupported coefficient %r" % (x,))

    def __add__(self, o):
        return _Expr(self.monos + _Expr.wrap(o).monos)

    __radd__ = __add__

    def __neg__(self):
        return _Expr([_Mono(-m.c, m.hpow, m.scal, m.dots, m.vec) for m in self.monos])

    def __sub__(self, o):
        return self + (-_Expr.wrap(o))

    def __rsub__(self, o):
        return _Expr.wrap(o) - self

    def __mul__(self, o):
        if isinstance(o, _Measure):
            return _Integral(self, o)
        o = _Expr.wrap(o)
        return _Expr([a.mul(b) for a in self.monos for b in o.monos])

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = _Expr.wrap(o)
        if len(o.monos) != 1 or o.monos[0].scal or o.monos[0].dots or o.monos[0].vec is not None:
            raise TypeError("can only divide by constants and powers of the mesh size")
        m = o.monos[0]
        return self * _Expr([_Mono(1.0 / m.c, -m.hpow)])

    def __rtruediv__(self, o):
        if len(self.monos) != 1 or self.monos[0].scal or self.monos[0].dots or self.monos[0].vec is not None:
            raise TypeError("can only divide by constants and powers of the mesh size")
        m = self.monos[0]
        return _Expr.wrap(o) * _Expr([_Mono(1.0 / m.c, -m.hpow)])

    def __pow__(self, p):
        if int(p) != p:
            raise TypeError("integer powers only")
        if len(self.monos) == 1 and not self.monos[0].scal and self.monos[0].vec is None and not self.monos[0].dots:
            m = self.monos[0]
            return _Expr([_Mono(m.c ** p, m.hpow * int(p))])
        if p < 1:
            raise TypeError("powers >= 1 of expressions with coefficient fields")
        out = self
        for _ in range(int(p) - 1):
            out = out * self
        return out

    def Other(self):
        out = []
        for m in self.monos:
            scal = tuple(((a[0], True) + tuple(a[2:])) if a[0] in ("u", "v", "dnu", "dnv") else a for a in m.scal)
            vec = m.vec
            if vec is not None and vec[0] in ("gu", "gv"):
                vec = (vec[0], True)
            out.append(_Mono(m.c, m.hpow, scal, m.dots, vec))
        return _Expr(out)


def grad(x):
    if isinstance(x, GridFunction):
        return _LsetGrad(x)
    if isinstance(x, _Expr) and len(x.monos) == 1 and len(x.monos[0].scal) == 1 and x.monos[0].scal[0][0] in ("u", "v"):
        return _Expr([_Mono(vec=("g" + x.monos[0].scal[0][0], x.monos[0].scal[0][1]))])
    raise TypeError("grad() of a trial/test function or a P1 level set GridFunction only")


def InnerProduct(a, b):
    return _Expr.wrap(a) * _Expr.wrap(b)


def dn(proxy, order, comp=-1, hdiv=False):
    """k-th derivative of a trial / test function along the outward unit normal
    of the facet's element it lives on (python_xfem.cpp:1068-1150, DiffOpDuDnk):
    for u.Other() that is the second element's normal, so the jump across a
    facet is dn(u, k) - (-1)^k dn(u.Other(), k).  Skeleton integrals only."""
    if comp != -1 or hdiv:
        raise NotImplementedError("dn of scalar H1 / L2 functions only")
    if not (isinstance(proxy, _Expr) and len(proxy.monos) == 1 and len(proxy.monos[0].scal) == 1
            and proxy.monos[0].scal[0][0] in ("u", "v") and proxy.monos[0].c == 1.0):
        raise TypeError("dn() of a trial or test function (or its .Other())")
    name, other = proxy.monos[0].scal[0][:2]
    if not 1 <= int(order) <= 3:
        raise NotImplementedError("dn of order 1..3")
    return _Expr([_Mono(scal=(("dn" + name, other, int(order)),))])


class _LsetGrad(_Expr):
    """grad(gf) of a GridFunction: a vector expression (Integrate's H1 errors,
    (grad(gfu) - grad(gfex)) ** 2); Normalize(grad(lset)) is the level set's
    unit normal."""

    def __init__(self, gf):
        super().__init__([_Mono(vec=("ggf", gf))])
        self.gf = gf


def Normalize(g):
    if isinstance(g, _LsetGrad):
        return _Expr([_Mono(vec=("n", id(g.gf)))])
    raise TypeError("Normalize(grad(lset)) only")


class _SpecialCF:
    @property
    def mesh_size(self):
        return _Expr([_Mono(hpow=1)])

    def normal(self, dim=None):
        """Unit normal of a facet, out of the facet's first element (skeleton
        integrals)."""
        return _Expr([_Mono(vec=("nF", None))])


specialcf = _SpecialCF()


def CoefficientFunction(x):
    return _Expr.wrap(x)


class _Measure:
    def __init__(self, kind, levelset=None, domain_type=None, order=None, definedonelements=None, **kw):
        self.kind, self.levelset, self.domain_type, self.order = kind, levelset, domain_type, order
        self.definedonelements = definedonelements
        self.scale = 1.0
        self.skeleton = bool(kw.get("skeleton", False))
        if self.skeleton and kind not in ("cut", "skel"):
            raise NotImplementedError("skeleton=True applies to dCut and dx")
        if self.skeleton and kind == "cut" and domain_type not in (NEG, POS):
            raise NotImplementedError("dCut(..., skeleton=True) on NEG or POS (codim-2 skeleton rules are not built)")
        for k in ("element_boundary", "element_vb"):
            if kw.get(k) is not None and kw.get(k) is not False:
                raise NotImplementedError("dCut/dFacetPatch option %r is not part of the GPU path" % k)
        self.deformation = kw.get("deformation")
        if self.deformation is not None:
            if kind not in ("cut", "patch", "vol") or not isinstance(self.deformation, LevelSetMeshAdaptation):
                raise NotImplementedError("deformation: dCut / dFacetPatch / dx(..., deformation="
                                          "LevelSetMeshAdaptation(..).CalcDeformation(..))")
        self.definedon = kw.get("definedon")
        if self.definedon is not None and (kind != "cut" or kw.get("vb", VOL) != BND):
            raise NotImplementedError("definedon (a region of BND elements) applies to dCut(..., vb=BND)")
        self.subdivlvl = int(kw.get("subdivlvl") or 0)
        t = kw.get("time_order", -1)
        self.time_order = -1 if t is None else int(t)
        self.tref = kw.get("tref")
        self.quad_dir_policy = int(kw.get("quad_dir_policy", OPTIMAL))
        self.vb = kw.get("vb", VOL)
        if kw.get("downscale", 1.0) != 1.0:
            raise NotImplementedError("downscale != 1 is not supported")

    def __rmul__(self, c):
        """delta_t * dCut(...): a measure scaled by a number."""
        if not isinstance(c, (int, float)):
            return NotImplemented
        out = _Measure.__new__(_Measure)
        out.__dict__.update(self.__dict__)
        out.scale = self.scale * float(c)
        return out


def dCut(levelset, domain_type, order=None, subdivlvl=None, time_order=-1, levelset_domain=None, **kwargs):
    """Differential symbol for cut integration (python/__init__.py:781-864)."""
    if levelset_domain is not None:
        levelset = levelset_domain["levelset"]
        domain_type = levelset_domain["domain_type"]
        order = levelset_domain.get("order", order)
        if "quad_dir_policy" in levelset_domain:
            kwargs.setdefault("quad_dir_policy", levelset_domain["quad_dir_policy"])
    return _Measure("cut", levelset, domain_type, order, kwargs.pop("definedonelements", None),
                    subdivlvl=subdivlvl, time_order=time_order, **kwargs)


def dx(skeleton=False, definedonelements=None, **kwargs):
    """Whole-element integrals (the element's own rule, cut or not) on the
    elements of definedonelements (all without it), e.g. TraceFEM's normal
    diffusion (grad(u) * n) * (grad(v) * n) * dx(definedonelements=ba_IF,
    deformation=...) in a BilinearForm with dCut terms of the same level set;
    with skeleton=True whole-facet skeleton integrals
    (SymbolicFacetBilinearFormIntegrator2, symboliccutbfi.cpp:1574-1735), e.g.
    the derivative-jump ghost penalty dn-jumps * dx(skeleton=True,
    definedonelements=ghost_facets)."""
    if not skeleton:
        return _Measure("vol", None, WHOLE, kwargs.pop("order", None), definedonelements, **kwargs)
    return _Measure("skel", None, WHOLE, kwargs.pop("order", None), definedonelements, skeleton=True, **kwargs)


def dFacetPatch(**kwargs):
    """Differential symbol for facet patch integrators (python/__init__.py:749-778)."""
    return _Measure("patch", None, None, kwargs.pop("order", None), kwargs.pop("definedonelements", None), **kwargs)


class _Integral:
    def __init__(self, expr, measure):
        self.expr, self.measure = expr, measure

    def __add__(self, o):
        return _SumOfIntegrals([self]) + o

    def terms(self, nrm_gf):
        """Maps the integrand onto the C ABI term menu (list of dicts)."""
        m = self.measure
        if getattr(m, "subdivlvl", 0):
            raise NotImplementedError("bilinear forms on subdivision rules (subdivlvl > 0) are not built; "
                                      "Integrate takes them")
        out = []
        if m.kind == "patch":
            # expect c * (u - u')(v - v') = c*(uv - u'v - uv' + u'v')
            for mono in self.expr.monos:
                if mono.dots or mono.vec is not None or len(mono.scal) != 2:
                    raise NotImplementedError("facet patch integrands: c * (u - u.Other()) * (v - v.Other()) only")
            sign = {(("u", False), ("v", False)): 1, (("u", True), ("v", False)): -1,
                    (("u", False), ("v", True)): -1, (("u", True), ("v", True)): 1}
            acc = {}
            for mono in self.expr.monos:
                key = tuple(sorted(mono.scal, key=repr))
                if key not in sign:
                    raise NotImplementedError("facet patch integrand outside the ghost-penalty form")
                acc.setdefault((key, mono.hpow), 0.0)
                acc[(key, mono.hpow)] += mono.c
            # one ghost-penalty term per power of the mesh size
            for hp in sorted({k[1] for k in acc}):
                vals = {k[0]: v for k, v in acc.items() if k[1] == hp}
                c_uv = vals.get((("u", False), ("v", False)), 0.0)
                for key, sgn in sign.items():
                    if abs(vals.get(key, 0.0) - sgn * c_uv) > 1e-14 * max(1.0, abs(c_uv)):
                        raise NotImplementedError("facet patch integrand is not c*(u-u.Other())*(v-v.Other())")
                out.append(dict(kind=TERM_GHOST_MASS, domain=NEG, order=-1 if m.order is None else m.order,
                                hpow=hp, coef=c_uv * m.scale, b=(0.0, 0.0, 0.0), defined_on=m.definedonelements))
            return out
        if m.skeleton:
            return self._skeleton_terms()
        dom = m.domain_type
        for mono in self.expr.monos:
            if mono.vec is not None:
                raise TypeError("integrand is a vector, not a scalar")
            scal = [a for a in mono.scal]
            # coefficient factors: one GridFunction, monomials of x, y, z
            gfs = [a[1] for a in scal if a[0] == "gf"]
            ex = [0, 0, 0]
            for a in scal:
                if a[0] == "xyz":
                    ex = [p + q for p, q in zip(ex, a[1])]
            scal = [a for a in scal if a[0] not in ("gf", "xyz")]
            if len(gfs) > 1:
                raise NotImplementedError("one GridFunction factor per integrand term")
            if any(a[1] for a in scal if a[0] in ("u", "v")):
                raise NotImplementedError(".Other() is only meaningful on facet patches")
            names = sorted(a[0] for a in scal)
            kind, b = None, (0.0, 0.0, 0.0)
            nrm_index = 0
            # n . n = 1 for the unit normal of one level set
            mono_dots = [d for d in mono.dots if not (d[0][0] == "n" and d[1][0] == "n" and d[0][1] == d[1][1])]
            dots = [tuple(sorted((d[0][0], d[1][0]))) for d in mono_dots]
            for d in mono_dots:
                for v in d:
                    if v[0] != "n" or nrm_gf is None:
                        continue
                    if isinstance(nrm_gf, (tuple, list)):
                        ids = [id(g) for g in nrm_gf]
                        if v[1] not in ids:
                            raise NotImplementedError("the normal must be Normalize(grad(l)) of one of the level sets")
                        nrm_index = ids.index(v[1])
                    elif v[1] != id(nrm_gf):
                        raise NotImplementedError("the normal must be Normalize(grad(levelset)) of the cut's level set")
            tb = None
            if names == ["u", "v"] and not dots:
                kind = TERM_MASS
            elif names == ["dtu", "v"] and not dots:
                kind = TERM_DT_U_V
            elif names == ["v"] and len(dots) == 1 and set(dots[0]) == {"gu", "tb"}:
                kind = TERM_CONV
                tb = [x for x in mono_dots[0] if x[0] == "tb"][0][1]
            elif not names and dots == [("gu", "gv")]:
                kind = TERM_LAPLACE
            elif not names and sorted(dots) == [("gu", "n"), ("gv", "n")]:
                kind = TERM_NGRADU_NGRADV
            elif names == ["v"] and dots == [("gu", "n")]:
                kind = TERM_NGRADU_V
            elif names == ["u"] and dots == [("gv", "n")]:
                kind = TERM_U_NGRADV
            elif names == ["v"] and len(dots) == 1 and set(dots[0]) == {"gu", "b"}:
                kind = TERM_CONV
                bv = [x for x in mono_dots[0] if x[0] == "b"][0][1]
                b = tuple(list(bv) + [0.0] * (3 - len(bv)))
            else:
                raise NotImplementedError("integrand term outside the supported menu: %s" % (names + dots,))
            out.append(dict(kind=kind, domain=dom, order=-1 if m.order is None else m.order, hpow=mono.hpow,
                            coef=mono.c * m.scale, b=b, defined_on=m.definedonelements, tb=tb,
                            tref=m.tref, time_order=m.time_order, normal_lset=nrm_index,
                            gf=gfs[0] if gfs else None, e=tuple(ex)))
        return out


    def _skeleton_terms(self):
        """Skeleton integrand -> XG_TERM_SKEL_* terms.  Every monomial is
        c * h^p * (trial factor) * (test factor), a factor being the value or
        the j-th derivative along n_F of the function on the facet's first
        (side 0) or second (side 1, .Other()) element; dn(w.Other(), k) is
        turned to n_F with (-1)^k.  The coefficients of each (trial kind, test
        kind) block must form one menu term: [u][v] (value, value), the
        flux {grad u . n_F}[v] (first derivative, value), its transpose, or
        [d^k u][d^k v] (k, k)."""
        m = self.measure
        blocks = {}
        for mono in self.expr.monos:
            if mono.vec is not None:
                raise TypeError("integrand is a vector, not a scalar")
            fac = {}
            c = mono.c
            for a in mono.scal:
                if a[0] in ("u", "v"):
                    fac.setdefault(a[0], []).append((0, 1 if a[1] else 0))
                elif a[0] in ("dnu", "dnv"):
                    k = a[2]
                    if a[1] and k % 2 == 1:
                        c = -c  # the second element's outward normal is -n_F
                    fac.setdefault(a[0][2], []).append((k, 1 if a[1] else 0))
                else:
                    raise NotImplementedError("skeleton integrands: trial / test values and normal derivatives")
            for d in mono.dots:
                names = [x[0] for x in d]
                if "nF" not in names:
                    raise NotImplementedError("skeleton integrands: gradients only as grad(.) * specialcf.normal")
                g = d[1] if d[0][0] == "nF" else d[0]
                if g[0] not in ("gu", "gv"):
                    raise NotImplementedError("skeleton integrands: gradients only as grad(.) * specialcf.normal")
                fac.setdefault(g[0][1], []).append((1, 1 if g[1] else 0))
            if len(fac.get("u", [])) != 1 or len(fac.get("v", [])) != 1:
                raise NotImplementedError("skeleton integrands need one trial and one test factor per product")
            (ku, su), (kv, sv) = fac["u"][0], fac["v"][0]
            key = (mono.hpow, ku, kv)
            blocks.setdefault(key, np.zeros((2, 2)))
            blocks[key][su, sv] += c
        jump = np.array([[1.0, -1.0], [-1.0, 1.0]])
        mean_jump = np.array([[1.0, -1.0], [1.0, -1.0]])  # [su][sv]: trial mean, test jump
        out = []
        for (hp, ku, kv), B in sorted(blocks.items()):
            if ku == kv == 0:
                kind, P = TERM_SKEL_JUMP, jump
            elif ku == 1 and kv == 0:
                kind, P = TERM_SKEL_FLUX, mean_jump
            elif ku == 0 and kv == 1:
                kind, P = TERM_SKEL_FLUX_T, mean_jump.T
            elif ku == kv and ku >= 1:
                kind, P = TERM_SKEL_DN1 + ku - 1, jump
            else:
                raise NotImplementedError("skeleton integrand block (%d, %d) is outside the menu" % (ku, kv))
            cc = B[0, 0] / P[0, 0]
            if np.abs(B - cc * P).max() > 1e-14 * max(1.0, abs(cc)):
                raise NotImplementedError("skeleton integrand is not a jump / average product: %s" % B.tolist())
            if cc == 0.0:
                continue
            out.append(dict(kind=kind, domain=m.domain_type, order=-1, hpow=hp, coef=cc * m.scale, b=(0.0, 0.0, 0.0),
                            defined_on=m.definedonelements, tb=None, tref=None, time_order=-1))
        return out


class _SumOfIntegrals:
    def __init__(self, items):
        self.items = list(items)

    def __add__(self, o):
        if isinstance(o, _Integral):
            return _SumOfIntegrals(self.items + [o])
        if isinstance(o, _SumOfIntegrals):
            return _SumOfIntegrals(self.items + o.items)
        raise TypeError("can only add integrals")


# ----------------------------------------------------------------------------
# bilinear forms
# ----------------------------------------------------------------------------
class SparseMatrix:
    """Compressed-row matrix over the form's active dofs (device tensors)."""

    def __init__(self, ndof, row_dof, rowptr, cols, vals, nrows, nnz):
        self.ndof, self.row_dof, self.rowptr, self.cols, self.vals = ndof, row_dof, rowptr, cols, vals
        self.nrows, self.nnz = nrows, nnz

    def global_coo(self):
        """(rows, cols, vals) numpy arrays in global dof numbering."""
        n, z = self.nrows, self.nnz
        rd = self.row_dof[:n].cpu().numpy()
        rp = self.rowptr[: n + 1].cpu().numpy()
        c = self.cols[:z].cpu().numpy()
        v = self.vals[:z].cpu().numpy()
        rows = np.repeat(rd, np.diff(rp))
        return rows, rd[c], v

    def to_scipy(self):
        import scipy.sparse as sp
        r, c, v = self.global_coo()
        return sp.csr_matrix((v, (r, c)), shape=(self.ndof, self.ndof))


def RestrictedBilinearForm(space, name="a", element_restriction=None, facet_restriction=None, check_unused=True,
                           **kwargs):
    """The reference's RestrictedBilinearForm (utils/restrictedblf.cpp:7-168):
    a BilinearForm whose sparsity graph holds only the couplings of the
    restricted elements and facets.  Here every form's pattern is that of its
    active elements and facets already (the integrators' definedonelements
    decide them), so this is a BilinearForm; the restrictions are kept as
    attributes."""
    a = BilinearForm(space, **kwargs)
    a.element_restriction, a.facet_restriction = element_restriction, facet_restriction
    return a


class BilinearForm:
    """BilinearForm over one H1 space: `a += integrand * dCut(...)` /
    `* dFacetPatch(...)`, `a.Assemble()` -> `a.mat` (SparseMatrix)."""

    def __init__(self, space, symmetric=False, precision=PREC_FP64, **kwargs):
        self.space = space
        self.integrals = []
        self.precision = precision
        self.mat = None
        self._form = None
        self._key = None
        self._out = None

    def __iadd__(self, integral):
        if isinstance(integral, _Integral):
            self.integrals.append(integral)
        elif isinstance(integral, _SumOfIntegrals):
            self.integrals.extend(integral.items)
        else:
            raise TypeError("add integrand * dCut(...) or integrand * dFacetPatch(...)")
        self._form = None
        return self

    def _levelset(self):
        ls = [i.measure.levelset for i in self.integrals if i.measure.kind == "cut"]
        if not ls:
            return None
        for l in ls[1:]:
            same = (l is ls[0]) or (isinstance(l, (tuple, list)) and isinstance(ls[0], (tuple, list)) and
                                    len(l) == len(ls[0]) and all(a is b for a, b in zip(l, ls[0])))
            if not same:
                raise NotImplementedError("all dCut integrals of one form must share the level set(s)")
        return ls[0]

    def _build_ml(self, lsets):
        """Form on regions of several level sets (xg_mlset_form_create): the
        region terms of the dCut integrals (domain types: a tuple, a list of
        tuples or a DomainTypeArray), the normals Normalize(grad(l_i)) of the
        level sets, ghost-penalty patch terms."""
        from .mlset import DomainTypeArray
        M = len(lsets)
        region, patch = [], []
        for it in self.integrals:
            if it.measure.kind == "patch":
                patch += it.terms(None)
                continue
            if it.measure.kind != "cut" or getattr(it.measure, "skeleton", False):
                raise NotImplementedError("forms on several level sets take dCut region terms and dFacetPatch")
            dom = it.measure.domain_type
            if not isinstance(dom, DomainTypeArray):
                dom = DomainTypeArray(list(dom) if isinstance(dom, list) else dom)
            tup = np.ascontiguousarray(np.array(dom.as_list, dtype=np.int8).reshape(-1, M))
            for t in it.terms(lsets):
                if t["kind"] not in (TERM_MASS, TERM_LAPLACE, TERM_NGRADU_V, TERM_U_NGRADV, TERM_CONV) or \
                        t.get("tb") is not None or t.get("gf") is not None or any(t.get("e", (0, 0, 0))):
                    raise NotImplementedError("region terms: mass, Laplace, Nitsche normal terms, convection")
                t["tuples"] = tup
                region.append(t)
        arr = (_lib.MlTerm * len(region))()
        self._keep = []
        for k, t in enumerate(region):
            arr[k].kind, arr[k].order, arr[k].hpow = t["kind"], t["order"], t["hpow"]
            arr[k].normal_lset, arr[k].coef = t["normal_lset"], t["coef"]
            for j in range(3):
                arr[k].b[j] = t["b"][j]
            arr[k].ntup = t["tuples"].shape[0]
            arr[k].h_tuples = t["tuples"].ctypes.data
            self._keep.append(t["tuples"])
            d = t["defined_on"]
            if d is not None:
                self._keep.append(d)
            arr[k].d_defined_on = d.words.data_ptr() if d is not None else None
        parr = (_lib.Term * max(len(patch), 1))()
        for k, t in enumerate(patch):
            parr[k].kind, parr[k].domain, parr[k].order, parr[k].hpow = t["kind"], 0, t["order"], t["hpow"]
            parr[k].coef = t["coef"]
            d = t["defined_on"]
            if d is not None:
                self._keep.append(d)
            parr[k].d_defined_on = d.words.data_ptr() if d is not None else None
        h = ctypes.c_void_p()
        _lib.call("xg_mlset_form_create", self.space.h, M, arr, len(region), parr, len(patch), self.precision,
                  ctypes.byref(h))
        self._form = h
        self._terms = region + patch
        self._ml = True
        cap = np.zeros(2, dtype=np.int64)
        _lib.call("xg_form_capacity", h, cap.ctypes.data_as(ctypes.c_void_p))
        self._alloc(int(cap[0]), int(cap[1]))

    def _build_st(self):
        """Space-time form (xg_st_form_create): slab terms (time_order of the
        measure) and fixed-time terms (tref), ghost-penalty patch terms."""
        lset = self._levelset()
        terms = []
        for it in self.integrals:
            terms += it.terms(lset)
        if any(t.get("gf") is not None or any(t.get("e", (0, 0, 0))) for t in terms):
            raise NotImplementedError("space-time forms take constant coefficients")
        orders = {t["time_order"] for t in terms if t.get("tref") is None and t["kind"] != TERM_GHOST_MASS}
        orders |= {it.measure.time_order for it in self.integrals if it.measure.kind == "patch"}
        orders.discard(-1)
        if len(orders) > 1:
            raise NotImplementedError("one time rule order per space-time form")
        order_time = orders.pop() if orders else 2 * self.space.order_time
        arr = (_lib.StTerm * len(terms))()
        for k, t in enumerate(terms):
            B = arr[k].base
            B.kind, B.domain, B.order, B.hpow, B.coef = t["kind"], t["domain"], t["order"], t["hpow"], t["coef"]
            for j in range(3):
                B.b[j] = t["b"][j]
            B.d_defined_on = None  # the space-time step marks HASNEG / IF / HASPOS and the ghost facets itself
            tb = t.get("tb")
            if tb is not None:
                for j in range(3):
                    B.b[j] = tb[0][j]
                    arr[k].bc[j] = tb[1][j]
                    arr[k].bs[j] = tb[2][j]
                arr[k].omega, arr[k].t0, arr[k].dt = tb[3], tb[4], tb[5]
            else:
                arr[k].omega, arr[k].t0, arr[k].dt = 0.0, 0.0, 1.0
            arr[k].tref = -1.0 if t.get("tref") is None else float(t["tref"])
        h = ctypes.c_void_p()
        kt_l = lset.space.order_time if isinstance(lset.space, SpaceTimeFESpace) else 0
        _lib.call("xg_st_form_create", self.space.h, kt_l, order_time, arr, len(terms), self.precision, ctypes.byref(h))
        self._form = h
        self._terms = terms
        cap = np.zeros(2, dtype=np.int64)
        _lib.call("xg_form_capacity", h, cap.ctypes.data_as(ctypes.c_void_p))
        self._alloc(int(cap[0]), int(cap[1]))

    def _build_quad(self, lset):
        """Q1 form on a quadrilateral / hexahedral mesh (xg_quad_form_create):
        volume terms of the menu, no facet or boundary terms."""
        terms = []
        for it in self.integrals:
            m = it.measure
            if m.kind != "cut" or getattr(m, "vb", VOL) == BND or m.skeleton or \
                    getattr(m, "deformation", None) is not None:
                raise NotImplementedError("forms on quadrilateral / hexahedral meshes take dCut volume terms")
            for t in it.terms(lset):
                if t["kind"] not in (TERM_MASS, TERM_LAPLACE, TERM_NGRADU_V, TERM_U_NGRADV, TERM_CONV) or \
                        t.get("tb") is not None or t.get("gf") is not None or any(t.get("e", (0, 0, 0))):
                    raise NotImplementedError("quad / hex forms: mass, Laplace, Nitsche and convection terms")
                terms.append(t)
        pols = {it.measure.quad_dir_policy for it in self.integrals}
        if len(pols) > 1:
            raise NotImplementedError("one quad_dir_policy per form")
        arr = (_lib.Term * max(len(terms), 1))()
        self._keep = []
        for k, t in enumerate(terms):
            arr[k].kind, arr[k].domain, arr[k].order, arr[k].hpow = t["kind"], t["domain"], t["order"], t["hpow"]
            arr[k].coef = t["coef"]
            for j in range(3):
                arr[k].b[j] = t["b"][j]
            d = t["defined_on"]
            if d is not None:
                self._keep.append(d)
            arr[k].d_defined_on = d.words.data_ptr() if d is not None else None
        h = ctypes.c_void_p()
        _lib.call("xg_quad_form_create", device_mesh(self.space.mesh).h, arr, len(terms), pols.pop(),
                  ctypes.byref(h))
        self._form = h
        self._quad = True
        self._terms = terms
        cap = np.zeros(2, dtype=np.int64)
        _lib.call("xg_quad_form_capacity", h, cap.ctypes.data_as(ctypes.c_void_p))
        self._alloc(int(cap[0]), int(cap[1]))

    def _build(self):
        if isinstance(self.space, SpaceTimeFESpace):
            return self._build_st()
        if getattr(self.space.mesh, "tensor", False):
            return self._build_quad(self._levelset())
        lset = self._levelset()
        if isinstance(lset, (tuple, list)):
            return self._build_ml(lset)
        terms, bterms, cterms = [], [], []
        for it in self.integrals:
            if it.measure.kind == "cut" and getattr(it.measure, "vb", VOL) == BND:
                bterms += self._bnd_terms(it, lset)
                continue
            # volume terms on the deformed mesh go to the coefficient kernel;
            # deformed patch terms stay patch terms (xg_form_set_deformation)
            deform = getattr(it.measure, "deformation", None) if it.measure.kind in ("cut", "vol") else None
            for t in it.terms(lset):
                t["deform"] = deform
                generic = t.get("gf") is not None or any(t.get("e", (0, 0, 0))) or deform is not None or \
                    t["kind"] == TERM_NGRADU_NGRADV or it.measure.kind == "vol"
                (cterms if generic else terms).append(t)
        arr = (_lib.Term * max(len(terms), 1))()
        self._keep = []
        for k, t in enumerate(terms):
            arr[k].kind, arr[k].domain, arr[k].order, arr[k].hpow = t["kind"], t["domain"], t["order"], t["hpow"]
            arr[k].coef = t["coef"]
            for j in range(3):
                arr[k].b[j] = t["b"][j]
            d = t["defined_on"]
            if d is not None:
                self._keep.append(d)
                arr[k].d_defined_on = d.words.data_ptr()
            else:
                arr[k].d_defined_on = None
        h = ctypes.c_void_p()
        _lib.call("xg_form_create", self.space.h, arr, len(terms), self.precision, ctypes.byref(h))
        self._form = h
        self._terms = terms
        pdef = {id(it.measure.deformation): it.measure.deformation for it in self.integrals
                if it.measure.kind == "patch"}
        if len(pdef) > 1:
            raise NotImplementedError("the facet-patch terms of one form share one deformation (or none)")
        pd = next(iter(pdef.values())) if pdef else None
        if pd is not None:
            gd = pd._edge_deformation()
            self._keep.append(gd)
            _lib.call("xg_form_set_deformation", h, gd.data_ptr())
        if bterms:
            barr = (_lib.BTerm * len(bterms))()
            for k, t in enumerate(bterms):
                barr[k].kind, barr[k].domain, barr[k].order, barr[k].hpow = t["kind"], t["domain"], t["order"], t["hpow"]
                barr[k].coef = t["coef"]
                d = t["defined_on"]
                if d is not None:
                    self._keep.append(d)
                barr[k].d_defined_on = d.words.data_ptr() if d is not None else None
            _lib.call("xg_form_set_bnd_terms", h, barr, len(bterms))
            self._bterms = bterms
        if cterms:
            carr = (_lib.CTerm * len(cterms))()
            for k, t in enumerate(cterms):
                if t["kind"] not in (TERM_MASS, TERM_LAPLACE, TERM_NGRADU_V, TERM_U_NGRADV, TERM_CONV,
                                     TERM_NGRADU_NGRADV) or t.get("tb") is not None:
                    raise NotImplementedError("coefficient fields and dx terms: mass, Laplace, Nitsche, convection "
                                              "and normal-normal terms")
                carr[k].kind, carr[k].domain, carr[k].order, carr[k].hpow = t["kind"], t["domain"], t["order"], t["hpow"]
                carr[k].coef = t["coef"]
                for j in range(3):
                    carr[k].b[j] = t["b"][j]
                    carr[k].e[j] = t["e"][j]
                g = t["gf"]
                if g is not None:
                    if not isinstance(g.space, H1) or g.space.mesh is not self.space.mesh:
                        raise ValueError("the coefficient GridFunction must live in an H1 space of the form's mesh")
                    self._keep.append(g)
                    carr[k].gf_space, carr[k].d_gf = g.space.h, g.vec.data_ptr()
                d = t["defined_on"]
                if d is not None:
                    self._keep.append(d)
                carr[k].d_defined_on = d.words.data_ptr() if d is not None else None
                if t.get("deform") is not None:
                    gd = t["deform"]._edge_deformation()
                    self._keep.append(gd)
                    carr[k].d_deform = gd.data_ptr()
            _lib.call("xg_form_set_coef_terms", h, carr, len(cterms))
            self._cterms = cterms
        cap = np.zeros(2, dtype=np.int64)
        _lib.call("xg_form_capacity", h, cap.ctypes.data_as(ctypes.c_void_p))
        self._alloc(int(cap[0]), int(cap[1]))

    def _bnd_terms(self, it, lset):
        """Boundary terms c * u * v * dCut(lset, dt, vb=BND[, definedon=
        mesh.Boundaries(..)][, definedonelements=BND BitArray]) (the
        reference's SymbolicCutBFI on boundary elements): mass terms only, the
        two restrictions intersected."""
        m = it.measure
        if getattr(m, "subdivlvl", 0):
            raise NotImplementedError("boundary terms take the straight cut of a P1 level set")
        mesh = self.space.mesh
        defined = _bnd_restriction(mesh, m.definedonelements, getattr(m, "definedon", None))
        out = []
        for mono in it.expr.monos:
            if mono.vec is not None or mono.dots or sorted(a[0] for a in mono.scal) != ["u", "v"] or \
                    any(a[1] for a in mono.scal):
                raise NotImplementedError("boundary terms of bilinear forms: c * u * v (times powers of h)")
            out.append(dict(kind=TERM_MASS, domain=m.domain_type, order=-1 if m.order is None else m.order,
                            hpow=mono.hpow, coef=mono.c * m.scale, defined_on=defined))
        return out

    def _alloc(self, cap_rows, cap_nnz):
        dev = _dev()
        self._row_dof = torch.zeros(cap_rows, dtype=torch.int32, device=dev)
        self._rowptr = torch.zeros(cap_rows + 1, dtype=torch.int64, device=dev)
        self._cols = torch.zeros(max(cap_nnz, 1), dtype=torch.int32, device=dev)
        self._vals = torch.zeros(max(cap_nnz, 1), dtype=torch.float64, device=dev)
        self._counts = torch.zeros(2, dtype=torch.int64, device=dev)
        c = _lib.Csr()
        c.d_row_dof, c.d_rowptr = self._row_dof.data_ptr(), self._rowptr.data_ptr()
        c.d_cols, c.d_vals, c.d_counts = self._cols.data_ptr(), self._vals.data_ptr(), self._counts.data_ptr()
        c.cap_rows, c.cap_nnz = cap_rows, cap_nnz
        self._csr = c

    def Assemble(self, cutinfo=None, reallocate=False):
        if self._form is None:
            self._build()
        lset = self._levelset()
        if getattr(self, "_quad", False):
            dm = device_mesh(self.space.mesh)
            _lib.call("xg_quad_form_assemble", self._form, _vp(_lset_vec(lset)), ctypes.byref(self._csr), _stream())
            torch.cuda.synchronize()
            dm.check()
            nrows, nnz = (int(x) for x in self._counts.cpu().tolist())
            self.mat = SparseMatrix(self.space.ndof, self._row_dof, self._rowptr, self._cols, self._vals, nrows, nnz)
            return self
        if isinstance(lset, (tuple, list)):
            nv = lset[0].space.mesh.nv
            vals = torch.stack([_lset_vec(g)[:nv] for g in lset]).contiguous()
            _lib.call("xg_mlset_form_assemble", self._form, _vp(vals), ctypes.byref(self._csr), _stream())
            torch.cuda.synchronize()
            _lib.check(_lib.load().xg_form_check(self._form), "device (form on several level sets)")
            nrows, nnz = (int(x) for x in self._counts.cpu().tolist())
            self.mat = SparseMatrix(self.space.ndof, self._row_dof, self._rowptr, self._cols, self._vals, nrows, nnz)
            return self
        if isinstance(self.space, SpaceTimeFESpace):
            # the space-time CutFEM step: marking, ghost facets and assembly in one call
            _lib.call("xg_st_cutfem_step", self._form, _vp(_lset_vec(lset)), ctypes.byref(self._csr), _stream())
            torch.cuda.synchronize()
            _lib.check(_lib.load().xg_form_check(self._form), "device (space-time form)")
            nrows, nnz = (int(x) for x in self._counts.cpu().tolist())
            self.mat = SparseMatrix(self.space.ndof, self._row_dof, self._rowptr, self._cols, self._vals, nrows, nnz)
            return self
        if cutinfo is None:
            if lset is None:
                # no cut integrals: every element counts as NEG for domain-free terms
                raise NotImplementedError("forms without dCut integrals are not part of the GPU path")
            cutinfo = CutInfo(self.space.mesh, lset)
        _lib.call("xg_form_assemble", self._form, _vp(_lset_vec(lset)), _vp(cutinfo.dom), ctypes.byref(self._csr),
                  _stream())
        torch.cuda.synchronize()
        _lib.check(_lib.load().xg_form_check(self._form), "device (form)")
        nrows, nnz = (int(x) for x in self._counts.cpu().tolist())
        self.mat = SparseMatrix(self.space.ndof, self._row_dof, self._rowptr, self._cols, self._vals, nrows, nnz)
        return self

    def __del__(self):
        if getattr(self, "_form", None) and _lib._lib is not None:
            if getattr(self, "_quad", False):
                _lib.load().xg_quad_form_destroy(self._form)
            else:
                _lib.load().xg_form_destroy(self._form)
            self._form = None


class LinearForm:
    """LinearForm over one H1 space: `f += coef * v * dCut(...)` with coef a
    number, a monomial of x, y, z or a GridFunction of the same space, and
    boundary terms `f += coef * v * dCut(lset, dt, vb=BND[, definedon=
    mesh.Boundaries(..)][, definedonelements=BND BitArray])` with coef a
    number or a monomial; `f.Assemble()` -> `f.vec` (device tensor, global
    dof numbering) (xfem/symboliccutlfi.cpp:57-180)."""

    def __init__(self, space, **kwargs):
        self.space = space
        self.integrals = []
        self.vec = torch.zeros(space.ndof, dtype=torch.float64, device=_dev())
        self._lf = None

    def __iadd__(self, integral):
        if isinstance(integral, _Integral):
            self.integrals.append(integral)
        elif isinstance(integral, _SumOfIntegrals):
            self.integrals.extend(integral.items)
        else:
            raise TypeError("add integrand * dCut(...)")
        self._lf = None
        return self

    def _terms(self):
        out = []
        for it in self.integrals:
            m = it.measure
            if m.kind != "cut":
                raise NotImplementedError("linear forms: dCut integrals only")
            for mono in it.expr.monos:
                if mono.dots or mono.vec is not None or mono.hpow != 0:
                    raise NotImplementedError("linear form integrands: coef * (monomial | GridFunction) * v")
                atoms = list(mono.scal)
                if ("v", False) not in atoms or any(a[0] == "u" for a in atoms):
                    raise NotImplementedError("linear form integrands need the test function v once")
                atoms.remove(("v", False))
                kind, e, gf = XG_LTERM_SOURCE, (0, 0, 0), None
                for a in atoms:
                    if a[0] == "xyz" and kind == XG_LTERM_SOURCE and e == (0, 0, 0):
                        e = a[1]
                    elif a[0] == "gf" and gf is None and e == (0, 0, 0):
                        kind, gf = XG_LTERM_SOURCE_GF, a[1]
                        gs = gf.space
                        if isinstance(gs, SpaceTimeFESpace) or gs.mesh is not self.space.mesh or \
                                getattr(gs, "h", None) is None:
                            raise ValueError("the coefficient GridFunction must live in a spatial H1 / L2 space "
                                             "of the form's mesh")
                    else:
                        raise NotImplementedError("one monomial or one GridFunction factor per term")
                defined = m.definedonelements
                if getattr(m, "vb", VOL) == BND:
                    if kind != XG_LTERM_SOURCE:
                        raise NotImplementedError("boundary linear form integrands: coef * monomial * v")
                    kind, defined = XG_LTERM_SOURCE_BND, _bnd_restriction(self.space.mesh, defined, m.definedon)
                out.append(dict(kind=kind, domain=m.domain_type, order=-1 if m.order is None else m.order, e=e,
                                coef=mono.c, gf=gf, defined_on=defined))
        return out

    def _levelset(self):
        ls = [i.measure.levelset for i in self.integrals]
        for l in ls[1:]:
            if l is not ls[0]:
                raise NotImplementedError("all dCut integrals of one linear form must share the level set")
        return ls[0] if ls else None

    def _build(self):
        terms = self._terms()
        defs = {id(it.measure.deformation): it.measure.deformation for it in self.integrals
                if getattr(it.measure, "vb", VOL) != BND}
        if len(defs) > 1:
            raise NotImplementedError("the volume terms of one linear form share one deformation (or none)")
        self._deform = next(iter(defs.values())) if defs else None
        arr = (_lib.LTerm * len(terms))()
        self._keep = []
        for k, t in enumerate(terms):
            arr[k].kind, arr[k].domain, arr[k].order, arr[k].coef = t["kind"], t["domain"], t["order"], t["coef"]
            for j in range(3):
                arr[k].e[j] = t["e"][j]
            arr[k].d_gf = t["gf"].vec.data_ptr() if t["gf"] is not None else None
            arr[k].gf_space = t["gf"].space.h.value if t["gf"] is not None else None
            d = t["defined_on"]
            if d is not None:
                self._keep.append(d)
            arr[k].d_defined_on = d.words.data_ptr() if d is not None else None
            if t["gf"] is not None:
                self._keep.append(t["gf"])
        h = ctypes.c_void_p()
        _lib.call("xg_lform_create", self.space.h, arr, len(terms), ctypes.byref(h))
        self._lf = h
        if self._deform is not None:
            gd = self._deform._edge_deformation()
            self._keep.append(gd)
            _lib.call("xg_lform_set_deformation", h, gd.data_ptr())

    def Assemble(self, cutinfo=None):
        if self._lf is None:
            self._build()
        lset = self._levelset()
        if lset is None:
            raise NotImplementedError("linear forms without dCut integrals are not part of the GPU path")
        if cutinfo is None:
            cutinfo = CutInfo(self.space.mesh, lset)
        _lib.call("xg_lform_assemble", self._lf, _vp(_lset_vec(lset)), _vp(cutinfo.dom), _vp(self.vec), _stream())
        torch.cuda.synchronize()
        _lib.check(_lib.load().xg_lform_check(self._lf), "device (linear form)")
        return self

    def __del__(self):
        if getattr(self, "_lf", None) and _lib._lib is not None:
            _lib.load().xg_lform_destroy(self._lf)
            self._lf = None


# ----------------------------------------------------------------------------
# Integrate
# ----------------------------------------------------------------------------
class _Monomial:
    def __init__(self, e=(0, 0, 0)):
        self.e = tuple(e)

    def __mul__(self, o):
        if isinstance(o, _Monomial):
            return _Monomial(tuple(a + b for a, b in zip(self.e, o.e)))
        if isinstance(o, _Measure):
            return ("integral", self, o)
        if isinstance(o, (_Expr, int, float, GridFunction)):
            return _Expr([_Mono(scal=(("xyz", self.e),))]) * o
        raise TypeError("monomial coefficient functions only")

    def __rmul__(self, o):
        if isinstance(o, (int, float)):
            return _Expr([_Mono(c=float(o), scal=(("xyz", self.e),))])
        return self.__mul__(o)

    def __pow__(self, p):
        return _Monomial(tuple(a * int(p) for a in self.e))


x, y, z = _Monomial((1, 0, 0)), _Monomial((0, 1, 0)), _Monomial((0, 0, 1))


def _integrate_fields(expr, meas, order):
    """Integrate(cf * dCut(lset, dt)) for cf a polynomial in GridFunctions
    (at most two factors per product, at most four fields) and x, y, z:
    xg_integrate_fields (the reference's Integrate with a CoefficientFunction
    of GridFunctions, cutint/cutintegral.cpp:126-212), e.g. the L2 error
    Integrate((gfu - gfex) ** 2 * dCut(lsetp1, NEG), mesh)."""
    if meas.kind != "cut" or meas.skeleton or meas.vb != VOL or meas.subdivlvl:
        raise NotImplementedError("Integrate of GridFunction integrands: dCut(P1 level set, dt[, order, "
                                  "definedonelements, deformation]) on volume elements")
    lset = meas.levelset
    if not isinstance(lset, GridFunction) or isinstance(lset.space, SpaceTimeFESpace):
        raise NotImplementedError("Integrate of GridFunction integrands takes one spatial P1 level set")
    lv = _lset_vec(lset)
    mesh = lset.space.mesh
    D = mesh.dim
    fields, monos = [], {}

    def field_index(g):
        if isinstance(g.space, SpaceTimeFESpace) or g.space.mesh is not mesh:
            raise ValueError("the GridFunctions must live in spatial spaces of the level set's mesh")
        k = next((i for i, f in enumerate(fields) if f is g), None)
        if k is None:
            fields.append(g)
            k = len(fields) - 1
        return k

    bad = "Integrate integrands: products of GridFunctions, their gradients and x, y, z"
    for m in expr.monos:
        if m.vec is not None or m.hpow:
            raise NotImplementedError(bad)
        # a product of sums: every dot product of two vectors is a sum over
        # the directions (factors (field, -1) = value, (field, d) = d/dx_d)
        branches = [(m.c, [])]
        ex = [0, 0, 0]
        for a in m.scal:
            if a[0] == "gf":
                branches = [(c, f + [(field_index(a[1]), -1)]) for c, f in branches]
            elif a[0] == "xyz":
                ex = [p + q for p, q in zip(ex, a[1])]
            else:
                raise NotImplementedError(bad)
        for d in m.dots:
            comps = []
            for v in d:
                if v[0] == "ggf":
                    k = field_index(v[1])
                    comps.append([(1.0, [(k, r)]) for r in range(D)])
                elif v[0] == "b":
                    b = list(v[1]) + [0.0] * (3 - len(v[1]))
                    comps.append([(b[r], []) for r in range(D)])
                else:
                    raise NotImplementedError(bad)
            branches = [(c * ca * cb, f + fa + fb) for c, f in branches
                        for (ca, fa), (cb, fb) in zip(comps[0], comps[1]) if ca * cb != 0.0]
        for c, f in branches:
            if len(f) > 2:
                raise NotImplementedError("Integrate integrands: at most two GridFunction factors per product")
            key = (tuple(ex), tuple(sorted(f)))
            monos[key] = monos.get(key, 0.0) + c
    monos = {k: c for k, c in monos.items() if c != 0.0}
    if len(fields) > 4 or len(monos) > 16:
        raise NotImplementedError("Integrate integrands: at most 4 GridFunctions and 16 distinct products")
    arr = (_lib.FMono * max(len(monos), 1))()
    for i, ((ex, f), c) in enumerate(monos.items()):
        arr[i].coef = c
        for r in range(3):
            arr[i].e[r] = ex[r]
        arr[i].f0, arr[i].d0 = f[0] if len(f) > 0 else (-1, -1)
        arr[i].f1, arr[i].d1 = f[1] if len(f) > 1 else (-1, -1)
    sp = (ctypes.c_void_p * max(len(fields), 1))(*[f.space.h.value for f in fields])
    dv = (ctypes.c_void_p * max(len(fields), 1))(*[f.vec.data_ptr() for f in fields])
    dm = device_mesh(mesh)
    res = torch.zeros(1, dtype=torch.float64, device=_dev())
    defined = meas.definedonelements
    q = meas.order if meas.order is not None else order
    gdef = meas.deformation._edge_deformation() if meas.deformation is not None else None
    _lib.call("xg_integrate_fields", dm.h, _vp(lv), meas.domain_type, int(q), len(fields), sp, dv, len(monos), arr,
              _vp(defined.words) if defined is not None else None, _vp(gdef), _vp(res), _stream())
    dm.check()
    return meas.scale * float(res.item())


def Integrate(levelset_domain=None, cf=None, mesh=None, order=5, integrand=None):
    """Integrate(x^a y^b z^c * dCut(lset, dt, order)) on the GPU
    (cutint/cutintegral.cpp:126-212): a deterministic fixed-order sum.  Also
    called as Integrate(x**2 * dCut(...), mesh) or Integrate(dCut(...), mesh)."""
    if isinstance(levelset_domain, _Integral):
        return _integrate_fields(levelset_domain.expr, levelset_domain.measure, order)
    if isinstance(levelset_domain, dict) and isinstance(cf, (_Expr, GridFunction)):
        meas = dCut(levelset_domain["levelset"], levelset_domain["domain_type"], levelset_domain.get("order", order),
                    **{k: v for k, v in levelset_domain.items() if k not in ("levelset", "domain_type", "order")})
        return _integrate_fields(_Expr.wrap(cf), meas, order)
    if isinstance(levelset_domain, _Measure):
        levelset_domain = ("integral", _Monomial(), levelset_domain)
    if isinstance(levelset_domain, tuple) and len(levelset_domain) == 3 and levelset_domain[0] == "integral":
        integrand, levelset_domain = levelset_domain, None
        if isinstance(cf, Mesh):
            mesh, cf = cf, None
    scale = integrand[2].scale if integrand is not None else 1.0
    if scale != 1.0:
        return scale * Integrate(levelset_domain, cf, mesh, order, ("integral", integrand[1], _unscaled(integrand[2])))
    if integrand is not None:
        _, mono, meas = integrand
        lset, dt, order = meas.levelset, meas.domain_type, meas.order if meas.order is not None else order
        defined = meas.definedonelements
    else:
        lset, dt = levelset_domain["levelset"], levelset_domain["domain_type"]
        order = levelset_domain.get("order", order)
        policy = levelset_domain.get("quad_dir_policy", OPTIMAL)
        mono = cf if isinstance(cf, _Monomial) else _Monomial()
        defined = None
    vb = VOL
    if integrand is not None:
        policy = getattr(meas, "quad_dir_policy", OPTIMAL)
        vb = getattr(meas, "vb", VOL)
    else:
        vb = levelset_domain.get("vb", VOL)
    deform = getattr(meas, "deformation", None) if integrand is not None else levelset_domain.get("deformation")
    if deform is not None:
        # Integrate on the deformed mesh: the adaptation's own mapped rule, for
        # its P1 level set (lset_p1) on all elements
        if vb == BND or defined is not None or isinstance(lset, (tuple, list)):
            raise NotImplementedError("Integrate with a deformation: VOL, one level set, no definedonelements")
        if not torch.equal(_lset_vec(lset)[: deform.mesh.nv], _lset_vec(deform.lset_p1)[: deform.mesh.nv]):
            raise ValueError("Integrate with a deformation takes the adaptation's lset_p1 as the level set")
        return deform.Integrate(dt, mono, order=order)
    if vb == BND:
        region = getattr(meas, "definedon", None) if integrand is not None else levelset_domain.get("definedon")
        return _integrate_bnd(lset, dt, order, mono, mesh, defined, region)
    if isinstance(lset, (tuple, list)):
        return _integrate_mlset(lset, dt, order, mono, defined, mesh)
    subdivlvl = getattr(meas, "subdivlvl", 0) if integrand is not None else levelset_domain.get("subdivlvl", 0)
    if isinstance(lset, GridFunction) and not isinstance(lset.space, SpaceTimeFESpace) and lset.space.order > 1:
        # a level set that is not P1: the subdivision rule (the reference's
        # CutIntegrationRule path, cutint/xintegration.cpp:102-116)
        res = torch.zeros(1, dtype=torch.float64, device=_dev())
        _lib.call("xg_integrate_subdiv", lset.space.h, _vp(lset.vec), dt, order, int(subdivlvl or 0), mono.e[0],
                  mono.e[1], mono.e[2], _vp(defined.words) if defined is not None else None, _vp(res), _stream())
        device_mesh(lset.space.mesh).check()
        return float(res.item())
    mesh = mesh if mesh is not None else lset.space.mesh
    dm = device_mesh(mesh)
    res = torch.zeros(1, dtype=torch.float64, device=_dev())
    _lib.call("xg_integrate_ex", dm.h, _vp(_lset_vec(lset)), dt, order, int(policy), mono.e[0], mono.e[1],
              mono.e[2], _vp(defined.words) if defined is not None else None, _vp(res), _stream())
    dm.check()
    return float(res.item())


def _unscaled(meas):
    out = _Measure.__new__(_Measure)
    out.__dict__.update(meas.__dict__)
    out.scale = 1.0
    return out


def _bnd_restriction(mesh, defined, region):
    """The bitset over the BND elements of definedonelements (a BitArray over
    them) and definedon (mesh.Boundaries(...)), intersected; None for all."""
    dm = device_mesh(mesh)
    nb = np.zeros(1, dtype=np.int64)
    _lib.call("xg_mesh_boundary", dm.h, nb.ctypes.data_as(ctypes.c_void_p), None)
    nbnd = int(nb[0])
    if region is not None:
        if region.mesh is not mesh or len(region.mask) != nbnd:
            raise ValueError("definedon: a region of this mesh's BND elements (mesh.Boundaries)")
        r = BitArray.from_numpy(region.mask)
        defined = r if defined is None else defined & r
    if defined is not None and len(defined) != nbnd:
        raise ValueError("definedonelements on vb=BND: a BitArray over the %d BND elements" % nbnd)
    return defined


def _integrate_bnd(lset, dt, order, mono, mesh, defined=None, region=None):
    """Integrate(f * dCut(lset, dt, vb=BND[, definedon=mesh.Boundaries(..)]
    [, definedonelements=BND BitArray])): xg_integrate_bnd; the two
    restrictions intersect."""
    mesh = mesh if mesh is not None else lset.space.mesh
    dm = device_mesh(mesh)
    defined = _bnd_restriction(mesh, defined, region)
    res = torch.zeros(1, dtype=torch.float64, device=_dev())
    _lib.call("xg_integrate_bnd", dm.h, _vp(_lset_vec(lset)), dt, order, mono.e[0], mono.e[1], mono.e[2],
              _vp(defined.words) if defined is not None else None, _vp(res), _stream())
    dm.check()
    return float(res.item())


def _mlset_args(lsets, domain):
    """(device [M][nv] level-set values, host int8 [ntup][M] domain tuples)."""
    from .mlset import DomainTypeArray
    if not isinstance(domain, DomainTypeArray):
        domain = DomainTypeArray(list(domain) if isinstance(domain, list) else domain)
    M = len(lsets)
    if len(domain.as_list[0]) != M:
        raise ValueError("domain tuples of length %d for %d level sets" % (len(domain.as_list[0]), M))
    nv = lsets[0].space.mesh.nv
    if any(g.space.mesh is not lsets[0].space.mesh or _lset_vec(g).numel() < nv for g in lsets):
        raise ValueError("the level sets must be P1 GridFunctions on one mesh")
    vals = torch.stack([_lset_vec(g)[:nv] for g in lsets]).contiguous()
    tup = np.ascontiguousarray(np.array(domain.as_list, dtype=np.int8).reshape(-1, M))
    return vals, tup


def _integrate_mlset(lsets, domain, order, mono, defined, mesh):
    """Integrate over a region of several level sets
    (cutint/mlsetintegration.cpp:6-180): xg_integrate_mlset."""
    mesh = mesh if mesh is not None else lsets[0].space.mesh
    dm = device_mesh(mesh)
    vals, tup = _mlset_args(lsets, domain)
    res = torch.zeros(1, dtype=torch.float64, device=_dev())
    _lib.call("xg_integrate_mlset", dm.h, _vp(vals), vals.shape[0], tup.ctypes.data_as(ctypes.c_void_p),
              tup.shape[0], order, mono.e[0], mono.e[1], mono.e[2],
              _vp(defined.words) if defined is not None else None, _vp(res), _stream())
    dm.check()
    return float(res.item())


_TRI_EDGES = ((0, 1), (0, 2), (1, 2))
_TET_EDGES = ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))


def P2ElementValues(mesh, f):
    """(ne, (D+1)(D+2)/2) values of f (a callable on coordinate arrays) at each
    element's vertices, then edge midpoints: the P2 nodal values the
    isoparametric mapping takes."""
    X = mesh.coords[mesh.elements]  # ne x (D+1) x D
    pts = [X[:, v] for v in range(mesh.dim + 1)]
    pts += [0.5 * (X[:, a] + X[:, b]) for a, b in (_TRI_EDGES if mesh.dim == 2 else _TET_EDGES)]
    return np.stack([np.asarray(f(*[p[:, k] for k in range(mesh.dim)]), dtype=np.float64) for p in pts], axis=1)


class LevelSetMeshAdaptation:
    """Isoparametric integration for a P2 level set (python/lsetcurv.py:281-356:
    LevelSetMeshAdaptation + CalcDeformation + Integrate on the deformed mesh),
    on the GPU (xg_iso_integrate_mesh): per band element the shift of the
    order-4 rule points to the level set of the P2 function (Newton along the
    element's own gradient, discontinuous_qn), its L2 projection onto P2 with
    the vertex coefficients dropped, the edge coefficients averaged over the
    band elements, and the straight cut rule of the P1 interpolant mapped by
    the deformation.  order 2 only."""

    def __init__(self, mesh, order=2, threshold=-1.0, discontinuous_qn=True, **kwargs):
        if order != 2:
            raise NotImplementedError("the isoparametric mapping is built for order 2")
        if not discontinuous_qn:
            raise NotImplementedError("the search direction is the element's own gradient (discontinuous_qn=True)")
        self.mesh, self.threshold = mesh, float(threshold)
        self.p2 = None
        self.nonconverged = 0

    def CalcDeformation(self, levelset):
        """levelset: a callable on coordinate arrays, or (ne, nn) P2 element values."""
        vals = P2ElementValues(self.mesh, levelset) if callable(levelset) else np.asarray(levelset, np.float64)
        D = self.mesh.dim
        if getattr(self.mesh, "tensor", False) or vals.shape != (self.mesh.ne, (D + 1) * (D + 2) // 2):
            raise ValueError("P2 element values of shape (ne, %d) on a simplex mesh expected"
                             % ((D + 1) * (D + 2) // 2))
        self.p2 = torch.from_numpy(np.ascontiguousarray(vals)).to(_dev())
        self._gdef = None
        return self

    def _edge_deformation(self):
        """[nedges][3] physical edge coefficients of the deformation
        (xg_iso_deformation), computed once per CalcDeformation."""
        if self.p2 is None:
            raise RuntimeError("CalcDeformation first")
        if getattr(self, "_gdef", None) is None:
            dm = device_mesh(self.mesh)
            info = np.zeros(8, dtype=np.int64)
            _lib.call("xg_mesh_info", dm.h, info.ctypes.data_as(ctypes.c_void_p))
            gd = torch.zeros((int(info[3]), 3), dtype=torch.float64, device=_dev())
            nc = torch.zeros(1, dtype=torch.int32, device=_dev())
            _lib.call("xg_iso_deformation", dm.h, _vp(self.p2), ctypes.c_double(self.threshold), _vp(gd), _vp(nc),
                      _stream())
            dm.check()
            self.nonconverged = int(nc.item())
            self._gdef = gd
        return self._gdef

    @property
    def lset_p1(self):
        """The P1 level set of the deformed-mesh forms: the P2 level set's
        vertex values with the |v| < 1e-14 -> 1e-14 perturbation."""
        if self.p2 is None:
            raise RuntimeError("CalcDeformation first")
        D = self.mesh.dim
        vals = np.zeros(self.mesh.nv)
        p2 = self.p2.cpu().numpy()
        for i in range(D + 1):
            vals[self.mesh.elements[:, i]] = p2[:, i]
        vals = np.where(np.abs(vals) < 1e-14, 1e-14, vals)
        g = GridFunction(H1(self.mesh, order=1))
        g.vec.copy_(torch.from_numpy(vals))
        return g

    def Integrate(self, domain_type, cf=None, order=4, deform=True):
        if self.p2 is None:
            raise RuntimeError("CalcDeformation first")
        mono = cf if isinstance(cf, _Monomial) else _Monomial()
        dm = device_mesh(self.mesh)
        res = torch.zeros(1, dtype=torch.float64, device=_dev())
        nc = torch.zeros(1, dtype=torch.int32, device=_dev())
        _lib.call("xg_iso_integrate_mesh", dm.h, _vp(self.p2), domain_type, order, ctypes.c_double(self.threshold),
                  1 if deform else 0, mono.e[0], mono.e[1], mono.e[2], _vp(res), _vp(nc), _stream())
        dm.check()
        self.nonconverged = int(nc.item())
        return float(res.item())


def MultiLevelsetCutIntegrationRules(mesh, levelsets, domain, elements, order, max_pts=None):
    """The per-element rules of a region of several level sets
    (CreateMultiLevelsetCutIntegrationRule for listed elements): (counts,
    points (n, max_pts, 3), weights (n, max_pts)) as device tensors, counts
    -1 where the element has no part of the region."""
    dm = device_mesh(mesh)
    vals, tup = _mlset_args(levelsets, domain)
    el = torch.as_tensor(np.asarray(elements, dtype=np.int32)).to(_dev())
    n = el.numel()
    if max_pts is None:
        max_pts = _lib.load().xg_mlset_rule_capacity(mesh.dim, vals.shape[0], tup.shape[0], order)
    dev = _dev()
    counts = torch.zeros(n, dtype=torch.int32, device=dev)
    pts = torch.zeros((n, max_pts, 3), dtype=torch.float64, device=dev)
    wts = torch.zeros((n, max_pts), dtype=torch.float64, device=dev)
    _lib.call("xg_cut_rules_mlset", dm.h, _vp(vals), vals.shape[0], tup.ctypes.data_as(ctypes.c_void_p),
              tup.shape[0], _vp(el), n, order, max_pts, _vp(counts), _vp(pts), _vp(wts), _stream())
    dm.check()
    return counts, pts, wts


# ----------------------------------------------------------------------------
# rule export
# ----------------------------------------------------------------------------
def CutIntegrationRules(mesh, levelset, elements, domain_type, order, max_pts=None, quad_dir_policy=None):
    """StraightCutIntegrationRule for a list of elements; returns (counts,
    points (n, max_pts, 3), weights (n, max_pts)) as device tensors.  On
    quadrilateral / hexahedral meshes quad_dir_policy (FIRST, OPTIMAL,
    FALLBACK; default OPTIMAL) selects the direction of the tensor rule."""
    dm = device_mesh(mesh)
    el = torch.as_tensor(np.asarray(elements, dtype=np.int32)).to(_dev())
    n = el.numel()
    policy = OPTIMAL if quad_dir_policy is None else int(quad_dir_policy)
    if max_pts is None and getattr(mesh, "tensor", False):
        max_pts = _lib.load().xg_quad_rule_capacity(mesh.dim, domain_type, order)
    if max_pts is None:
        sd = mesh.dim - 1 if domain_type == IF else mesh.dim
        max_pts = max(3 * _lib.load().xg_base_rule_size(sd, order), _lib.load().xg_base_rule_size(mesh.dim, order))
    dev = _dev()
    counts = torch.zeros(n, dtype=torch.int32, device=dev)
    pts = torch.zeros((n, max_pts, 3), dtype=torch.float64, device=dev)
    wts = torch.zeros((n, max_pts), dtype=torch.float64, device=dev)
    _lib.call("xg_cut_rules_ex", dm.h, _vp(_lset_vec(levelset)), _vp(el), n, domain_type, order, policy, max_pts,
              _vp(counts), _vp(pts), _vp(wts), _stream())
    dm.check()
    return counts, pts, wts

"""Regions of several level sets (python/mlset.py of ngsxfem): a region is a
union of domain tuples, one entry per level set (NEG, POS or IF; ANY expands
to both NEG and POS).  A tuple with k IF entries describes a set of
codimension k.  Integrate(levelset_domain={"levelset": (gf_1, ..., gf_M),
"domain_type": <tuple | list of tuples | DomainTypeArray>}, ...) integrates
over the union on the GPU (xg_integrate_mlset).

Kept from the reference: ANY expansion, the set semantics of a region, union,
intersection (tuples of different codimension combine into the common
boundary: entries that differ between NEG / POS and IF become IF), the
complement among the tuples of the same codimension, Boundary() (an entry is
replaced by IF unless both of its volume neighbours belong to the region) and
Compress (tuples of zero measure for given level sets are dropped), and
GetOuterNormals (the unit normals of the boundary pieces, for the Nitsche
terms of a BilinearForm).  The CoefficientFunction helpers Indicator and
IndicatorSmoothed have no counterpart here.  The tuples are kept sorted, so
the integration order is fixed.
"""
from itertools import product

from .xfem import ANY, IF, NEG, POS

_VOL = (NEG, POS)


def _expand(dtt):
    """All NEG / POS fillings of the ANY entries of one tuple."""
    slots = [(dt,) if dt != ANY else _VOL for dt in dtt]
    return [tuple(c) for c in product(*slots)]


class DomainTypeArray:
    def __init__(self, dtlist, lsets=None, persistent_compress=False, do_safety_checks=True):
        if isinstance(dtlist, tuple):
            dtlist = [dtlist]
        if not isinstance(dtlist, list) or not dtlist or not isinstance(dtlist[0], tuple):
            raise TypeError("Invalid input: dtlist must be a tuple or a list of tuples")
        n = len(dtlist[0])
        self.codim = sum(1 for dt in dtlist[0] if dt == IF)
        if do_safety_checks:
            for dtt in dtlist:
                if len(dtt) != n:
                    raise ValueError("DomainTypeArray initialised with tuples of different length")
                if any(dt not in (NEG, POS, IF, ANY) for dt in dtt):
                    raise ValueError("DomainTypeArray entries must be NEG, POS, IF or ANY")
                if dtt.count(IF) != self.codim:
                    raise ValueError("DomainTypeArray initialised with tuples of different co-dimension")
            if lsets is not None and len(lsets) != n:
                raise ValueError("the number of level sets does not match the length of the domain tuples")
        tuples = set()
        for dtt in dtlist:
            tuples.update(_expand(dtt))
        self.as_list = sorted(tuples)
        self.lsets = lsets
        self.persistent_compress = persistent_compress
        if lsets is not None:
            self.Compress(lsets, persistent_compress)
        if not persistent_compress:
            self.lsets = None

    # ---- container protocol ----
    def __len__(self):
        return len(self.as_list)

    def __iter__(self):
        return iter(self.as_list)

    def __contains__(self, dtt):
        return dtt in self.as_list

    def __eq__(self, other):
        return isinstance(other, DomainTypeArray) and self.codim == other.codim and \
            sorted(self.as_list) == sorted(other.as_list)

    def __ne__(self, other):
        return not self.__eq__(other)

    def __str__(self):
        return "DomainTypeArray:\n  Co-dim : %d\n  Domains: [%s]" % (
            self.codim, ", ".join(str(t) for t in self.as_list))

    def _combined_compression(self, other):
        if self.persistent_compress and other.persistent_compress:
            if any(a is not b for a, b in zip(self.lsets, other.lsets)):
                raise ValueError("operator only possible for domains with the same level sets")
            return self.lsets, True
        return None, False

    # ---- region algebra ----
    def __or__(self, other):
        if self.codim != other.codim:
            raise ValueError("co-dimensions don't match: union not possible")
        lsets, pers = self._combined_compression(other)
        return DomainTypeArray(self.as_list + other.as_list, lsets, pers)

    def __and__(self, other):
        lsets, pers = self._combined_compression(other)
        out = [t for t in self.as_list if t in other.as_list]
        if not out:
            for a, b in product(self.as_list, other.as_list):
                comb = []
                for x, y in zip(a, b):
                    if x == y:
                        comb.append(x)
                    elif x in _VOL and y in _VOL:
                        break  # NEG against POS: empty
                    else:
                        comb.append(IF)
                else:
                    out.append(tuple(comb))
        if not out:
            raise ValueError("empty intersection")
        return DomainTypeArray(out, lsets, pers)

    def __invert__(self):
        n = len(self.as_list[0])
        alphabet = _VOL if self.codim == 0 else (NEG, POS, IF)
        mine = set(self.as_list)
        rest = [t for t in product(alphabet, repeat=n) if t.count(IF) == self.codim and t not in mine]
        return DomainTypeArray(rest, self.lsets, self.persistent_compress)

    def __ior__(self, other):
        return self.__or__(other)

    def __iand__(self, other):
        return self.__and__(other)

    # ---- with level sets ----
    def Compress(self, lsets, persistent=False):
        """Drops the tuples whose region has zero measure (|integral of 1| <=
        1e-12 at order 0) for the given level sets."""
        from .xfem import Integrate
        if len(lsets) != len(self.as_list[0]):
            raise ValueError("the number of level sets does not match the length of the domain tuples")
        mesh = lsets[0].space.mesh
        self.as_list = [t for t in self.as_list
                        if abs(Integrate({"levelset": tuple(lsets), "domain_type": t}, cf=None, mesh=mesh,
                                         order=0)) > 1e-12]
        if persistent:
            self.persistent_compress = True
            self.lsets = lsets

    def Boundary(self):
        """The boundary of the region: each entry replaced by IF unless both
        of its volume neighbours belong to the region (and, with attached
        level sets, unless the piece has zero measure)."""
        if self.codim >= 3:
            raise ValueError("Boundary does not make sense for codim >= 3")
        from .xfem import Integrate
        out = []
        for dtt in self.as_list:
            for i, dt in enumerate(dtt):
                if dt == IF:
                    continue
                if dtt[:i] + (POS,) + dtt[i + 1:] in self and dtt[:i] + (NEG,) + dtt[i + 1:] in self:
                    continue
                cand = dtt[:i] + (IF,) + dtt[i + 1:]
                if self.lsets is not None:
                    w = Integrate({"levelset": tuple(self.lsets), "domain_type": cand}, cf=None,
                                  mesh=self.lsets[0].space.mesh, order=0)
                    if abs(w) < 1e-12:
                        continue
                out.append(cand)
        if self.persistent_compress:
            return DomainTypeArray(out, self.lsets, True)
        return DomainTypeArray(out)


def _outer_normals(self, lsets):
    """For each piece of self.Boundary() the outward unit normal
    (python/mlset.py GetOuterNormals): Normalize(grad(l_i)) of the level set
    whose entry is IF on the piece, negated where the region is POS in it."""
    from .xfem import Normalize, grad
    if self.codim > 0:
        raise NotImplementedError("GetOuterNormals is available for codim = 0")
    out = {}
    bnd = self.Boundary()
    for dtt in self.as_list:
        for i, dt in enumerate(dtt):
            piece = dtt[:i] + (IF,) + dtt[i + 1:]
            if piece not in bnd:
                continue
            n = Normalize(grad(lsets[i]))
            out[piece] = -1.0 * n if dt == POS else n
    return out


DomainTypeArray.GetOuterNormals = _outer_normals


def TensorUnion(*args):
    """Union of regions of disjoint sets of level sets (the other level sets'
    entries ANY): the tuples grow to the total number of level sets."""
    codim = args[0].codim
    widths = []
    for dta in args:
        if not isinstance(dta, DomainTypeArray):
            raise TypeError("TensorUnion only possible for DomainTypeArrays")
        if dta.codim != codim:
            raise ValueError("cannot form TensorUnion for arrays of different codimension")
        widths.append(len(dta.as_list[0]))
    total, start, out = sum(widths), 0, []
    for w, dta in zip(widths, args):
        for dtt in dta.as_list:
            t = [ANY] * total
            t[start:start + w] = dtt
            out.append(tuple(t))
        start += w
    return DomainTypeArray(out)


def TensorIntersection(*args):
    """Intersection of regions of disjoint sets of level sets: every
    combination of their tuples, concatenated."""
    for dta in args:
        if not isinstance(dta, DomainTypeArray):
            raise TypeError("TensorIntersection only possible for DomainTypeArrays")
    return DomainTypeArray([sum(c, ()) for c in product(*[dta.as_list for dta in args])])


class MultiLevelsetCutInfo:
    """Element markers of regions of several level sets
    (MultiLevelsetCutInformation, xfem/cutinfo.cpp:286-419): the level sets are
    copied at construction and by Update(); every marker handed out is kept
    and recomputed in place by Update()."""

    def __init__(self, mesh, levelset):
        from .xfem import device_mesh
        self.mesh = mesh
        lsets = self._check(levelset)
        self.M = len(lsets)
        self._dm = device_mesh(mesh)
        self._vals = self._copy(lsets)
        self._markers = []  # (mode, int8 tuples, BitArray)

    @staticmethod
    def _check(levelset):
        from .xfem import GridFunction
        if not isinstance(levelset, (tuple, list)) or not all(isinstance(g, GridFunction) for g in levelset):
            raise TypeError("MultiLevelsetCutInfo needs a tuple of P1 GridFunctions")
        return tuple(levelset)

    def _copy(self, lsets):
        import torch
        from .xfem import _lset_vec
        return torch.stack([_lset_vec(g)[: self.mesh.nv] for g in lsets]).clone().contiguous()

    def Mesh(self):
        return self.mesh

    def _tuples(self, domain):
        import numpy as np
        if not isinstance(domain, DomainTypeArray):
            domain = DomainTypeArray(list(domain) if isinstance(domain, list) else domain)
        if len(domain.as_list[0]) != self.M:
            raise ValueError("domain tuples of length %d for %d level sets" % (len(domain.as_list[0]), self.M))
        return np.ascontiguousarray(np.array(domain.as_list, dtype=np.int8).reshape(-1, self.M))

    def _mark(self, mode, tup, bits):
        import ctypes
        from . import _lib
        from .xfem import _stream, _vp
        _lib.call("xg_mlset_mark", self._dm.h, _vp(self._vals), self.M, tup.ctypes.data_as(ctypes.c_void_p),
                  tup.shape[0], mode, _vp(bits.words), _stream())
        self._dm.check()

    def _get(self, mode, domain):
        from .xfem import BitArray
        tup = self._tuples(domain)
        key = sorted(map(tuple, tup.tolist()))
        for m, t, bits in self._markers:
            if m == mode and sorted(map(tuple, t.tolist())) == key:
                return bits
        bits = BitArray(self.mesh.ne)
        self._mark(mode, tup, bits)
        self._markers.append((mode, tup, bits))
        return bits

    def GetElementsOfType(self, domain_type):
        """Elements whose level-set domain types equal one of the tuples."""
        return self._get(0, domain_type)

    def GetElementsWithContribution(self, domain_type):
        """Elements on which the region has a part of positive measure."""
        return self._get(1, domain_type)

    def Update(self, levelset):
        lsets = self._check(levelset)
        if len(lsets) != self.M:
            raise ValueError("the new level sets must be as many as the original ones")
        self._vals.copy_(self._copy(lsets))
        for mode, tup, bits in self._markers:
            self._mark(mode, tup, bits)

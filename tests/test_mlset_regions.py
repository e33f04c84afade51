"""Region algebra of ngsxfem_gb300.mlset against the expected sets of
ngsxfem's tests/pytests/test_mlset_module_functionality.py (complement,
boundary, union, intersection into interfaces, ANY expansion, tensor union and
intersection).  Pure Python, CPU."""
import pytest

from ngsxfem_gb300.mlset import DomainTypeArray as R
from ngsxfem_gb300.mlset import TensorIntersection, TensorUnion
from ngsxfem_gb300.xfem import ANY, IF, NEG, POS


def test_triangle_of_three_level_sets():
    tri = R([(NEG, NEG, NEG)])
    assert ~tri == R([(NEG, NEG, POS), (NEG, POS, NEG), (NEG, POS, POS), (POS, NEG, NEG), (POS, NEG, POS),
                      (POS, POS, NEG), (POS, POS, POS)])
    sides = tri.Boundary()
    assert sides == R([(IF, NEG, NEG), (NEG, IF, NEG), (NEG, NEG, IF)]) and sides.codim == 1
    assert (sides | sides) == sides and (sides & sides) == sides
    corners = sides.Boundary()
    assert corners == R([(IF, IF, NEG), (NEG, IF, IF), (IF, NEG, IF)]) and corners.codim == 2


def test_union_intersection_complement():
    a, b = R((POS, NEG)), R((POS, POS))
    u = a | b
    assert (POS, NEG) in u and (POS, POS) in u and len(u) == 2
    u |= R([(NEG, POS)])
    assert u == R([(POS, NEG), (POS, POS), (NEG, POS)])
    assert (u & a) == R([(POS, NEG)])
    u &= a | b
    assert u == R([(POS, NEG), (POS, POS)])
    assert ~u == R([(NEG, POS), (NEG, NEG)])
    # a volume and a side meet on the side; two sides meet on their corner
    s = R([(IF, NEG)]) & R([(POS, NEG)])
    assert s == R([(IF, NEG)])
    s &= R([(POS, IF)])
    assert s == R([(IF, IF)])
    line = R([(IF, NEG, POS)])
    line &= R([(POS, IF, POS)])
    assert ~line == R([(IF, NEG, IF), (POS, IF, IF), (IF, POS, IF), (NEG, IF, IF), (IF, IF, NEG)])
    assert R([(NEG, NEG, NEG)]).Boundary() == R([(NEG, IF, NEG), (NEG, NEG, IF), (IF, NEG, NEG)])
    assert R([(POS, IF, NEG)]).Boundary() == R([(POS, IF, IF), (IF, IF, NEG)])


def test_any_expansion():
    assert R((NEG, ANY, ANY)) == R([(NEG, NEG, NEG), (NEG, NEG, POS), (NEG, POS, NEG), (NEG, POS, POS)])
    assert R([(NEG, ANY, ANY), (POS, ANY, ANY)]) == R([(ANY, ANY, ANY)])
    assert R([(IF, ANY, ANY), (POS, IF, ANY)]) == R([(IF, NEG, NEG), (IF, NEG, POS), (IF, POS, NEG), (IF, POS, POS),
                                                     (POS, IF, NEG), (POS, IF, POS)])


def test_tensor_union_and_intersection():
    one, two, three = R((POS,)), R([(POS, NEG), (POS, POS)]), R((NEG, NEG, IF))
    assert TensorUnion(one, two) == R([(POS, ANY, ANY), (ANY, POS, NEG), (ANY, POS, POS)])
    with pytest.raises(Exception):
        TensorUnion(one, two, three)  # different codimensions
    assert TensorIntersection(one, two) == R([(POS, POS, NEG), (POS, POS, POS)])
    assert TensorIntersection(one, two, three) == R([(POS, POS, NEG, NEG, NEG, IF), (POS, POS, POS, NEG, NEG, IF)])

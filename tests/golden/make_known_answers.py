"""Writes known_answers.json: the closed-form values ngsxfem's own tests assert
for the straight-cut path (tests/pytests/test_straightcutrule.py,
tests/pytests/test_spacetimecutrule.py, tests/pytests/test_quadchallenges.py,
tests/pytests/test_mlset_integration.py, tests/pytests/test_bndcut.py).  The reference cannot run here (it
needs NGSolve), so these closed forms are the golden vectors the oracle is
pinned against.  Run: python tests/golden/make_known_answers.py
"""
import json
import math
import os

out = {
    "source": "ngsxfem tests/pytests/test_straightcutrule.py, test_spacetimecutrule.py",
    "planar2d": {  # test_straightcutrule.py:106-126, lset 1-2x-2y on [0,1]^2
        "lset": [1.0, -2.0, -2.0, 0.0], "N": [1, 10, 30], "orders": [2, 4, 8],
        "values": {"NEG": 7 / 8, "POS": 1 / 8, "IF": 1 / math.sqrt(2)}, "tol": "5e-15*(order+1)^2"},
    "planar3d": {  # :187-207, lset 1-2x-2y-2z on [0,1]^3
        "lset": [1.0, -2.0, -2.0, -2.0], "N": [1], "orders": [2, 4, 8],
        "values": {"NEG": 47 / 48, "POS": 1 / 48, "IF": math.sqrt(3) / 8}, "tol": "5e-15*(order+1)^2"},
    "mono2d": [  # :157-185, x^alpha / y^alpha on the planar 2D cut, orders 2,4,8
        {"alpha": a, "POS": 2 ** (-a - 2) / (a * a + 3 * a + 2),
         "NEG": 1 / (a + 1) - 2 ** (-a - 2) / (a * a + 3 * a + 2)} for a in (0, 1, 2)],
    "mono3d": [  # :209-235, order 4
        {"alpha": a, "POS": 2 ** (-a - 3) / (a ** 3 + 6 * a * a + 11 * a + 6),
         "NEG": 1 / (a + 1) - 2 ** (-a - 3) / (a ** 3 + 6 * a * a + 11 * a + 6)} for a in (0, 1, 2)],
    "orth2d": {  # :237-280, lset 1-2x+eps(y-1/2), N=1, order 2
        "eps": [1e-1, 1e-2, 5e-3, 1e-3, 0.0],
        "NEG": 0.5, "POS": 0.5, "IF": "sqrt(1+eps^2/4)"},
    "circle_eoc": {  # :33-68, sqrt(x^2+y^2)-0.6 on [0,1]^2, mean EOC > 1.75
        "r": 0.6, "NEG": math.pi * 0.36 / 4, "POS": 1 - math.pi * 0.36 / 4, "IF": 0.6 * math.pi / 2,
        "min_mean_eoc": 1.75},
    # quadrilaterals / hexahedra (the same files, quad=True / hexes=True, and
    # tests/pytests/test_quadchallenges.py)
    "orth_axis2d": {  # test_straightcutrule.py:237-257, lset 1-3x (or 1-3y), N=1, order 2
        "slope": 3.0, "NEG": 2 / 3, "POS": 1 / 3, "IF": 1.0},
    "orth_axis3d": {  # :260-279, lset 1-2x (y, z), N=1, order 2
        "slope": 2.0, "NEG": 0.5, "POS": 0.5, "IF": 1.0},
    "sphere_eoc": {  # :70-104, sqrt(x^2+y^2+z^2)-r on [0,1]^3 hexes 2^i, i<6, orders 2,4
        "r": 0.7234436998, "NEG": math.pi * 0.7234436998 ** 3 / 6, "POS": 1 - math.pi * 0.7234436998 ** 3 / 6,
        "orders": [2, 4], "n_ref": 6, "min_mean_eoc": 1.75},
    "quad3d_planar": {  # test_quadchallenges.py:8-28: planar3d on 2x2x2 hexes, orders 2,4,8
        "N": 2, "orders": [2, 4, 8]},
    "quad3d_mono": {  # test_quadchallenges.py:31-57: mono3d on 5x5x5 hexes, order 4, OPTIMAL
        "N": 5, "order": 4},
    "zero_val": {  # test_quadchallenges.py:59-79: 2x2x2 hexes, POS, x^2, order 4, OPTIMAL
        "N": 2, "order": 4, "alpha": 2, "POS": 2 ** (-5) / (8 + 24 + 22 + 6)},
    "tpmc_hex": {  # test_quadchallenges.py:81-103: one hex, vertex values by vertex number of a
        # mesh numbered z fastest (vertex 4x+2y+z), orders 2,4,6
        "vals": [-4, 4, -1, -1, 2, -3, 5, -1], "orders": [2, 4, 6],
        "NEG": 0.5167820912197415, "POS": 0.4825797907263282, "tol": 0.75, "IF_below": 10.0},
    "tpmc_10": {  # test_quadchallenges.py:105-141: phi = x((7y-13)z+6) + y(3-8z) + 8z - 4
        # on 10x10x10 hexes (interpolated exactly), orders 2,4
        "orders": [2, 4], "NEG": 0.51681, "POS": 0.48319, "IF": 1.82169, "tol_vol": 1e-3, "tol_if": 5e-3},
    # several level sets (tests/pytests/test_mlset_integration.py)
    "mlset2d": {  # :38-128, level sets y-1, 2x-y, -2x-y on [-1,1]x[-0.5,1.5], order 0
        "box": [[-1.0, 1.0], [-0.5, 1.5]],
        "area_neg0": 3.0, "triangle": 0.5, "complement": 3.5,
        "side_t": 1.0, "side_r": math.sqrt(5 / 4), "side_l": math.sqrt(5 / 4), "perimeter": 1 + math.sqrt(5),
        "x_plus_y": {"tl": 1.5, "tr": 0.5, "b": 0.0, "corners": 2.0}, "tol": 1e-12},
    "mlset2d_ho": {  # :131-153, -y, x-1, y-1, -x on [-0.2,1.2]^2, x(1-x)y(1-y), order 4
        "box": [[-0.2, 1.2], [-0.2, 1.2]], "value": 1 / 36, "tol": 1e-12},
    "mlset3d": {  # :289-395, x -+ 0.5, y -+ 0.5, z -+ 0.5 on [-0.8,0.8]^3, order 0
        "box": [-0.8, 0.8], "cube": 1.0, "complement": 1.6 ** 3 - 1.0, "side": 1.0, "surface": 6.0,
        "edge": 1.0, "edges": 12.0,
        "corners_x_plus_y_plus_z": {"ppp": 1.5, "ppn": 0.5, "pnp": 0.5, "npp": 0.5, "pnn": -0.5, "npn": -0.5,
                                    "nnp": -0.5, "nnn": -1.5}, "tol": 1e-12},
    "mlset3d_lines": {  # test_mlset_integration.py:398-470, lines (codimension 2) in [-0.8,0.8]^3
        "line": math.sqrt(2), "cross": 2 * math.sqrt(3), "lines": 1.9 * math.sqrt(3), "tol": 1e-12},
    # boundary cut integrals (tests/pytests/test_bndcut.py), lset x - cut on the unit square / cube
    "bnd2d": {"cuts": [0.3, 0.5, 0.7], "NEG": "2 cut + 1", "IF_points": 2.0,
              "if_x_at_half": 1.0, "if_y_at_half": 1.0, "perimeter": 4.0, "tol": 1e-10},
    "bnd3d": {"cut": 0.3, "NEG": 1.0 + 4.0 * 0.3, "tol": 1e-10},
    # definedon=mesh.Boundaries(side) (test_bndcut.py:51-59, 203-217): NEG on the bottom side = cut;
    # interface points on the bottom side at cut 0.5: 1, on the left side: 0
    "bnd2d_definedon": {"cuts": [0.3, 0.7], "bottom_NEG": "cut", "bottom_IF_at_half": 1.0,
                        "left_IF_at_half": 0.0, "tol": 1e-10},
}
path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json")
with open(path, "w") as f:
    json.dump(out, f, indent=1)
print(path)

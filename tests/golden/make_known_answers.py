"""Writes known_answers.json: the closed-form values ngsxfem's own tests assert
for the straight-cut path (tests/pytests/test_straightcutrule.py,
tests/pytests/test_spacetimecutrule.py).  The reference cannot run here (it
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
}
path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json")
with open(path, "w") as f:
    json.dump(out, f, indent=1)
print(path)

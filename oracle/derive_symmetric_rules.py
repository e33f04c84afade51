"""Derives the fully symmetric simplex rules of the rule family by solving
their moment equations (Newton / least squares in 50-digit arithmetic):

  trig degree 4: S21(a1) w1 + S21(a2) w2                      (6 points)
  trig degree 5: S3 w0 + S21(a1) w1 + S21(a2) w2              (7 points)
  tet  degree 5: S31(a1) w1 + S31(a2) w2 + S22(c) w3          (14 points)

S21(a): barycentric (a, a, 1-2a) and permutations; S31(a): (a, a, a, 1-3a);
S22(c): (c, c, 1/2-c, 1/2-c).  Weights sum to the reference measure (1/2, 1/6).
The printed literals are embedded in oracle/xg_oracle.cpp and
ngsxfem_gb300/csrc/xg_host.cpp.  Run: python oracle/derive_symmetric_rules.py
"""
import itertools

import mpmath as mp

mp.mp.dps = 50


def orbit(lam):
    return sorted(set(itertools.permutations(lam)))


def exact(d, exps):
    num = mp.mpf(1)
    for e in exps:
        num *= mp.factorial(e)
    return num / mp.factorial(sum(exps) + d)


def residual(d, deg, build):
    def f(*params):
        pts = build(*params)
        res = []
        for exps in itertools.product(range(deg + 1), repeat=d):
            if sum(exps) > deg:
                continue
            s = mp.mpf(0)
            for lam, w in pts:
                t = w
                for k in range(d):
                    t *= lam[k] ** exps[k]
                s += t
            res.append(s - exact(d, exps))
        return res
    return f


def solve(d, deg, build, x0):
    f = residual(d, deg, build)
    x = mp.matrix(x0)
    for it in range(100):
        r = mp.matrix(f(*x))
        J = mp.matrix(len(r), len(x))
        h = mp.mpf(10) ** -30
        for j in range(len(x)):
            xp = x.copy()
            xp[j] += h
            rp = mp.matrix(f(*xp))
            for i in range(len(r)):
                J[i, j] = (rp[i] - r[i]) / h
        dx = mp.lu_solve(J.T * J, J.T * r)
        x -= dx
        if mp.norm(dx) < mp.mpf(10) ** -45:
            break
    return x, mp.norm(mp.matrix(f(*x)))


def trig4(a1, a2, w1, w2):
    return [(p, w1) for p in orbit((a1, a1, 1 - 2 * a1))] + [(p, w2) for p in orbit((a2, a2, 1 - 2 * a2))]


def trig5(a1, a2, w0, w1, w2):
    c = mp.mpf(1) / 3
    return [((c, c, c), w0)] + trig4(a1, a2, w1, w2)


def tet5(a1, a2, c, w1, w2, w3):
    return ([(p, w1) for p in orbit((a1, a1, a1, 1 - 3 * a1))] + [(p, w2) for p in orbit((a2, a2, a2, 1 - 3 * a2))] +
            [(p, w3) for p in orbit((c, c, mp.mpf(1) / 2 - c, mp.mpf(1) / 2 - c))])


def show(name, build, x, res):
    print("%s  residual %s" % (name, mp.nstr(res, 5)))
    for lam, w in build(*x):
        print("  %s  w=%s" % (", ".join(mp.nstr(v, 20) for v in lam), mp.nstr(w, 20)))
    print("  params:", [mp.nstr(v, 20) for v in x])


if __name__ == "__main__":
    x, r = solve(2, 4, lambda a1, a2, w1, w2: [(l[:2], w) for l, w in trig4(a1, a2, w1, w2)],
                 [0.44, 0.09, 0.11, 0.055])
    show("trig deg4", trig4, x, r)
    x, r = solve(2, 5, lambda *p: [(l[:2], w) for l, w in trig5(*p)], [0.47, 0.10, 0.11, 0.066, 0.063])
    show("trig deg5", trig5, x, r)
    x, r = solve(3, 5, lambda *p: [(l[:3], w) for l, w in tet5(*p)], [0.0927, 0.3108, 0.4544, 0.0122, 0.0187, 0.0071])
    show("tet deg5", tet5, x, r)

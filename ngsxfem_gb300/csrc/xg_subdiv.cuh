// Subdivision cut rules of a higher-order level set, host and device.
//
// Follows ngsxfem's CutIntegrationRule with subdivlvl
// (cutint/xintegration.cpp:1626-1754) and
// NumericalIntegrationStrategy<ET_TRIG / ET_TET, ET_POINT>::MakeQuadRule
// (:757-1063):
//   CheckIfCut (:620-751)   the level set's signs at the lattice of a simplex
//                           with spacing 1/2^L (>= 0 counts as positive; the
//                           reference's distance threshold is left at 1e99
//                           by CutIntegrationRule, so it never decides)
//   refinement (:820-914)   the reference's children of a cut simplex, down
//                           to level 0
//   level 0 (:925-988)      the vertex signs (Simplex::CheckIfCut,
//                           xdecompose.hpp:34-80: a side holding less than
//                           1e-14 of sum |l| does not count) and, if cut, the
//                           straight cut of the linear interpolant
//                           (CutSimplex::MakeQuad); a vertex value of 0 is
//                           positive and is cut against its negative
//                           neighbours at the vertex
// The reference refines breadth by recursion; here a thread walks the same
// tree (or one subtree of it) depth first with an explicit stack (children in
// order) and hands every rule point to a callback, on the physical image of
// each simplex, so points are physical and weights are physical measures
// (NEG / POS volumes, IF surface measure).
#pragma once
#include "xg_basis.cuh"
#include "xg_quadcut.cuh"

namespace xg {
namespace sd {

constexpr int kMaxLevels = 6;

// a level set of order K on one element and the element's affine map
template <int D, int K>
struct Elem {
  static constexpr int N = ndof_el(D, K);
  double x0[3];      // x = x0 + F xi (x0 = vertex D)
  double F[3][3];
  double coef[N];    // coefficients in the H1 basis (xg_basis.cuh)
  int desc[N];       // the basis functions (fn_desc, with the element's edge orientation)
};

template <int D, int K>
XG_QHD double lset_at(const Elem<D, K>& el, const double* xi) {
  double lam[D + 1], s = 0.0;
  for (int i = 0; i < D; i++) {
    lam[i] = xi[i];
    s += xi[i];
  }
  lam[D] = 1.0 - s;
  double v = 0.0;
  for (int i = 0; i < Elem<D, K>::N; i++) v += el.coef[i] * eval_fn_value<D, double>(el.desc[i], lam);
  return v;
}

// lattice point of index I (spacing 1/2^L) of simplex v
template <int D>
XG_QHD void lattice_point(const double (*v)[3], const int* I, double dx, double* xi) {
  for (int d = 0; d < 3; d++) xi[d] = d < D ? v[0][d] : 0.0;
  for (int j = 0; j < D; j++)
    for (int d = 0; d < D; d++) xi[d] += I[j] * dx * (v[j + 1][d] - v[0][d]);
}

// CheckIfCut on the lattice of simplex v (reference coordinates) at level L
template <int D, int K>
XG_QHD int lattice_domain(const Elem<D, K>& el, const double (*v)[3], int L) {
  const int np = 1 << L;
  const double dx = 1.0 / np;
  bool pos = false, neg = false;
  int I[3] = {0, 0, 0};
  for (;;) {
    double xi[3];
    lattice_point<D>(v, I, dx, xi);
    if (lset_at(el, xi) >= 0.0) pos = true;
    else neg = true;
    if (pos && neg) return XG_IF;
    I[0]++;
    int c = 0;
    while (c < D) {
      int sum = 0;
      for (int i = 0; i < D; i++) sum += I[i];
      if (sum <= np) break;
      if (c == D - 1) return pos ? XG_POS : XG_NEG;
      I[c] = 0;
      I[c + 1]++;
      c++;
    }
  }
}

// Simplex::CheckIfCut on the vertex values
XG_QHD int vertex_domain(const double* l, int n) {
  bool pos = false, neg = false;
  double sp = 0.0, sn = 0.0;
  for (int i = 0; i < n; i++) {
    if (l[i] >= 0.0) {
      sp += l[i];
      pos = true;
    } else {
      sn -= l[i];
      neg = true;
    }
  }
  const double s = sp + sn;
  if (sp / s < 1e-14) pos = false;
  if (sn / s < 1e-14) neg = false;
  if (pos && neg) return XG_IF;
  return pos ? XG_POS : (neg ? XG_NEG : XG_POS);
}

// child c of the simplex v: the reference's barycentric points (weights on
// the parent's vertices) and children (xintegration.cpp:826-841, 896-906)
template <int D>
XG_QHD void child(const double (*v)[3], int c, double (*w)[3]) {
  // 2D: points (0,0,1) (.5,0,.5) (1,0,0) (0,.5,.5) (.5,.5,0) (0,1,0)
  // 3D: points (0,0,0,1) (.5,0,0,.5) (1,0,0,0) (0,.5,0,.5) (.5,.5,0,0) (0,1,0,0)
  //            (0,0,.5,.5) (.5,0,.5,0) (0,.5,.5,0) (0,0,1,0)
  const signed char P2[6][2] = {{2, 2}, {0, 2}, {0, 0}, {1, 2}, {0, 1}, {1, 1}};  // midpoint of vertices (a, b)
  const signed char P3[10][2] = {{3, 3}, {0, 3}, {0, 0}, {1, 3}, {0, 1}, {1, 1}, {2, 3}, {0, 2}, {1, 2}, {2, 2}};
  const signed char K2[4][3] = {{0, 1, 3}, {1, 2, 4}, {1, 3, 4}, {3, 4, 5}};
  const signed char K3[8][4] = {{1, 2, 4, 7}, {3, 4, 5, 8}, {6, 7, 8, 9}, {3, 4, 8, 6},
                                {3, 4, 1, 6}, {0, 1, 3, 6}, {8, 6, 1, 7}, {8, 4, 1, 7}};
  for (int j = 0; j <= D; j++) {
    const int pt = D == 2 ? K2[c][j] : K3[c][j];
    const int a = D == 2 ? P2[pt][0] : P3[pt][0], b = D == 2 ? P2[pt][1] : P3[pt][1];
    for (int r = 0; r < 3; r++) w[j][r] = r < D ? 0.5 * v[a][r] + 0.5 * v[b][r] : 0.0;
  }
}

// the plain rule (l == nullptr) or the straight cut of the vertex values l on
// the physical image of the reference-coordinate simplex v
template <int D, int K, class E>
XG_QNI int fill(const RuleTable* Rp, const Elem<D, K>& el, const double (*v)[3], const double* l, int dt, int order,
                E& emit) {
  qc::Pt s[4];
  for (int i = 0; i <= D; i++)
    for (int r = 0; r < 3; r++) {
      double x = r < D ? el.x0[r] : 0.0;
      if (r < D)
        for (int c = 0; c < D; c++) x += el.F[r][c] * v[i][c];
      s[i].x[r] = x;
    }
  if (!l) {
    qc::qsimplex_plain(Rp, s, D + 1, order, emit);
    return 0;
  }
  double lc[4];
  for (int i = 0; i <= D; i++) lc[i] = l[i] == 0.0 ? 2.2250738585072014e-308 : l[i];
  return qc::qcut_simplex<D>(Rp, s, lc, dt, order, emit);
}

// the rule of the sub-simplex v (reference coordinates) of an element at
// refinement level L: emit(physical point, physical weight) per point;
// returns 0 or the first xg error of a cut
template <int D, int K, class E>
XG_QNI int node_rule(const RuleTable* Rp, const Elem<D, K>& el, const double (*v)[3], int L, int dt, int order,
                     E& emit) {
  struct Frame {
    double v[4][3];
    int L, next;
  };
  Frame st[kMaxLevels + 1];
  int sp = 1;
  for (int i = 0; i < 4; i++)
    for (int r = 0; r < 3; r++) st[0].v[i][r] = v[i][r];
  st[0].L = L;
  st[0].next = -1;
  int status = 0;
  while (sp > 0) {
    Frame& f = st[sp - 1];
    if (f.next < 0) {
      const int dself = lattice_domain(el, f.v, f.L);
      if (dself != XG_IF || f.L == 0) {
        if (dself != XG_IF) {
          if (dself == dt) fill(Rp, el, f.v, (const double*)nullptr, dt, order, emit);
        } else {
          double l[4];
          for (int i = 0; i <= D; i++) l[i] = lset_at(el, f.v[i]);
          const int dv = vertex_domain(l, D + 1);
          if (dv == XG_IF) {
            const int s2 = fill(Rp, el, f.v, l, dt, order, emit);
            if (s2 && !status) status = s2;
          } else if (dv == dt) {
            fill(Rp, el, f.v, (const double*)nullptr, dt, order, emit);
          }
        }
        sp--;
        continue;
      }
      f.next = 0;
    }
    if (f.next >= (D == 2 ? 4 : 8)) {
      sp--;
      continue;
    }
    Frame& c = st[sp];
    child<D>(f.v, f.next, c.v);
    f.next++;
    c.L = f.L - 1;
    c.next = -1;
    sp++;
  }
  return status;
}

// the reference simplex (1,0,0),(0,1,0),(0,0,1),(0,0,0) (first D+1 rows)
XG_QHD void ref_simplex(int D, double (*v)[3]) {
  for (int i = 0; i < 4; i++)
    for (int r = 0; r < 3; r++) v[i][r] = (i < D && r == i) ? 1.0 : 0.0;
}

// the rule of one element (the whole refinement tree from level `levels`)
template <int D, int K, class E>
XG_QNI int element_rule(const RuleTable* Rp, const Elem<D, K>& el, int dt, int order, int levels, E& emit) {
  double v[4][3];
  ref_simplex(D, v);
  return node_rule(Rp, el, v, levels, dt, order, emit);
}

}  // namespace sd
}  // namespace xg

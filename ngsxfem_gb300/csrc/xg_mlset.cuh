// Straight-cut rules of several level sets on simplices, host and device.
//
// Follows ngsxfem:
//   cutint/straightcutrule.cpp:679-812   StraightCutsIntegrationRule
//   cutint/straightcutrule.cpp:41-64, 131-204  the cut of a simplex of any
//                                         dimension and position
//   cutint/straightcutrule.cpp:503-556   LevelsetWrapper, update_initial_coefs
//   cutint/mlsetintegration.cpp:6-180    per element and domain tuple:
//                                         compatibility, condensing to the
//                                         cutting level sets, the parts
// The reference refines a list of simplices level set by level set (breadth
// first).  Here one thread walks the same refinement depth first with an
// explicit stack, children in order, which visits the final simplices in the
// same order (the final list is ordered by the child index at each level) with
// at most 2 M + 1 simplices held.  Every rule point is handed to a callback.
// Compiled with -fmad=false the operation order reproduces the CPU statement.
#pragma once
#include "xg_quadcut.cuh"

namespace xg {
namespace ml {

constexpr int kMaxLsets = 8;
constexpr int kMaxTuples = 256;

// the domain tuples of one integration domain (a union of tuples)
struct MlDesc {
  int M, ntup;
  int8_t dt[kMaxTuples * kMaxLsets];  // [ntup][M]: XG_NEG / XG_POS / XG_IF
};

struct Simp {
  qc::Pt p[4];
  int np, level;
};

// affine element map x = x_D + F xi (F(:,k) = x_k - x_D), inverse, determinant
struct AGeo {
  double x0[3], F[3][3], Finv[3][3], det;
};

template <int D>
XG_QHD void make_ageo(const double (*xv)[3], AGeo& g) {
  for (int i = 0; i < 3; i++) {
    g.x0[i] = i < D ? xv[D][i] : 0.0;
    for (int k = 0; k < 3; k++) g.F[i][k] = g.Finv[i][k] = 0.0;
  }
  for (int k = 0; k < D; k++)
    for (int i = 0; i < D; i++) g.F[i][k] = xv[k][i] - xv[D][i];
  if (D == 2) {
    const double a = g.F[0][0], b = g.F[0][1], c = g.F[1][0], d = g.F[1][1];
    g.det = a * d - b * c;
    const double id = 1.0 / g.det;
    g.Finv[0][0] = d * id;
    g.Finv[0][1] = -b * id;
    g.Finv[1][0] = -c * id;
    g.Finv[1][1] = a * id;
  } else {
    const double(*F)[3] = g.F;
    const double c00 = F[1][1] * F[2][2] - F[1][2] * F[2][1];
    const double c01 = F[1][2] * F[2][0] - F[1][0] * F[2][2];
    const double c02 = F[1][0] * F[2][1] - F[1][1] * F[2][0];
    g.det = F[0][0] * c00 + F[0][1] * c01 + F[0][2] * c02;
    const double id = 1.0 / g.det;
    g.Finv[0][0] = c00 * id;
    g.Finv[1][0] = c01 * id;
    g.Finv[2][0] = c02 * id;
    g.Finv[0][1] = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) * id;
    g.Finv[1][1] = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) * id;
    g.Finv[2][1] = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) * id;
    g.Finv[0][2] = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) * id;
    g.Finv[1][2] = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) * id;
    g.Finv[2][2] = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) * id;
  }
}

// LevelsetWrapper of a linear level set from its values at the reference
// vertices (1,0,0), (0,1,0), (0,0,1), (0,0,0)
template <int D>
XG_QHD qc::QL ql_simplex(const double* v) {
  qc::QL L;
  qc::ql_zero(L);
  L.c[0][0][0] = v[D];
  L.c[1][0][0] = v[0] - v[D];
  L.c[0][1][0] = v[1] - v[D];
  if (D == 3) L.c[0][0][1] = v[2] - v[D];
  return L;
}

XG_QHD void ql_normal(const qc::QL& L, double* n) {
  const double g[3] = {L.c[1][0][0], L.c[0][1][0], L.c[0][0][1]};
  const double nn = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
  for (int k = 0; k < 3; k++) n[k] = g[k] / nn;
}

// Decompose of simplex s (s.np points) by the values l and domain dt into at
// most 3 simplices.  Returns their number or -(xg error).
XG_QHD int split(const Simp& s, const double* l, int dt, Simp* out) {
  const int D = s.np - 1;
  if (qc::qcheck(l, s.np, 0.0) != XG_IF) return -XG_ERR_PLAIN_CUT;
  qc::Pt c[4];
  int nc = 0;
  if (s.np == 2) {
    c[nc++] = qc::qseg_point(s.p[0], s.p[1], l[0], l[1]);
  } else {
    for (int i = 0; i < s.np; i++)
      for (int j = i + 1; j < s.np; j++)
        if ((l[i] >= 0) != (l[j] >= 0)) {
          const double lij[2] = {l[i], l[j]};
          if (qc::qcheck(lij, 2, 0.0) != XG_IF) return -XG_ERR_PLAIN_CUT;
          c[nc++] = qc::qseg_point(s.p[i], s.p[j], l[i], l[j]);
        }
  }
  if (dt == XG_IF) {
    if (nc == D) {
      for (int i = 0; i < nc; i++) out[0].p[i] = c[i];
      out[0].np = nc;
      return 1;
    }
    if (nc == 4 && D == 3) {
      out[0].p[0] = c[0]; out[0].p[1] = c[1]; out[0].p[2] = c[3]; out[0].np = 3;
      out[1].p[0] = c[0]; out[1].p[1] = c[2]; out[1].p[2] = c[3]; out[1].np = 3;
      return 2;
    }
    return -XG_ERR_BAD_DECOMP;
  }
  int rel[4], nr = 0;
  for (int i = 0; i < s.np; i++)
    if (((dt == XG_POS) && (l[i] >= 0)) || ((dt == XG_NEG) && (l[i] < 0))) rel[nr++] = i;
  if (nr == 1) {
    for (int i = 0; i < nc; i++) out[0].p[i] = c[i];
    out[0].p[nc] = s.p[rel[0]];
    out[0].np = nc + 1;
    return 1;
  }
  if (nr == 2 && D == 2) {
    out[0].p[0] = s.p[rel[0]]; out[0].p[1] = s.p[rel[1]]; out[0].p[2] = c[1]; out[0].np = 3;
    out[1].p[0] = c[0]; out[1].p[1] = c[1]; out[1].p[2] = s.p[rel[0]]; out[1].np = 3;
    return 2;
  }
  if (nr == 2 && D == 3) {
    if (nc != 4) return -XG_ERR_BAD_DECOMP;
    out[0].p[0] = s.p[rel[1]]; out[0].p[1] = c[1]; out[0].p[2] = c[2]; out[0].p[3] = c[3];
    out[1].p[0] = s.p[rel[0]]; out[1].p[1] = s.p[rel[1]]; out[1].p[2] = c[1]; out[1].p[3] = c[2];
    out[2].p[0] = c[0]; out[2].p[1] = c[1]; out[2].p[2] = c[2]; out[2].p[3] = s.p[rel[0]];
    out[0].np = out[1].np = out[2].np = 4;
    return 3;
  }
  if (nr == 3 && D == 3) {
    if (nc != 3) return -XG_ERR_BAD_DECOMP;
    out[0].p[0] = c[0]; out[0].p[1] = c[1]; out[0].p[2] = c[2]; out[0].p[3] = s.p[rel[2]];
    out[1].p[0] = s.p[rel[0]]; out[1].p[1] = s.p[rel[1]]; out[1].p[2] = s.p[rel[2]]; out[1].p[3] = c[1];
    out[2].p[0] = c[0]; out[2].p[1] = c[1]; out[2].p[2] = s.p[rel[0]]; out[2].p[3] = s.p[rel[2]];
    out[0].np = out[1].np = out[2].np = 4;
    return 3;
  }
  return -XG_ERR_BAD_DECOMP;
}

// plain rule of a final simplex, weights through the codimension transform:
// mode 0: w; 1: w * fac; 2: w * fac / |det|; 3: w / |det|
template <class E>
XG_QNI void leaf_rule(const RuleTable* Rp, const Simp& s, int order, int mode, double fac, double adet, E& emit) {
  const RuleTable& R = *Rp;
  const double trafofac = qc::qsimplex_volume(s.p, s.np);
  const int d = s.np - 1, o = clamp_order(order);
  const int off = R.off[d][o], cnt = R.cnt[d][o];
  for (int q = 0; q < cnt; q++) {
    const double* ip = R.x[off + q];
    double originweight = 1.0;
    for (int m = 0; m < s.np - 1; ++m) originweight -= ip[m];
    double pt[3];
    for (int k = 0; k < 3; k++) pt[k] = originweight * s.p[0].x[k];
    for (int m = 0; m < s.np - 1; ++m)
      for (int k = 0; k < 3; k++) pt[k] += ip[m] * s.p[m + 1].x[k];
    double w = R.w[off + q] * trafofac;
    if (mode == 1) w = w * fac;
    else if (mode == 2) w = w * fac / adet;
    else if (mode == 3) w = w / adet;
    emit(pt, w);
  }
}

// StraightCutsIntegrationRule for an element cut by all Mc level sets lv[i]
// (values at the element vertices) with domains dts[i].  *npts += points
// emitted.  Returns 0 or an xg error.
template <int D, class E>
XG_QNI int straight_cuts(const RuleTable* Rp, const AGeo& g, int Mc, const double (*lv)[D + 1], const int* dts,
                         int order, E& emit, int* npts) {
  // codimension transform (constant on a simplex)
  // (more than 3 interface level sets, or 3 in 2D, are rejected after the
  // decomposition and only if the rule has points, as in the reference)
  int ifs[3], nif = 0;
  for (int i = 0; i < Mc; i++)
    if (dts[i] == XG_IF) {
      if (nif < 3) ifs[nif] = i;
      nif++;
    }
  const bool unsupported = nif > 3 || (nif == 3 && D != 3);
  int mode = 0;
  double fac = 1.0;
  const double adet = fabs(g.det);
  if (nif == 1) {
    double n[3];
    ql_normal(ql_simplex<D>(lv[ifs[0]]), n);
    double np[3] = {0, 0, 0};
    for (int k = 0; k < D; k++) {
      double s = 0;
      for (int j = 0; j < D; j++) s += g.Finv[j][k] * n[j];
      np[k] = s;
    }
    fac = qc::qnorm3(np[0], np[1], np[2]);
    mode = 1;
  } else if (nif == 2 && D == 2) {
    mode = 3;
  } else if (nif == 2) {
    double n0[3], n1[3];
    ql_normal(ql_simplex<D>(lv[ifs[0]]), n0);
    ql_normal(ql_simplex<D>(lv[ifs[1]]), n1);
    const double cr[3] = {n0[1] * n1[2] - n0[2] * n1[1], n0[2] * n1[0] - n0[0] * n1[2], n0[0] * n1[1] - n0[1] * n1[0]};
    const double cp_fac = 1. / qc::qnorm3(cr[0], cr[1], cr[2]);
    double nv[3];
    for (int i = 0; i < 3; i++) nv[i] = cp_fac * (g.F[i][0] * cr[0] + g.F[i][1] * cr[1] + g.F[i][2] * cr[2]);
    fac = qc::qnorm3(nv[0], nv[1], nv[2]);
    mode = 2;
  } else if (nif == 3) {
    mode = 3;
  }
  int produced = 0;
  // level 0: the reference simplex cut by the raw values of level set 0
  Simp root;
  for (int i = 0; i <= D; i++) {
    for (int k = 0; k < 3; k++) root.p[i].x[k] = (i < D && k == i) ? 1.0 : 0.0;
  }
  root.np = D + 1;
  root.level = 0;
  Simp stack[2 * kMaxLsets + 2];
  int top = 0;
  {
    Simp ch[3];
    const int n = split(root, lv[0], dts[0], ch);
    if (n < 0) return -n;
    for (int c = n - 1; c >= 0; c--) {
      ch[c].level = 1;
      stack[top++] = ch[c];
    }
  }
  while (top > 0) {
    const Simp s = stack[--top];
    if (s.level == Mc) {
      const int cnt = Rp->cnt[s.np - 1][clamp_order(order)];
      produced += cnt;
      if (!unsupported) {
        leaf_rule(Rp, s, order, mode, fac, adet, emit);
        *npts += cnt;
      }
      continue;
    }
    const qc::QL L = ql_simplex<D>(lv[s.level]);
    double l[4];
    for (int i = 0; i < s.np; i++) {
      const double d = qc::ql_val(L, s.p[i].x[0], s.p[i].x[1], s.p[i].x[2]);
      l[i] = fabs(d) > 1e-14 ? d : 1e-14;
    }
    const int dom = qc::qcheck(l, s.np, 0.0);
    if (dom == XG_IF) {
      Simp ch[3];
      const int n = split(s, l, dts[s.level], ch);
      if (n < 0) return -n;
      if (top + n > 2 * kMaxLsets + 2) return XG_ERR_CAPACITY;
      for (int c = n - 1; c >= 0; c--) {
        ch[c].level = s.level + 1;
        stack[top++] = ch[c];
      }
    } else if (dom == dts[s.level]) {
      Simp t = s;
      t.level = s.level + 1;
      stack[top++] = t;
    }
  }
  return (unsupported && produced > 0) ? XG_ERR_UNSUPPORTED : 0;
}

// CreateMultiLevelsetCutIntegrationRule for one element: for every domain
// tuple the standard rule (uncut, compatible), the rule of its one cutting
// level set, or StraightCutsIntegrationRule of its cutting level sets; parts
// in tuple order.  dts: ntup tuples of M entries; lv: the M level sets'
// values at the element vertices.
// *npts = points emitted (0: "no rule").  Returns 0 or an xg error.
template <int D, class E>
XG_QNI int element_rule(const RuleTable* Rp, const AGeo& g, int M, int ntup, const int8_t* dts,
                        const double (*lv)[D + 1], int order, E& emit, int* npts) {
  int ldt[kMaxLsets];
  for (int i = 0; i < M; i++) ldt[i] = qc::qcheck(lv[i], D + 1, 0.0);
  *npts = 0;
  for (int t = 0; t < ntup; t++) {
    const int8_t* dt = dts + t * M;
    bool compatible = true, cut = false;
    for (int i = 0; i < M; i++) {
      if (ldt[i] != XG_IF && ldt[i] != dt[i]) compatible = false;
      else if (ldt[i] == XG_IF) cut = true;
    }
    if (!compatible) continue;
    if (!cut) {
      const RuleTable& R = *Rp;
      const int o = clamp_order(order), off = R.off[D][o], cnt = R.cnt[D][o];
      for (int q = 0; q < cnt; q++) emit(R.x[off + q], R.w[off + q]);
      *npts += cnt;
      continue;
    }
    double cl[kMaxLsets][D + 1];
    int cdt[kMaxLsets], mc = 0;
    for (int i = 0; i < M; i++)
      if (ldt[i] == XG_IF || ldt[i] != dt[i]) {
        for (int v = 0; v <= D; v++) cl[mc][v] = lv[i][v];
        cdt[mc++] = dt[i];
      }
    const int e = straight_cuts<D>(Rp, g, mc, cl, cdt, order, emit, npts);
    if (e) return e;
  }
  return 0;
}

}  // namespace ml
}  // namespace xg

namespace xg {
namespace ml {

// StraightCutIntegrationRule on a boundary element (a (D-1)-simplex in D
// dimensions; cutint/straightcutrule.cpp:582-677, the point measure of
// :641-651 for IF on 2D boundary segments): emit(physical point, weight,
// measure) with weight * measure the point's share.  xv: the D vertices, l
// their level-set values.  Returns 0 or an xg error (IF on 3D boundary
// triangles is not supported).
template <int D, class E>
XG_QNI int bnd_rule(const RuleTable* Rp, const double (*xv)[3], const double* l, int dt, int order, E& emit) {
  const RuleTable& R = *Rp;
  constexpr int d = D - 1;
  double F[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  for (int k = 0; k < d; k++)
    for (int r = 0; r < 3; r++) F[r][k] = xv[k][r] - xv[d][r];
  double meas;
  if (d == 1) {
    meas = qc::qnorm3(F[0][0], F[1][0], F[2][0]);
  } else {
    meas = qc::qnorm3(F[1][0] * F[2][1] - F[2][0] * F[1][1], F[2][0] * F[0][1] - F[0][0] * F[2][1],
                      F[0][0] * F[1][1] - F[1][0] * F[0][1]);
  }
  auto to_phys = [&](const double* xi, double w) {
    double x[3];
    for (int r = 0; r < 3; r++) {
      double s = xv[d][r];
      for (int k = 0; k < d; k++) s += F[r][k] * xi[k];
      x[r] = s;
    }
    emit(x, w, meas);
  };
  const int dom = qc::qcheck(l, d + 1, 0.0);
  if (dom != XG_IF) {
    if (dom != dt) return 0;
    const int o = clamp_order(order), off = R.off[d][o], cnt = R.cnt[d][o];
    for (int q = 0; q < cnt; q++) to_phys(R.x[off + q], R.w[off + q]);
    return 0;
  }
  if (dt == XG_IF && d != 1) return XG_ERR_UNSUPPORTED;
  Simp root;
  for (int i = 0; i <= d; i++)
    for (int k = 0; k < 3; k++) root.p[i].x[k] = (i < d && k == i) ? 1.0 : 0.0;
  root.np = d + 1;
  Simp ch[3];
  const int n = split(root, l, dt, ch);
  if (n < 0) return -n;
  auto on_point = [&](const double* xi, double w) { to_phys(xi, dt == XG_IF ? w / meas : w); };
  for (int c = 0; c < n; c++) qc::qsimplex_plain(Rp, ch[c].p, ch[c].np, order, on_point);
  return 0;
}

}  // namespace ml
}  // namespace xg

// Mesh-level isoparametric integration for P2 level sets, host and device
// (ngsxfem's LevelSetMeshAdaptation workflow: python/lsetcurv.py:281-356).
//
// Per element (ShiftIntegrator::CalcElementVector,
// lsetcurving/shiftintegrators.cpp:38-122; SearchCorrespondingPoint,
// lsetcurving/calcpointshift.cpp:143-201; ProjectShift,
// lsetcurving/projshift.cpp:58-135): elements whose P1 values (InterpolateToP1
// perturbation) have both signs or a zero get a P2 deformation: at every point
// of the order-4 rule a Newton search (at most 20 steps, tolerance 1e-14)
// along J^-1 J^-T grad(phi_ho) for the point where phi_ho equals phi_p1, the
// shift (clipped at `threshold` if >= 0) projected in L2 onto the hierarchical
// P2 functions, vertex coefficients dropped.  The edge coefficients J theta
// are then averaged over the band elements sharing each edge
// (projshift.cpp:140-197), and every element is integrated with the straight
// cut rule of phi_p1 mapped by xhat -> xhat + Theta(xhat): weights times
// |det(J A)|, A = I + grad Theta, on the interface times |(J A)^-T n_ref|.
// The arithmetic follows the CPU statement (oracle/xg_oracle_iso.cpp); the
// cut rule itself is the single-level-set case of xg_mlset.cuh.
#pragma once
#include "xg_mlset.cuh"

namespace xg {
namespace iso {

template <int D>
XG_QHD int nedge() {
  return D == 2 ? 3 : 6;
}
template <int D>
XG_QHD void edge_ends(int e, int& a, int& b) {
  const int tri[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  const int tet[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  a = D == 2 ? tri[e][0] : tet[e][0];
  b = D == 2 ? tri[e][1] : tet[e][1];
}

template <int D>
XG_QHD void lambdas(const double* x, double* l) {
  double s = 0.0;
  for (int i = 0; i < D; i++) {
    l[i] = x[i];
    s += x[i];
  }
  l[D] = 1.0 - s;
}

template <int D>
XG_QHD double dlam(int i, int j) {
  return i < D ? (i == j ? 1.0 : 0.0) : -1.0;
}

// P2 nodal interpolant (vertices, then edge midpoints): value, reference gradient
template <int D>
XG_QHD double p2_value(const double* v, const double* x, double* grad) {
  double l[4];
  lambdas<D>(x, l);
  double val = 0.0;
  for (int j = 0; j < D; j++) grad[j] = 0.0;
  for (int i = 0; i <= D; i++) {
    val += v[i] * l[i] * (2.0 * l[i] - 1.0);
    const double dn = 4.0 * l[i] - 1.0;
    for (int j = 0; j < D; j++) grad[j] += v[i] * dn * dlam<D>(i, j);
  }
  for (int e = 0; e < nedge<D>(); e++) {
    int a, b;
    edge_ends<D>(e, a, b);
    const double c = v[D + 1 + e];
    val += c * 4.0 * l[a] * l[b];
    for (int j = 0; j < D; j++) grad[j] += c * 4.0 * (dlam<D>(a, j) * l[b] + l[a] * dlam<D>(b, j));
  }
  return val;
}

// hierarchical P2 functions: lambda_i, then lambda_a lambda_b per edge
template <int D>
XG_QHD void p2h_shape(const double* x, double* phi, double (*dphi)[3]) {
  double l[4];
  lambdas<D>(x, l);
  for (int i = 0; i <= D; i++) {
    phi[i] = l[i];
    for (int j = 0; j < D; j++) dphi[i][j] = dlam<D>(i, j);
  }
  for (int e = 0; e < nedge<D>(); e++) {
    int a, b;
    edge_ends<D>(e, a, b);
    phi[D + 1 + e] = l[a] * l[b];
    for (int j = 0; j < D; j++) dphi[D + 1 + e][j] = dlam<D>(a, j) * l[b] + l[a] * dlam<D>(b, j);
  }
}

template <int D>
XG_QHD bool invert(const double (*A)[3], double (*Ai)[3], double* det) {
  if (D == 2) {
    const double d = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    if (d == 0.0) return false;
    Ai[0][0] = A[1][1] / d;
    Ai[0][1] = -A[0][1] / d;
    Ai[1][0] = -A[1][0] / d;
    Ai[1][1] = A[0][0] / d;
    *det = d;
    return true;
  }
  const double d = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
                   A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                   A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
  if (d == 0.0) return false;
  Ai[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / d;
  Ai[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / d;
  Ai[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / d;
  Ai[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / d;
  Ai[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / d;
  Ai[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / d;
  Ai[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / d;
  Ai[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / d;
  Ai[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / d;
  *det = d;
  return true;
}

// Gaussian elimination with partial pivoting, n <= 10 unknowns, D right-hand sides
template <int D>
XG_QHD void solve(int n, double (*M)[10], double (*rhs)[3]) {
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++)
      if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
    if (p != c) {
      for (int k = 0; k < n; k++) {
        const double t = M[c][k];
        M[c][k] = M[p][k];
        M[p][k] = t;
      }
      for (int k = 0; k < D; k++) {
        const double t = rhs[c][k];
        rhs[c][k] = rhs[p][k];
        rhs[p][k] = t;
      }
    }
    for (int r = c + 1; r < n; r++) {
      const double f = M[r][c] / M[c][c];
      for (int k = c; k < n; k++) M[r][k] -= f * M[c][k];
      for (int k = 0; k < D; k++) rhs[r][k] -= f * rhs[c][k];
    }
  }
  for (int c = n - 1; c >= 0; c--)
    for (int k = 0; k < D; k++) {
      double s = rhs[c][k];
      for (int j = c + 1; j < n; j++) s -= M[c][j] * rhs[j][k];
      rhs[c][k] = s / M[c][c];
    }
}

// the element map x = x_D + J xhat: J, J^-1, det (J(2,2) = 1 in 2D)
struct Aff {
  double J[3][3], Ji[3][3], det;
};

template <int D>
XG_QHD bool make_aff(const double (*xv)[3], Aff& a) {
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) a.J[r][c] = (r == c && r >= D) ? 1.0 : 0.0;
  for (int j = 0; j < D; j++)
    for (int r = 0; r < D; r++) a.J[r][j] = xv[j][r] - xv[D][r];
  return invert<D>(a.J, a.Ji, &a.det);
}

template <int D>
XG_QHD void perturbed_p1(const double* p2, double* p1) {
  for (int i = 0; i <= D; i++) {
    p1[i] = p2[i];
    if (fabs(p1[i]) < 1e-14) p1[i] = 1e-14;
  }
}

// per-element deformation: edge coefficients theta[e][d] (reference frame);
// false outside the relevant band.  *nonconv counts searches that did not
// converge (their shift is zero).
template <int D>
XG_QNI bool deformation(const RuleTable* Rp, const Aff& A, const double* p2, const double* p1, double threshold,
                        double (*theta)[3], int* nonconv) {
  const RuleTable& R = *Rp;
  constexpr int NE = D == 2 ? 3 : 6, ND = D + 1 + NE;
  for (int e = 0; e < NE; e++)
    for (int d = 0; d < 3; d++) theta[e][d] = 0.0;
  bool has_neg = false, has_pos = false;
  for (int i = 0; i <= D; i++) {
    if (p1[i] == 0.0) has_neg = has_pos = true;
    if (p1[i] > 0.0) has_pos = true;
    if (p1[i] < 0.0) has_neg = true;
  }
  if (!(has_neg && has_pos)) return false;
  const int o = clamp_order(4), off = R.off[D][o], nq = R.cnt[D][o];
  double M[10][10], rhs[10][3];
  for (int i = 0; i < ND; i++) {
    for (int j = 0; j < ND; j++) M[i][j] = 0.0;
    for (int r = 0; r < 3; r++) rhs[i][r] = 0.0;
  }
  double G[3][3];
  for (int r = 0; r < D; r++)
    for (int c = 0; c < D; c++) {
      double s = 0.0;
      for (int k = 0; k < D; k++) s += A.Ji[r][k] * A.Ji[c][k];
      G[r][c] = s;
    }
  for (int q = 0; q < nq; q++) {
    const double* x0 = R.x[off + q];
    const double wq = R.w[off + q];
    double phi[10], dphi[10][3];
    p2h_shape<D>(x0, phi, dphi);
    for (int i = 0; i < ND; i++)
      for (int j = 0; j < ND; j++) M[i][j] += wq * phi[i] * phi[j];
    double l[4];
    lambdas<D>(x0, l);
    double goal = 0.0;
    for (int i = 0; i <= D; i++) goal += p1[i] * l[i];
    double g0[3];
    p2_value<D>(p2, x0, g0);
    double s[3];
    for (int r = 0; r < D; r++) {
      s[r] = 0.0;
      for (int c = 0; c < D; c++) s[r] += G[r][c] * g0[c];
    }
    double cur[3] = {x0[0], x0[1], D == 3 ? x0[2] : 0.0};
    int it = 0;
    for (it = 0; it < 20; ++it) {
      double g[3];
      const double val = p2_value<D>(p2, cur, g);
      const double defect = goal - val;
      if (fabs(defect) < 1e-14) break;
      double dn = 0.0;
      for (int r = 0; r < D; r++) dn += g[r] * s[r];
      for (int r = 0; r < D; r++) cur[r] += defect / dn * s[r];
    }
    double dist[3] = {0.0, 0.0, 0.0};
    if (it == 20) {
      (*nonconv)++;
    } else {
      for (int r = 0; r < D; r++) dist[r] = cur[r] - x0[r];
    }
    if (threshold >= 0.0) {
      double n2 = 0.0;
      for (int r = 0; r < D; r++) n2 += dist[r] * dist[r];
      const double n = sqrt(n2);
      if (n > threshold)
        for (int r = 0; r < D; r++) dist[r] *= threshold / n;
    }
    for (int i = 0; i < ND; i++)
      for (int r = 0; r < D; r++) rhs[i][r] += wq * phi[i] * dist[r];
  }
  solve<D>(ND, M, rhs);
  for (int e = 0; e < NE; e++)
    for (int r = 0; r < D; r++) theta[e][r] = rhs[D + 1 + e][r];
  return true;
}

// deformed point y = x + Theta(x) and A = I + grad Theta (reference frame)
template <int D>
XG_QHD void deform_at(const double (*theta)[3], const double* x, double* y, double (*Am)[3]) {
  constexpr int NE = D == 2 ? 3 : 6;
  double phi[10], dphi[10][3];
  p2h_shape<D>(x, phi, dphi);
  for (int r = 0; r < 3; r++) {
    y[r] = r < D ? x[r] : 0.0;
    for (int c = 0; c < 3; c++) Am[r][c] = r == c ? 1.0 : 0.0;
  }
  for (int e = 0; e < NE; e++) {
    const int k = D + 1 + e;
    for (int r = 0; r < D; r++) {
      y[r] += theta[e][r] * phi[k];
      for (int c = 0; c < D; c++) Am[r][c] += theta[e][r] * dphi[k][c];
    }
  }
}

// the straight cut rule of p1 on the reference element mapped by the
// deformation: emit(physical point, weight).  Returns 0 or an xg error.
template <int D, class E>
XG_QNI int mapped_rule(const RuleTable* Rp, const Aff& A, const double* x0, const double* p1,
                       const double (*theta)[3], int dt, int order, E& emit) {
  // the reference element as an element (identity map)
  double rv[D + 1][3];
  for (int i = 0; i <= D; i++)
    for (int k = 0; k < 3; k++) rv[i][k] = (i < D && k == i) ? 1.0 : 0.0;
  ml::AGeo g;
  ml::make_ageo<D>(rv, g);
  double nref[3] = {0, 0, 0};
  for (int j = 0; j < D; j++) nref[j] = p1[j] - p1[D];
  double nn = 0.0;
  for (int j = 0; j < D; j++) nn += nref[j] * nref[j];
  nn = sqrt(nn);
  for (int j = 0; j < D; j++) nref[j] /= nn;
  int st = 0;
  auto on_point = [&](const double* xr, double wr) {
    if (st) return;
    double y[3], Am[3][3];
    deform_at<D>(theta, xr, y, Am);
    double F[3][3], Fi[3][3], detF;
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) {
        double s = 0.0;
        for (int k = 0; k < 3; k++) s += A.J[r][k] * Am[k][c];
        F[r][c] = s;
      }
    if (!invert<D>(F, Fi, &detF)) {
      st = XG_ERR_NONFINITE;
      return;
    }
    double w = wr * fabs(detF);
    if (dt == XG_IF) {
      double t2 = 0.0;
      for (int r = 0; r < D; r++) {
        double s = 0.0;
        for (int k = 0; k < D; k++) s += Fi[k][r] * nref[k];
        t2 += s * s;
      }
      w *= sqrt(t2);
    }
    double xp[3] = {0, 0, 0};
    for (int r = 0; r < D; r++) {
      double s = x0[r];
      for (int k = 0; k < D; k++) s += A.J[r][k] * y[k];
      xp[r] = s;
    }
    emit(xp, w);
  };
  const int dom = qc::qcheck(p1, D + 1, 0.0);
  if (dom != XG_IF) {
    if (dom != dt) return 0;
    const RuleTable& R = *Rp;
    const int o = clamp_order(order), off = R.off[D][o], cnt = R.cnt[D][o];
    for (int q = 0; q < cnt; q++) on_point(R.x[off + q], R.w[off + q]);
    return st;
  }
  double l1[1][D + 1];
  for (int i = 0; i <= D; i++) l1[0][i] = p1[i];
  const int dts[1] = {dt};
  int npts = 0;
  const int e = ml::straight_cuts<D>(Rp, g, 1, l1, dts, order, on_point, &npts);
  return e ? e : st;
}

// step 1 of the mesh-level mapping for one element (vertex coordinates xv,
// P2 nodal values p2): the physical edge contributions J theta and whether
// the element is in the band.  Returns false if the element map is singular.
template <int D>
XG_QHD bool element_contrib(const RuleTable* Rp, const double (*xv)[3], const double* p2, double threshold,
                            double (*contrib)[3], bool* band, int* nonconv) {
  constexpr int NE = D == 2 ? 3 : 6;
  Aff A;
  if (!make_aff<D>(xv, A)) return false;
  double p1[4];
  perturbed_p1<D>(p2, p1);
  double theta[6][3];
  *band = deformation<D>(Rp, A, p2, p1, threshold, theta, nonconv);
  for (int j = 0; j < NE; j++)
    for (int r = 0; r < 3; r++) {
      double s = 0.0;
      if (r < D)
        for (int c = 0; c < D; c++) s += A.J[r][c] * theta[j][c];
      contrib[j][r] = s;
    }
  return true;
}

// step 3: the element's mapped rule with the averaged physical edge
// deformations gdef[local edge][3]; emit(physical point, weight).
template <int D, class E>
XG_QHD int element_rule(const RuleTable* Rp, const double (*xv)[3], const double* p2, const double (*gdef)[3],
                        int dt, int order, E& emit) {
  constexpr int NE = D == 2 ? 3 : 6;
  Aff A;
  if (!make_aff<D>(xv, A)) return XG_ERR_NONFINITE;
  double theta[6][3];
  for (int j = 0; j < NE; j++)
    for (int r = 0; r < 3; r++) {
      double s = 0.0;
      if (r < D)
        for (int c = 0; c < D; c++) s += A.Ji[r][c] * gdef[j][c];
      theta[j][r] = s;
    }
  double p1[4];
  perturbed_p1<D>(p2, p1);
  return mapped_rule<D>(Rp, A, xv[D], p1, theta, dt, order, emit);
}

}  // namespace iso
}  // namespace xg

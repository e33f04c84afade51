// Oracle: CPU restatement of ngsxfem's straight-cut assembly path.
// TEST INFRASTRUCTURE ONLY (see xg_oracle.h).  Built with -ffp-contract=off so
// that x86 and Arm hosts produce identical bits.
//
// Reference files restated here (paths inside the ngsxfem project):
//   cutint/straightcutrule.cpp:11-24   CheckIfStraightCut
//   cutint/straightcutrule.cpp:41-64   SimpleX::CalcIFPolytopEUsingLset
//   cutint/straightcutrule.cpp:66-72   SimpleX::GetVolume
//   cutint/straightcutrule.cpp:80-100  SimpleX::GetPlainIntegrationRule
//   cutint/straightcutrule.cpp:131-196 LevelsetCutSimplex::Decompose
//   cutint/straightcutrule.cpp:503-538 LevelsetWrapper (coefficients, gradient, normal)
//   cutint/straightcutrule.cpp:558-578 TransformQuadUntrafoToIRInterface
//   cutint/straightcutrule.cpp:582-677 StraightCutIntegrationRule
//   xfem/cutinfo.cpp:61-132            CutInformation::Update (element part)
//   xfem/cutinfo.cpp:476-538           GetFacetsWithNeighborTypes
//   xfem/symboliccutbfi.cpp:76-313     SymbolicCutBilinearFormIntegrator::T_CalcElementMatrixAdd
//   xfem/symboliccutbfi.cpp:1747-1846  MapPatchIntegrationPoint
//   xfem/symboliccutbfi.cpp:1982-2377  SymbolicFacetPatchBilinearFormIntegrator::T_CalcFacetMatrix
//   utils/p1interpol.cpp:104-107       vertex perturbation of InterpolateToP1
//   cutint/cutintegral.cpp:126-212     CutIntegral::T_CutIntegrate (Integrate)
// NGSolve pieces the reference calls but which are not in the reference tree
// (quadrature tables, H1 shape functions, the sparse scatter) are replaced by
// this project's own definitions, stated next to the code below.
#include "xg_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Quadrature: Golub-Welsch for Gauss-Jacobi nodes (weight (1-x)^a on [-1,1]),
// eigenvalues by the cyclic Jacobi rotation method.
// Rule family (shared definition with the product):
//   segment order p : Gauss-Legendre, n = p/2+1 points on [0,1]
//   trig   order p : p<=1 centroid; p==2 3-point (1/6,1/6,2/3); p==4 6-point and
//                    p==5 7-point fully symmetric rules; otherwise collapsed
//                    Gauss-Jacobi conical product, n = p/2+1 per direction
//   tet    order p : p<=1 centroid; p==2 4-point (a,b,b,b), a=(5+3sqrt5)/20;
//                    p==4,5 14-point fully symmetric rule; otherwise conical
//                    product n = p/2+1 per direction
// The symmetric rules' parameters come from oracle/derive_symmetric_rules.py.
// ---------------------------------------------------------------------------
void sym_eig(int n, std::vector<double>& A, std::vector<double>& V) {
  V.assign(n * n, 0.0);
  for (int i = 0; i < n; i++) V[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) off += A[p * n + q] * A[p * n + q];
    if (off < 1e-34) break;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        double apq = A[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        double app = A[p * n + p], aqq = A[q * n + q];
        double theta = (aqq - app) / (2 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; k++) {
          double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {
          double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
}

// nodes/weights on [0,1] for weight (1-u)^alpha
void gauss_jacobi01(int n, int alpha, std::vector<double>& x, std::vector<double>& w) {
  const double a = alpha, b = 0.0;
  std::vector<double> J(n * n, 0.0), V;
  for (int k = 0; k < n; k++) {
    double diag;
    if (k == 0) diag = (b - a) / (a + b + 2);
    else diag = (b * b - a * a) / ((2 * k + a + b) * (2 * k + a + b + 2));
    J[k * n + k] = diag;
    if (k >= 1) {
      double kk = k;
      double num = 4 * kk * (kk + a) * (kk + b) * (kk + a + b);
      double s = 2 * kk + a + b;
      double den = s * s * (s + 1) * (s - 1);
      double off = std::sqrt(num / den);
      J[(k - 1) * n + k] = off;
      J[k * n + (k - 1)] = off;
    }
  }
  sym_eig(n, J, V);
  double mu0 = (alpha == 0) ? 2.0 : (alpha == 1 ? 2.0 : 8.0 / 3.0);
  std::vector<std::pair<double, double>> nw(n);
  for (int i = 0; i < n; i++) nw[i] = {J[i * n + i], mu0 * V[0 * n + i] * V[0 * n + i]};
  std::sort(nw.begin(), nw.end());
  // Newton polish of the eigenvalues on P_n^{(a,0)} (values and derivatives by
  // the recurrences of P_n and of P'_n), weights from the Christoffel formula
  // 2^{a+1} / ((1 - x^2) P_n'(x)^2)
  auto jac = [&](double xx, double& pv, double& dv) {
    double p0 = 1.0, p1 = 0.5 * (a - b) + 0.5 * (a + b + 2.0) * xx;
    double d0 = 0.0, d1 = 0.5 * (a + b + 2.0);
    if (n == 0) { pv = 1.0; dv = 0.0; return; }
    for (int k = 2; k <= n; k++) {
      double c = 2.0 * k + a + b;
      double A1 = 2.0 * k * (k + a + b) * (c - 2.0);
      double A2 = (c - 1.0) * (a * a - b * b);
      double A3 = (c - 2.0) * (c - 1.0) * c;
      double A4 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * c;
      double p2 = ((A2 + A3 * xx) * p1 - A4 * p0) / A1;
      double d2 = ((A2 + A3 * xx) * d1 + A3 * p1 - A4 * d0) / A1;
      p0 = p1; p1 = p2; d0 = d1; d1 = d2;
    }
    pv = p1; dv = d1;
  };
  for (int i = 0; i < n; i++) {
    double xx = nw[i].first;
    if (alpha == 0 && (n % 2) == 1 && i == n / 2) xx = 0.0;
    for (int it = 0; it < 3; it++) {
      double pv, dv;
      jac(xx, pv, dv);
      xx -= pv / dv;
    }
    double pv, dv;
    jac(xx, pv, dv);
    nw[i] = {xx, std::ldexp(1.0, alpha + 1) / ((1.0 - xx * xx) * dv * dv)};
  }
  x.resize(n);
  w.resize(n);
  double scale = std::ldexp(1.0, -alpha - 1);
  for (int i = 0; i < n; i++) {
    x[i] = (1.0 + nw[i].first) * 0.5;
    w[i] = nw[i].second * scale;
  }
}

struct Rule {
  std::vector<double> p;  // 3 per point
  std::vector<double> w;
  int size() const { return (int)w.size(); }
};

Rule make_rule(int d, int p) {
  Rule r;
  if (p < 0) p = 0;
  auto add = [&](double a, double b, double c, double w) {
    r.p.push_back(a); r.p.push_back(b); r.p.push_back(c); r.w.push_back(w);
  };
  int n = p / 2 + 1;
  if (d == 0) { add(0, 0, 0, 1.0); return r; }
  if (d == 1) {
    std::vector<double> x, w;
    gauss_jacobi01(n, 0, x, w);
    for (int i = 0; i < n; i++) add(x[i], 0, 0, w[i]);
    return r;
  }
  // orbits in barycentric coordinates (lambda_0, lambda_1, lambda_2[, lambda_3]); point = (lambda_0, lambda_1[, lambda_2])
  auto s21 = [&](double a, double w) {
    double b = 1.0 - 2.0 * a;
    add(a, a, 0, w); add(a, b, 0, w); add(b, a, 0, w);
  };
  auto s31 = [&](double a, double w) {
    double b = 1.0 - 3.0 * a;
    add(a, a, a, w); add(a, a, b, w); add(a, b, a, w); add(b, a, a, w);
  };
  auto s22 = [&](double c, double w) {
    double dd = 0.5 - c;
    add(c, c, dd, w); add(c, dd, c, w); add(c, dd, dd, w); add(dd, c, c, w); add(dd, c, dd, w); add(dd, dd, c, w);
  };
  if (d == 2) {
    if (p <= 1) { add(1.0 / 3, 1.0 / 3, 0, 0.5); return r; }
    if (p == 2) {
      add(1.0 / 6, 1.0 / 6, 0, 1.0 / 6);
      add(2.0 / 3, 1.0 / 6, 0, 1.0 / 6);
      add(1.0 / 6, 2.0 / 3, 0, 1.0 / 6);
      return r;
    }
    if (p == 4) {
      s21(0.4459484909159648863183293, 0.1116907948390057328475035);
      s21(0.09157621350977074345957146, 0.05497587182766093381916316);
      return r;
    }
    if (p == 5) {
      add(1.0 / 3, 1.0 / 3, 0, 0.1125);
      s21(0.4701420641051150897704412, 0.06619707639425309036882469);
      s21(0.1012865073234563388009874, 0.06296959027241357629784197);
      return r;
    }
    std::vector<double> xu, wu, xv, wv;
    gauss_jacobi01(n, 1, xu, wu);
    gauss_jacobi01(n, 0, xv, wv);
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) add(xu[i], xv[j] * (1 - xu[i]), 0, wu[i] * wv[j]);
    return r;
  }
  // d == 3
  if (p <= 1) { add(0.25, 0.25, 0.25, 1.0 / 6); return r; }
  if (p == 2) {
    double a = (5.0 + 3.0 * std::sqrt(5.0)) / 20.0, b = (5.0 - std::sqrt(5.0)) / 20.0;
    add(a, b, b, 1.0 / 24);
    add(b, a, b, 1.0 / 24);
    add(b, b, a, 1.0 / 24);
    add(b, b, b, 1.0 / 24);
    return r;
  }
  if (p == 4 || p == 5) {
    s31(0.09273525031089122640232391, 0.01224884051939365825728503);
    s31(0.3108859192633006097973457, 0.01878132095300264179986428);
    s22(0.4544962958743503505081195, 0.007091003462846911073011571);
    return r;
  }
  std::vector<double> xu, wu, xv, wv, xw, ww;
  gauss_jacobi01(n, 2, xu, wu);
  gauss_jacobi01(n, 1, xv, wv);
  gauss_jacobi01(n, 0, xw, ww);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) {
        double u = xu[i], v = xv[j], t = xw[k];
        add(u, (1 - u) * v, (1 - u) * (1 - v) * t, wu[i] * wv[j] * ww[k]);
      }
  return r;
}

const Rule& get_rule(int d, int p) {
  static std::vector<Rule> cache[4];
  static bool init = false;
  if (!init) {
    for (int dd = 0; dd < 4; dd++)
      for (int pp = 0; pp <= 16; pp++) cache[dd].push_back(make_rule(dd, pp));
    init = true;
  }
  if (p < 0) p = 0;
  if (p > 16) p = 16;
  return cache[d][p];
}
struct RuleInit { RuleInit() { get_rule(0, 0); } } rule_init_instance;

// ---------------------------------------------------------------------------
// Straight-cut geometry (restatement of cutint/straightcutrule.cpp).
// ---------------------------------------------------------------------------
struct P3 { double c[3]; };
enum { NEG = 0, POS = 1, IF = 2 };
enum { ERR_PLAIN_CUT = -2, ERR_BAD_DECOMP = -3, ERR_CAPACITY = -4 };

// straightcutrule.cpp:11-24
int check_if_straight_cut(const double* v, int n, double eps = 0.0) {
  bool haspos = false, hasneg = false;
  for (int i = 0; i < n; i++) {
    if (!haspos && (v[i] > eps)) haspos = true;
    if (!hasneg && (v[i] < -eps)) hasneg = true;
    if (haspos && hasneg) break;
  }
  if ((hasneg && haspos) || (!hasneg && !haspos)) return IF;
  return hasneg ? NEG : POS;
}

P3 seg_point(const P3& a, const P3& b, double la, double lb) {
  // straightcutrule.cpp:50  p0 + (l0/(l0-l1))*(p1-p0)
  double t = la / (la - lb);
  P3 r;
  for (int k = 0; k < 3; k++) r.c[k] = a.c[k] + t * (b.c[k] - a.c[k]);
  return r;
}

// straightcutrule.cpp:41-64; returns #points or error
int calc_if_points(const P3* pts, int np, const double* l, P3* out) {
  if (check_if_straight_cut(l, np) != IF) return ERR_PLAIN_CUT;
  if (np == 2) { out[0] = seg_point(pts[0], pts[1], l[0], l[1]); return 1; }
  int n = 0;
  for (int i = 0; i < np; i++)
    for (int j = i + 1; j < np; j++)
      if ((l[i] >= 0) != (l[j] >= 0)) {
        double lij[2] = {l[i], l[j]};
        if (check_if_straight_cut(lij, 2) != IF) return ERR_PLAIN_CUT;
        out[n++] = seg_point(pts[i], pts[j], l[i], l[j]);
      }
  return n;
}

double l2norm3(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

// straightcutrule.cpp:66-72
double simplex_volume(const P3* p, int np) {
  int D = np - 1;
  if (D == 0) return 1;
  if (D == 1) {
    double d[3] = {p[1].c[0] - p[0].c[0], p[1].c[1] - p[0].c[1], p[1].c[2] - p[0].c[2]};
    return l2norm3(d);
  }
  if (D == 2) {
    double a[3], b[3], c[3];
    for (int k = 0; k < 3; k++) { a[k] = p[2].c[k] - p[0].c[k]; b[k] = p[1].c[k] - p[0].c[k]; }
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
    return l2norm3(c);
  }
  double a[3], b[3], c[3];
  for (int k = 0; k < 3; k++) {
    a[k] = p[3].c[k] - p[0].c[k]; b[k] = p[2].c[k] - p[0].c[k]; c[k] = p[1].c[k] - p[0].c[k];
  }
  double det = a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) +
               a[2] * (b[0] * c[1] - b[1] * c[0]);
  return std::fabs(det);
}

struct Sub { int np; P3 p[4]; };

// straightcutrule.cpp:80-100
void plain_rule(const Sub& s, int order, std::vector<double>& pts, std::vector<double>& wts) {
  double trafofac = simplex_volume(s.p, s.np);
  const Rule& r = get_rule(s.np - 1, order);
  for (int q = 0; q < r.size(); q++) {
    const double* ip = &r.p[3 * q];
    double originweight = 1.0;
    for (int m = 0; m < s.np - 1; ++m) originweight -= ip[m];
    double pt[3];
    for (int k = 0; k < 3; k++) pt[k] = originweight * s.p[0].c[k];
    for (int m = 0; m < s.np - 1; ++m)
      for (int k = 0; k < 3; k++) pt[k] += ip[m] * s.p[m + 1].c[k];
    pts.push_back(pt[0]); pts.push_back(pt[1]); pts.push_back(pt[2]);
    wts.push_back(r.w[q] * trafofac);
  }
}

void ref_simplex(int D, P3* p) {
  // straightcutrule.hpp:55-60 reference vertices
  for (int i = 0; i <= D; i++)
    for (int k = 0; k < 3; k++) p[i].c[k] = 0.0;
  for (int i = 0; i < D; i++) p[i].c[i] = 1.0;
}

// straightcutrule.cpp:131-196
int decompose(int D, const double* lset, int dt, Sub* subs) {
  P3 s[4];
  ref_simplex(D, s);
  P3 cut[4];
  int nc = calc_if_points(s, D + 1, lset, cut);
  if (nc < 0) return nc;
  int ns = 0;
  if (dt == IF) {
    if (nc == D) {
      subs[0].np = nc;
      for (int i = 0; i < nc; i++) subs[0].p[i] = cut[i];
      return 1;
    } else if (nc == 4 && D == 3) {
      subs[0].np = 3; subs[0].p[0] = cut[0]; subs[0].p[1] = cut[1]; subs[0].p[2] = cut[3];
      subs[1].np = 3; subs[1].p[0] = cut[0]; subs[1].p[1] = cut[2]; subs[1].p[2] = cut[3];
      return 2;
    }
    return ERR_BAD_DECOMP;
  }
  int rel[4], nr = 0;
  for (int i = 0; i < D + 1; i++)
    if (((dt == POS) && (lset[i] >= 0)) || ((dt == NEG) && (lset[i] < 0))) rel[nr++] = i;
  if (nr == 1) {
    Sub& a = subs[ns++];
    a.np = nc + 1;
    for (int i = 0; i < nc; i++) a.p[i] = cut[i];
    a.p[nc] = s[rel[0]];
    if (a.np != D + 1) return ERR_BAD_DECOMP;
  } else if (nr == 2 && D == 2) {
    Sub& a = subs[ns++];
    a.np = 3; a.p[0] = s[rel[0]]; a.p[1] = s[rel[1]]; a.p[2] = cut[1];
    Sub& b = subs[ns++];
    b.np = 3; b.p[0] = cut[0]; b.p[1] = cut[1]; b.p[2] = s[rel[0]];
  } else if (nr == 2 && D == 3) {
    if (nc != 4) return ERR_BAD_DECOMP;
    Sub& a = subs[ns++];
    a.np = 4; a.p[0] = s[rel[1]]; a.p[1] = cut[1]; a.p[2] = cut[2]; a.p[3] = cut[3];
    Sub& b = subs[ns++];
    b.np = 4; b.p[0] = s[rel[0]]; b.p[1] = s[rel[1]]; b.p[2] = cut[1]; b.p[3] = cut[2];
    Sub& c = subs[ns++];
    c.np = 4; c.p[0] = cut[0]; c.p[1] = cut[1]; c.p[2] = cut[2]; c.p[3] = s[rel[0]];
  } else if (nr == 3 && D == 3) {
    if (nc != 3) return ERR_BAD_DECOMP;
    Sub& a = subs[ns++];
    a.np = 4; a.p[0] = cut[0]; a.p[1] = cut[1]; a.p[2] = cut[2]; a.p[3] = s[rel[2]];
    Sub& b = subs[ns++];
    b.np = 4; b.p[0] = s[rel[0]]; b.p[1] = s[rel[1]]; b.p[2] = s[rel[2]]; b.p[3] = cut[1];
    Sub& c = subs[ns++];
    c.np = 4; c.p[0] = cut[0]; c.p[1] = cut[1]; c.p[2] = s[rel[0]]; c.p[3] = s[rel[2]];
  } else {
    return ERR_BAD_DECOMP;
  }
  return ns;
}

// Element geometry: x(xi) = x_D + F xi, F(:,k) = x_k - x_D (reference vertices
// (1,0,0),(0,1,0),(0,0,1),(0,0,0) as in straightcutrule.hpp:55-60).
struct Geo {
  int D;
  double x0[3];      // x_D
  double F[3][3];    // F[i][k] = d x_i / d xi_k
  double Finv[3][3];
  double det;
};

void make_geo(int D, const double* elc, Geo& g) {
  g.D = D;
  for (int i = 0; i < 3; i++) {
    g.x0[i] = 0;
    for (int k = 0; k < 3; k++) { g.F[i][k] = (i == k && i >= D) ? 1.0 : 0.0; g.Finv[i][k] = g.F[i][k]; }
  }
  for (int i = 0; i < D; i++) g.x0[i] = elc[D * D + i];
  for (int k = 0; k < D; k++)
    for (int i = 0; i < D; i++) g.F[i][k] = elc[k * D + i] - elc[D * D + i];
  if (D == 2) {
    double a = g.F[0][0], b = g.F[0][1], c = g.F[1][0], d = g.F[1][1];
    g.det = a * d - b * c;
    double id = 1.0 / g.det;
    g.Finv[0][0] = d * id; g.Finv[0][1] = -b * id;
    g.Finv[1][0] = -c * id; g.Finv[1][1] = a * id;
  } else {
    const double(*F)[3] = g.F;
    double c00 = F[1][1] * F[2][2] - F[1][2] * F[2][1];
    double c01 = F[1][2] * F[2][0] - F[1][0] * F[2][2];
    double c02 = F[1][0] * F[2][1] - F[1][1] * F[2][0];
    g.det = F[0][0] * c00 + F[0][1] * c01 + F[0][2] * c02;
    double id = 1.0 / g.det;
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

// LevelsetWrapper gradient for simplices (straightcutrule.cpp:509-513, 525-538):
// constant reference gradient (v0-vD, v1-vD, v2-vD), normalised.
void lset_ref_normal(int D, const double* l, double* n) {
  double g[3] = {0, 0, 0};
  for (int k = 0; k < D; k++) g[k] = l[k] - l[D];
  double nn = l2norm3(g);
  double inv = 1.0 / nn;
  for (int k = 0; k < 3; k++) n[k] = g[k] * inv;
}

// straightcutrule.cpp:582-677 for simplices; returns #points, -1 for nullptr, <-1 error
int straight_cut_rule(const Geo& g, const double* lset, int dt, int order,
                      std::vector<double>& pts, std::vector<double>& wts) {
  int D = g.D;
  pts.clear(); wts.clear();
  int element_domain = check_if_straight_cut(lset, D + 1);
  if (element_domain == IF) {
    Sub subs[3];
    int ns = decompose(D, lset, dt, subs);
    if (ns < 0) return ns;
    for (int i = 0; i < ns; i++) plain_rule(subs[i], order, pts, wts);
    if (dt == IF) {
      // TransformQuadUntrafoToIRInterface (straightcutrule.cpp:558-578)
      double nref[3];
      lset_ref_normal(D, lset, nref);
      double nphys[3] = {0, 0, 0};
      for (int k = 0; k < D; k++) {
        double s = 0;
        for (int j = 0; j < D; j++) s += g.Finv[j][k] * nref[j];
        nphys[k] = s;
      }
      double fac = l2norm3(nphys);
      for (auto& w : wts) w = w * fac;
    }
    return (int)wts.size();
  }
  if (element_domain != dt) return -1;
  const Rule& r = get_rule(D, order);
  pts = r.p;
  wts = r.w;
  return r.size();
}

// ---------------------------------------------------------------------------
// H1 basis of this project (NGSolve's own shape functions are not available):
// vertex i: lambda_i; edge (a,b) with s/e the endpoints of smaller/larger global
// vertex number: lambda_s*lambda_e (k>=2), lambda_s*lambda_e*(lambda_s-lambda_e) (k=3);
// face (a,b,c) (3D, k=3) or cell (2D, k=3): lambda_a*lambda_b*lambda_c.
// Local order: vertices, then edges (dofs of one edge adjacent), then faces.
// ---------------------------------------------------------------------------
const int TRI_EDGES[3][2] = {{0, 1}, {0, 2}, {1, 2}};
const int TET_EDGES[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
const int TET_FACES[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

int ndof_el(int D, int k) { return D == 2 ? (k + 1) * (k + 2) / 2 : (k + 1) * (k + 2) * (k + 3) / 6; }

// phi[n], dphi[n][3] (reference gradient)
void basis(int D, int k, const int* gv, const double* xi, double* phi, double (*dphi)[3]) {
  double lam[4], dl[4][3];
  double s = 0;
  for (int i = 0; i < D; i++) { lam[i] = xi[i]; s += xi[i]; }
  lam[D] = 1.0 - s;
  for (int i = 0; i <= D; i++)
    for (int c = 0; c < 3; c++) dl[i][c] = (i < D) ? (c == i ? 1.0 : 0.0) : (c < D ? -1.0 : 0.0);
  int n = 0;
  for (int i = 0; i <= D; i++, n++) {
    phi[n] = lam[i];
    for (int c = 0; c < 3; c++) dphi[n][c] = dl[i][c];
  }
  if (k >= 2) {
    int ne = D == 2 ? 3 : 6;
    for (int e = 0; e < ne; e++) {
      int a = D == 2 ? TRI_EDGES[e][0] : TET_EDGES[e][0];
      int b = D == 2 ? TRI_EDGES[e][1] : TET_EDGES[e][1];
      int si = gv[a] < gv[b] ? a : b, ei = gv[a] < gv[b] ? b : a;
      double ls = lam[si], le = lam[ei];
      double q = ls * le;
      double dq[3];
      for (int c = 0; c < 3; c++) dq[c] = le * dl[si][c] + ls * dl[ei][c];
      phi[n] = q;
      for (int c = 0; c < 3; c++) dphi[n][c] = dq[c];
      n++;
      if (k >= 3) {
        double t = ls - le;
        phi[n] = q * t;
        for (int c = 0; c < 3; c++) dphi[n][c] = dq[c] * t + q * (dl[si][c] - dl[ei][c]);
        n++;
      }
    }
  }
  if (k >= 3) {
    int nf = D == 2 ? 1 : 4;
    for (int f = 0; f < nf; f++) {
      int a = D == 2 ? 0 : TET_FACES[f][0], b = D == 2 ? 1 : TET_FACES[f][1], c2 = D == 2 ? 2 : TET_FACES[f][2];
      phi[n] = lam[a] * lam[b] * lam[c2];
      for (int c = 0; c < 3; c++)
        dphi[n][c] = lam[b] * lam[c2] * dl[a][c] + lam[a] * lam[c2] * dl[b][c] + lam[a] * lam[b] * dl[c2][c];
      n++;
    }
  }
}

void parallel_for(int64_t n, int nthreads, const std::function<void(int64_t, int64_t)>& f) {
  if (nthreads <= 1 || n < 2 * nthreads) { f(0, n); return; }
  std::vector<std::thread> th;
  std::atomic<int64_t> next(0);
  const int64_t chunk = std::max<int64_t>(64, n / (nthreads * 16));
  for (int t = 0; t < nthreads; t++)
    th.emplace_back([&]() {
      for (;;) {
        int64_t b = next.fetch_add(chunk);
        if (b >= n) break;
        f(b, std::min(n, b + chunk));
      }
    });
  for (auto& t : th) t.join();
}

inline bool test_bit(const uint64_t* bits, int64_t i) { return (bits[i >> 6] >> (i & 63)) & 1u; }

}  // namespace

// ---------------------------------------------------------------------------
// Mesh / space
// ---------------------------------------------------------------------------
struct orc_space {
  int D, k, nv, ne, nd;  // nd = ndof per element
  std::vector<double> coords;
  std::vector<int32_t> elv;
  int64_t nedges = 0, nfaces = 0, nfacets = 0, ndof = 0;
  std::vector<int32_t> el_edges, el_faces, el_facets;  // per element
  std::vector<int32_t> facet_els;                      // 2 per facet, -1 boundary
  std::vector<int32_t> el_dofs;
  std::vector<int64_t> dof_adj_ptr;
  std::vector<int32_t> dof_adj;  // element*32 + local
};

extern "C" {

int orc_check_if_straight_cut(const double* vals, int n, double eps) {
  return check_if_straight_cut(vals, n, eps);
}

// utils/p1interpol.cpp:104-107
void orc_interpolate_p1_perturb(double* vals, int n, double eps) {
  for (int i = 0; i < n; i++)
    if (std::fabs(vals[i]) < eps) vals[i] = eps;
}

int orc_base_rule(int d, int p, double* pts, double* wts, int maxpts) {
  const Rule& r = get_rule(d, p);
  if (r.size() > maxpts) return ERR_CAPACITY;
  std::memcpy(pts, r.p.data(), sizeof(double) * 3 * r.size());
  std::memcpy(wts, r.w.data(), sizeof(double) * r.size());
  return r.size();
}

int orc_straight_cut_rule(int D, const double* elc, const double* lset, int dt, int order,
                          double* pts, double* wts, int maxpts) {
  Geo g;
  make_geo(D, elc, g);
  std::vector<double> p, w;
  int n = straight_cut_rule(g, lset, dt, order, p, w);
  if (n < 0) return n;
  if (n > maxpts) return ERR_CAPACITY;
  std::memcpy(pts, p.data(), sizeof(double) * 3 * n);
  std::memcpy(wts, w.data(), sizeof(double) * n);
  return n;
}

orc_space* orc_space_create(int D, int nv, const double* coords, int ne, const int32_t* elv, int order) {
  if ((D != 2 && D != 3) || order < 1 || order > 3) return nullptr;
  auto* s = new orc_space();
  s->D = D; s->k = order; s->nv = nv; s->ne = ne; s->nd = ndof_el(D, order);
  s->coords.assign(coords, coords + (size_t)nv * D);
  s->elv.assign(elv, elv + (size_t)ne * (D + 1));
  // edges: sorted unique (min,max) pairs
  const int ne_loc = D == 2 ? 3 : 6;
  std::vector<uint64_t> keys;
  keys.reserve((size_t)ne * ne_loc);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < ne_loc; j++) {
      int a = elv[e * (D + 1) + (D == 2 ? TRI_EDGES[j][0] : TET_EDGES[j][0])];
      int b = elv[e * (D + 1) + (D == 2 ? TRI_EDGES[j][1] : TET_EDGES[j][1])];
      if (a > b) std::swap(a, b);
      keys.push_back(((uint64_t)a << 32) | (uint32_t)b);
    }
  std::vector<uint64_t> ek(keys);
  std::sort(ek.begin(), ek.end());
  ek.erase(std::unique(ek.begin(), ek.end()), ek.end());
  s->nedges = (int64_t)ek.size();
  s->el_edges.resize((size_t)ne * ne_loc);
  for (size_t i = 0; i < keys.size(); i++)
    s->el_edges[i] = (int32_t)(std::lower_bound(ek.begin(), ek.end(), keys[i]) - ek.begin());
  // faces (3D): sorted unique triples, packed 21 bits each
  std::vector<uint64_t> fk;
  std::vector<uint64_t> fkeys;
  if (D == 3) {
    fkeys.reserve((size_t)ne * 4);
    for (int e = 0; e < ne; e++)
      for (int j = 0; j < 4; j++) {
        int v[3];
        for (int m = 0; m < 3; m++) v[m] = elv[e * 4 + TET_FACES[j][m]];
        std::sort(v, v + 3);
        fkeys.push_back(((uint64_t)v[0] << 42) | ((uint64_t)v[1] << 21) | (uint64_t)v[2]);
      }
    fk = fkeys;
    std::sort(fk.begin(), fk.end());
    fk.erase(std::unique(fk.begin(), fk.end()), fk.end());
    s->nfaces = (int64_t)fk.size();
    s->el_faces.resize((size_t)ne * 4);
    for (size_t i = 0; i < fkeys.size(); i++)
      s->el_faces[i] = (int32_t)(std::lower_bound(fk.begin(), fk.end(), fkeys[i]) - fk.begin());
  }
  // facets
  const int nfl = D + 1;
  s->nfacets = D == 2 ? s->nedges : s->nfaces;
  s->el_facets.resize((size_t)ne * nfl);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < nfl; j++)
      s->el_facets[(size_t)e * nfl + j] = D == 2 ? s->el_edges[(size_t)e * 3 + j] : s->el_faces[(size_t)e * 4 + j];
  s->facet_els.assign((size_t)s->nfacets * 2, -1);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < nfl; j++) {
      int f = s->el_facets[(size_t)e * nfl + j];
      if (s->facet_els[2 * f] < 0) s->facet_els[2 * f] = e;
      else s->facet_els[2 * f + 1] = e;
    }
  // dofs
  const int k = order;
  int64_t nbub = (k == 3) ? (D == 3 ? s->nfaces : ne) : 0;
  s->ndof = nv + s->nedges * (k - 1) + nbub;
  s->el_dofs.resize((size_t)ne * s->nd);
  for (int e = 0; e < ne; e++) {
    int32_t* d = &s->el_dofs[(size_t)e * s->nd];
    int n = 0;
    for (int i = 0; i <= D; i++) d[n++] = elv[e * (D + 1) + i];
    for (int j = 0; j < ne_loc && k >= 2; j++)
      for (int m = 0; m < k - 1; m++) d[n++] = (int32_t)(nv + (int64_t)s->el_edges[(size_t)e * ne_loc + j] * (k - 1) + m);
    if (k == 3) {
      if (D == 3)
        for (int j = 0; j < 4; j++) d[n++] = (int32_t)(nv + s->nedges * 2 + s->el_faces[(size_t)e * 4 + j]);
      else
        d[n++] = (int32_t)(nv + s->nedges * 2 + e);
    }
  }
  // dof -> (element, local) adjacency, ascending elements
  s->dof_adj_ptr.assign(s->ndof + 1, 0);
  for (size_t i = 0; i < s->el_dofs.size(); i++) s->dof_adj_ptr[s->el_dofs[i] + 1]++;
  for (int64_t i = 0; i < s->ndof; i++) s->dof_adj_ptr[i + 1] += s->dof_adj_ptr[i];
  s->dof_adj.resize(s->el_dofs.size());
  std::vector<int64_t> fill(s->dof_adj_ptr.begin(), s->dof_adj_ptr.end() - 1);
  for (int e = 0; e < ne; e++)
    for (int i = 0; i < s->nd; i++) s->dof_adj[fill[s->el_dofs[(size_t)e * s->nd + i]]++] = e * 32 + i;
  return s;
}

void orc_space_destroy(orc_space* s) { delete s; }

// L2(mesh, order, dgjumps=True) stand-in: the H1 element basis with
// element-local dofs (the reference's L2 uses NGSolve's own discontinuous
// basis; any basis of P_k per element spans the same space).
orc_space* orc_space_create_l2(int D, int nv, const double* coords, int ne, const int32_t* elv, int order) {
  orc_space* s = orc_space_create(D, nv, coords, ne, elv, order);
  if (!s) return nullptr;
  s->ndof = (int64_t)ne * s->nd;
  for (int e = 0; e < ne; e++)
    for (int i = 0; i < s->nd; i++) s->el_dofs[(size_t)e * s->nd + i] = (int32_t)((int64_t)e * s->nd + i);
  s->dof_adj_ptr.assign(s->ndof + 1, 0);
  s->dof_adj.resize(s->el_dofs.size());
  for (int64_t i = 0; i < s->ndof; i++) {
    s->dof_adj_ptr[i + 1] = i + 1;
    s->dof_adj[i] = (int32_t)((i / s->nd) * 32 + i % s->nd);
  }
  return s;
}

int orc_space_info(const orc_space* s, int64_t* out) {
  out[0] = s->ndof; out[1] = s->nedges; out[2] = s->nfaces; out[3] = s->nfacets; out[4] = s->nd;
  return 0;
}
int orc_space_el_dofs(const orc_space* s, int32_t* out) {
  std::memcpy(out, s->el_dofs.data(), sizeof(int32_t) * s->el_dofs.size());
  return 0;
}
int orc_space_facet_els(const orc_space* s, int32_t* out) {
  std::memcpy(out, s->facet_els.data(), sizeof(int32_t) * s->facet_els.size());
  return 0;
}

}  // extern "C"

namespace {

void element_geo(const orc_space* s, int e, Geo& g, double* lset_el, const double* lset_vertex) {
  double elc[12];
  const int D = s->D;
  for (int i = 0; i <= D; i++) {
    int v = s->elv[(size_t)e * (D + 1) + i];
    for (int c = 0; c < D; c++) elc[i * D + c] = s->coords[(size_t)v * D + c];
    if (lset_el) lset_el[i] = lset_vertex[v];
  }
  make_geo(D, elc, g);
}

void phys_grad(const Geo& g, const double* dref, double* dphys) {
  // grad_x = F^{-T} grad_xi
  for (int i = 0; i < 3; i++) {
    double s = 0;
    for (int k = 0; k < g.D; k++) s += g.Finv[k][i] * dref[k];
    dphys[i] = (i < g.D) ? s : 0.0;
  }
}

int default_order(int kind, int k) {
  switch (kind) {
    case ORC_TERM_MASS: return 2 * k;
    case ORC_TERM_LAPLACE: return 2 * k - 2;
    case ORC_TERM_NGRADU_V: case ORC_TERM_U_NGRADV: case ORC_TERM_CONV: return 2 * k - 1;
    case ORC_TERM_GHOST_MASS: return 2 * k;
    case ORC_TERM_NGRADU_NGRADV: return 2 * k - 2;
  }
  return 2 * k;
}

double hcoef(const orc_term& t, const Geo& g) {
  double c = t.coef;
  if (t.hpow != 0) {
    double h = std::pow(std::fabs(g.det), 1.0 / g.D);
    c *= std::pow(h, (double)t.hpow);
  }
  return c;
}

// T_CalcElementMatrixAdd (symboliccutbfi.cpp:76-313) restated for the term menu.
int element_matrix(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms, int e,
                   double* elmat) {
  const int D = s->D, n = s->nd;
  Geo g;
  double l[4];
  element_geo(s, e, g, l, lset_vertex);
  const int* gv = &s->elv[(size_t)e * (D + 1)];
  std::vector<double> pts, wts;
  double phi[20], dphi[20][3], gphys[20][3];
  std::fill(elmat, elmat + n * n, 0.0);
  // unit normal of the P1 level set (Normalize(grad(lsetp1)))
  double gl[3] = {0, 0, 0}, nrm[3];
  {
    double gr[3] = {0, 0, 0};
    for (int k = 0; k < D; k++) gr[k] = l[k] - l[D];
    phys_grad(g, gr, gl);
    double nn = l2norm3(gl);
    for (int c = 0; c < 3; c++) nrm[c] = gl[c] / nn;
  }
  for (int t = 0; t < nterms; t++) {
    const orc_term& T = terms[t];
    if (T.kind == ORC_TERM_GHOST_MASS || T.kind >= ORC_TERM_SKEL_JUMP) continue;
    if (T.defined_on && !test_bit(T.defined_on, e)) continue;
    int order = T.order >= 0 ? T.order : default_order(T.kind, s->k);
    int np = straight_cut_rule(g, l, T.domain, order, pts, wts);
    if (np < -1) return np;
    if (np <= 0) continue;
    double c = hcoef(T, g);
    double meas = std::fabs(g.det);
    for (int q = 0; q < np; q++) {
      basis(D, s->k, gv, &pts[3 * q], phi, dphi);
      for (int i = 0; i < n; i++) phys_grad(g, dphi[i], gphys[i]);
      double w = wts[q] * meas * c;
      for (int i = 0; i < n; i++)      // test
        for (int j = 0; j < n; j++) {  // trial
          double v;
          switch (T.kind) {
            case ORC_TERM_MASS: v = phi[i] * phi[j]; break;
            case ORC_TERM_LAPLACE: v = gphys[i][0] * gphys[j][0] + gphys[i][1] * gphys[j][1] + gphys[i][2] * gphys[j][2]; break;
            case ORC_TERM_NGRADU_V: v = (nrm[0] * gphys[j][0] + nrm[1] * gphys[j][1] + nrm[2] * gphys[j][2]) * phi[i]; break;
            case ORC_TERM_U_NGRADV: v = phi[j] * (nrm[0] * gphys[i][0] + nrm[1] * gphys[i][1] + nrm[2] * gphys[i][2]); break;
            case ORC_TERM_CONV: v = (T.b[0] * gphys[j][0] + T.b[1] * gphys[j][1] + T.b[2] * gphys[j][2]) * phi[i]; break;
            default: v = 0;
          }
          elmat[i * n + j] += w * v;
        }
    }
  }
  return 0;
}

// Coefficient terms: T_CalcElementMatrixAdd with the CoefficientFunction
// evaluated at the rule's points (symboliccutbfi.cpp:168-194), here a field
// given by its element coefficients times a monomial of x; added to elmat.
int element_matrix_coef(const orc_space* s, const double* lset_vertex, const orc_cterm* terms, int nterms, int e,
                        double* elmat) {
  const int D = s->D, n = s->nd;
  Geo g;
  double l[4];
  element_geo(s, e, g, l, lset_vertex);
  const int* gv = &s->elv[(size_t)e * (D + 1)];
  std::vector<double> pts, wts;
  double phi[20], dphi[20][3], gphys[20][3], phig[20], dphig[20][3];
  double gl[3] = {0, 0, 0}, nrm[3];
  {
    double gr[3] = {0, 0, 0};
    for (int k = 0; k < D; k++) gr[k] = l[k] - l[D];
    phys_grad(g, gr, gl);
    double nn = l2norm3(gl);
    for (int c = 0; c < 3; c++) nrm[c] = gl[c] / nn;
  }
  for (int t = 0; t < nterms; t++) {
    const orc_cterm& T = terms[t];
    if (T.defined_on && !test_bit(T.defined_on, e)) continue;
    const int order = T.order >= 0 ? T.order : default_order(T.kind, s->k);
    // on the deformed mesh: the rule of the reference element (its weights
    // in reference measure), mapped point by point
    const double* th = T.theta_el ? T.theta_el + (size_t)e * 18 : nullptr;
    Geo gref;
    if (th) {
      const double ref2[6] = {1, 0, 0, 1, 0, 0}, ref3[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
      make_geo(D, D == 2 ? ref2 : ref3, gref);
    }
    // the whole element (dx): the element's own rule, whatever the cut
    int np;
    if (T.domain == ORC_WHOLE) {
      const Rule& r = get_rule(D, order);
      pts = r.p;
      wts = r.w;
      np = r.size();
    } else {
      np = straight_cut_rule(th ? gref : g, l, T.domain, order, pts, wts);
    }
    if (np < -1) return np;
    if (np <= 0) continue;
    double c = T.coef;
    if (T.hpow != 0) c *= std::pow(std::pow(std::fabs(g.det), 1.0 / D), (double)T.hpow);
    const double meas = std::fabs(g.det);
    const int ng = T.gf_order > 0 ? (D == 2 ? (T.gf_order + 1) * (T.gf_order + 2) / 2
                                            : (T.gf_order + 1) * (T.gf_order + 2) * (T.gf_order + 3) / 6)
                                  : 0;
    for (int q = 0; q < np; q++) {
      const double* xi = &pts[3 * q];
      basis(D, s->k, gv, xi, phi, dphi);
      double wq = wts[q] * meas, cq = c, xq[3] = {0, 0, 0};
      const double* bnq = nrm;
      double nq[3] = {0, 0, 0};
      if (!th) {
        for (int i = 0; i < n; i++) phys_grad(g, dphi[i], gphys[i]);
        for (int r = 0; r < D; r++) {
          double acc = g.x0[r];
          for (int k = 0; k < D; k++) acc += g.F[r][k] * xi[k];
          xq[r] = acc;
        }
      } else {
        // y = xi + Theta(xi), A = I + grad Theta (edge shapes lambda_a lambda_b), F = J A
        double lam[4], sl = 0.0;
        for (int k = 0; k < D; k++) {
          lam[k] = xi[k];
          sl += xi[k];
        }
        lam[D] = 1.0 - sl;
        double y[3] = {xi[0], xi[1], D == 3 ? xi[2] : 0.0}, Am[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        const int E2[3][2] = {{0, 1}, {0, 2}, {1, 2}}, E3[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
        for (int j = 0; j < (D == 2 ? 3 : 6); j++) {
          const int a = D == 2 ? E2[j][0] : E3[j][0], b = D == 2 ? E2[j][1] : E3[j][1];
          const double ph = lam[a] * lam[b];
          double dph[3];
          for (int k = 0; k < D; k++) {
            const double da = a < D ? (a == k ? 1.0 : 0.0) : -1.0, db = b < D ? (b == k ? 1.0 : 0.0) : -1.0;
            dph[k] = da * lam[b] + lam[a] * db;
          }
          for (int r = 0; r < D; r++) {
            y[r] += th[j * 3 + r] * ph;
            for (int k = 0; k < D; k++) Am[r][k] += th[j * 3 + r] * dph[k];
          }
        }
        double elc[12];
        Geo gd;  // the point's Jacobian F = J A as an element map (for its inverse and determinant)
        {
          double F[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
          for (int r = 0; r < D; r++)
            for (int k = 0; k < D; k++)
              for (int q2 = 0; q2 < D; q2++) F[r][k] += g.F[r][q2] * Am[q2][k];
          for (int v = 0; v <= D; v++)
            for (int r = 0; r < D; r++) elc[v * D + r] = v < D ? F[r][v] : 0.0;
          make_geo(D, elc, gd);
        }
        for (int i = 0; i < n; i++) phys_grad(gd, dphi[i], gphys[i]);
        double gr[3] = {0, 0, 0}, gp[3];
        for (int k = 0; k < D; k++) gr[k] = l[k] - l[D];
        phys_grad(gd, gr, gp);
        const double gpn = l2norm3(gp), grn = l2norm3(gr);
        for (int r = 0; r < 3; r++) nq[r] = gp[r] / gpn;
        bnq = nq;
        wq = wts[q] * std::fabs(gd.det);
        if (T.domain == ORC_IF) wq *= gpn / grn;
        if (T.hpow != 0) cq = T.coef * std::pow(std::pow(std::fabs(gd.det), 1.0 / D), (double)T.hpow);
        for (int r = 0; r < D; r++) {
          double acc = g.x0[r];
          for (int k = 0; k < D; k++) acc += g.F[r][k] * y[k];
          xq[r] = acc;
        }
      }
      double f = 1.0;
      if (ng > 0) {
        basis(D, T.gf_order, gv, xi, phig, dphig);
        f = 0.0;
        for (int i = 0; i < ng; i++) f += T.gf_el[(size_t)e * ng + i] * phig[i];
      }
      if (T.e[0] || T.e[1] || T.e[2])
        for (int r = 0; r < 3; r++)
          for (int p = 0; p < T.e[r]; p++) f *= xq[r];
      const double w = wq * cq * f;
      const double* bb = T.kind == ORC_TERM_CONV ? T.b : bnq;
      for (int i = 0; i < n; i++)      // test
        for (int j = 0; j < n; j++) {  // trial
          double v;
          switch (T.kind) {
            case ORC_TERM_MASS: v = phi[i] * phi[j]; break;
            case ORC_TERM_LAPLACE: v = gphys[i][0] * gphys[j][0] + gphys[i][1] * gphys[j][1] + gphys[i][2] * gphys[j][2]; break;
            case ORC_TERM_U_NGRADV: v = phi[j] * (bb[0] * gphys[i][0] + bb[1] * gphys[i][1] + bb[2] * gphys[i][2]); break;
            case ORC_TERM_NGRADU_NGRADV:
              v = (bb[0] * gphys[j][0] + bb[1] * gphys[j][1] + bb[2] * gphys[j][2]) *
                  (bb[0] * gphys[i][0] + bb[1] * gphys[i][1] + bb[2] * gphys[i][2]);
              break;
            default: v = (bb[0] * gphys[j][0] + bb[1] * gphys[j][1] + bb[2] * gphys[j][2]) * phi[i]; break;
          }
          elmat[i * n + j] += w * v;
        }
    }
  }
  return 0;
}

// MapPatchIntegrationPoint (symboliccutbfi.cpp:1747-1846) for affine elements.
void map_patch_point(const Geo& from, const Geo& to, const double* xi_from, double w_from, double* xi_to,
                     double* w_to) {
  const int D = from.D;
  double vec[3] = {0, 0, 0};
  for (int i = 0; i < D; i++) {
    double sacc = from.x0[i];
    for (int k = 0; k < D; k++) sacc += from.F[i][k] * xi_from[k];
    vec[i] = sacc;
  }
  const double h = std::sqrt(from.det);  // GetJacobiDet (may be negative -> NaN as in the reference)
  // low order guess: A = [x(e_d) - x(0)] = F_to, x00 = A^{-1} (vec - x(0))
  double x00[3] = {0, 0, 0}, f[3];
  for (int i = 0; i < D; i++) f[i] = vec[i] - to.x0[i];
  for (int i = 0; i < D; i++) {
    double sacc = 0;
    for (int k = 0; k < D; k++) sacc += to.Finv[i][k] * f[k];
    x00[i] = sacc;
  }
  double x0[3] = {x00[0], x00[1], x00[2]};
  const double eps = 1e-12;  // EPS_FACET_PATCH_INTEGRATOR (utils/ngsxstd.cpp:72)
  const int maxit = 15;      // NEWTON_ITER_TRESHOLD (utils/ngsxstd.cpp:73)
  int its = 0;
  double diffn = 0, w = 0;
  while (its == 0 || (diffn > eps * h && its < maxit)) {
    double diff[3];
    for (int i = 0; i < D; i++) {
      double sacc = to.x0[i];
      for (int k = 0; k < D; k++) sacc += to.F[i][k] * x0[k];
      diff[i] = vec[i] - sacc;
    }
    diffn = 0;
    for (int i = 0; i < D; i++) diffn += diff[i] * diff[i];
    diffn = std::sqrt(diffn);
    for (int i = 0; i < D; i++) {
      double sacc = 0;
      for (int k = 0; k < D; k++) sacc += to.Finv[i][k] * diff[k];
      x0[i] += sacc;
    }
    its++;
    w = std::fabs(to.det);
  }
  double mipw = w_from * std::fabs(from.det);
  double dist = 0;
  for (int i = 0; i < D; i++) dist += (x0[i] - x00[i]) * (x0[i] - x00[i]);
  dist = std::sqrt(dist);
  if (its >= maxit || diffn > eps * h || dist > 10.0) {
    for (int i = 0; i < 3; i++) xi_to[i] = x00[i];
    *w_to = mipw / std::fabs(to.det);
  } else {
    for (int i = 0; i < 3; i++) xi_to[i] = x0[i];
    *w_to = mipw / w;
  }
}

// T_CalcFacetMatrix (symboliccutbfi.cpp:1982-2377), non-space-time, downscale = 1.
int patch_matrix(const orc_space* s, const orc_term* terms, int nterms, int f, double* elmat) {
  const int D = s->D, n = s->nd, n2 = 2 * n;
  std::fill(elmat, elmat + n2 * n2, 0.0);
  int e1 = s->facet_els[2 * f], e2 = s->facet_els[2 * f + 1];
  if (e1 < 0 || e2 < 0) return -5;  // LocalFacetNr2==-1 (symboliccutbfi.cpp:1992)
  Geo g1, g2;
  element_geo(s, e1, g1, nullptr, nullptr);
  element_geo(s, e2, g2, nullptr, nullptr);
  const int* gv1 = &s->elv[(size_t)e1 * (D + 1)];
  const int* gv2 = &s->elv[(size_t)e2 * (D + 1)];
  for (int t = 0; t < nterms; t++) {
    const orc_term& T = terms[t];
    if (T.kind != ORC_TERM_GHOST_MASS) continue;
    if (T.defined_on && !test_bit(T.defined_on, f)) continue;
    int order = T.order >= 0 ? T.order : 2 * s->k;
    const Rule& r = get_rule(D, order);
    const int nq = r.size();
    std::vector<double> p1(3 * 2 * nq, 0.0), p2(3 * 2 * nq, 0.0), w1(2 * nq);
    for (int l = 0; l < 2 * nq; l++) {
      if (l < nq) {
        for (int c = 0; c < 3; c++) p1[3 * l + c] = r.p[3 * l + c];
        w1[l] = r.w[l];
        double wdummy;
        map_patch_point(g1, g2, &p1[3 * l], w1[l], &p2[3 * l], &wdummy);
      } else {
        int m = l - nq;
        for (int c = 0; c < 3; c++) p2[3 * l + c] = r.p[3 * m + c];
        map_patch_point(g2, g1, &p2[3 * l], r.w[m], &p1[3 * l], &w1[l]);
      }
    }
    double c = hcoef(T, g1);
    double phi1[20], phi2[20], dphi[20][3];
    double sh[40];
    for (int l = 0; l < 2 * nq; l++) {
      basis(D, s->k, gv1, &p1[3 * l], phi1, dphi);
      basis(D, s->k, gv2, &p2[3 * l], phi2, dphi);
      for (int i = 0; i < n; i++) { sh[i] = phi1[i]; sh[n + i] = -phi2[i]; }
      double W = w1[l] * std::fabs(g1.det) * c;
      for (int i = 0; i < n2; i++)
        for (int j = 0; j < n2; j++) elmat[i * n2 + j] += W * sh[i] * sh[j];
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Skeleton terms on interior facets.
//
// SymbolicCutFacetBilinearFormIntegrator::T_CalcFacetMatrix
// (symboliccutbfi.cpp:886-1572): the facet's level-set values (the P1 vertex
// values) give StraightCutIntegrationRuleUntransformed on the facet simplex
// with order 2 * maxorder (:947-1042); the rule is mapped into both elements
// (Facet2ElementTrafo, :1044-1048) and weighted by the facet measure of the
// first element's mapped point (:1126-1130, codim 1).  The uncut facet
// integrator SymbolicFacetBilinearFormIntegrator2 (:1574-1735) is the same on
// the plain facet rule.  Test and trial functions of the first element fill
// rows / columns [0, n), those of the second (.Other()) [n, 2n) (:1098-1109).
// The integrands are the menu ORC_TERM_SKEL_*; dn(w, k) of the reference
// (python_xfem.cpp:1068-1150, DiffOpDuDnk) differentiates along the normal of
// the element w lives on, so with n_F = the first element's outward normal
// the jump [d^k_n w] = d^k_nF w - d^k_nF w' is dn(w, k) - (-1)^k dn(w.Other(), k).
// ---------------------------------------------------------------------------

// CentralFDStencils (ghostpenalty.cpp:8-140): the central stencil of width
// w = acc/2 + floor(k - 1/2)/2 with sum_l c_l (l - w)^m / m! = delta_{m,k}
// (m = 0 .. 2w), by Gaussian elimination with partial pivoting; GetOptimalEps
// = ((2w + 1) eps_mach)^(1 / (acc + k)).
int fd_stencil(int k, int acc, double* c, double* eps) {
  const int w = (acc + 1) / 2 + (int)(k - 0.5) / 2, n = 2 * w + 1;
  std::vector<double> A((size_t)n * (n + 1));
  double inv_fact = 1.0;
  for (int m = 0; m < n; m++) {
    if (m > 0) inv_fact /= m;
    for (int l = 0; l < n; l++) A[(size_t)m * (n + 1) + l] = std::pow((double)(l - w), m) * inv_fact;
    A[(size_t)m * (n + 1) + n] = m == k ? 1.0 : 0.0;
  }
  for (int col = 0; col < n; col++) {
    int piv = col;
    for (int r = col + 1; r < n; r++)
      if (std::fabs(A[(size_t)r * (n + 1) + col]) > std::fabs(A[(size_t)piv * (n + 1) + col])) piv = r;
    if (piv != col)
      for (int q = 0; q <= n; q++) std::swap(A[(size_t)col * (n + 1) + q], A[(size_t)piv * (n + 1) + q]);
    for (int r = 0; r < n; r++) {
      if (r == col) continue;
      const double fct = A[(size_t)r * (n + 1) + col] / A[(size_t)col * (n + 1) + col];
      for (int q = col; q <= n; q++) A[(size_t)r * (n + 1) + q] -= fct * A[(size_t)col * (n + 1) + q];
    }
  }
  for (int l = 0; l < n; l++) c[l] = A[(size_t)l * (n + 1) + n] / A[(size_t)l * (n + 1) + l];
  *eps = std::pow((2 * w + 1) * 2.220446049250313e-16, 1.0 / (acc + k));
  return w;
}

// barycentric coordinates of the physical point x in element g
void phys_to_lam(const Geo& g, const double* x, double* lam) {
  const int D = g.D;
  double s = 0;
  for (int i = 0; i < D; i++) {
    double v = 0;
    for (int k = 0; k < D; k++) v += g.Finv[i][k] * (x[k] - g.x0[k]);
    lam[i] = v;
    s += v;
  }
  lam[D] = 1.0 - s;
}

// d lambda_i / d n (physical direction n) for all D + 1 barycentrics
void lam_dir(const Geo& g, const double* n, double* del) {
  const int D = g.D;
  double s = 0;
  for (int i = 0; i < D; i++) {
    double v = 0;
    for (int k = 0; k < D; k++) v += g.Finv[i][k] * n[k];
    del[i] = v;
    s += v;
  }
  del[D] = -s;
}

// j-th derivative along t of prod_m lambda_f[m](x + t n) at t = 0: j! times the
// coefficient of t^j in prod_m (lam_f[m] + t del_f[m])
double prod_dir(const int* f, int nf, const double* lam, const double* del, int j) {
  if (j > nf) return 0.0;
  double poly[4] = {1.0, 0.0, 0.0, 0.0};
  for (int m = 0; m < nf; m++) {
    for (int p = m + 1; p >= 1; p--) poly[p] = poly[p] * lam[f[m]] + poly[p - 1] * del[f[m]];
    poly[0] *= lam[f[m]];
  }
  double fact = 1.0;
  for (int i = 2; i <= j; i++) fact *= i;
  return fact * poly[j];
}

// j-th derivative along n of every basis function (the products of basis())
void basis_dir(int D, int k, const int* gv, const double* lam, const double* del, int j, double* out) {
  int n = 0;
  for (int i = 0; i <= D; i++) {
    const int f[1] = {i};
    out[n++] = prod_dir(f, 1, lam, del, j);
  }
  if (k >= 2) {
    const int ne = D == 2 ? 3 : 6;
    for (int e = 0; e < ne; e++) {
      const int a = D == 2 ? TRI_EDGES[e][0] : TET_EDGES[e][0];
      const int b = D == 2 ? TRI_EDGES[e][1] : TET_EDGES[e][1];
      const int si = gv[a] < gv[b] ? a : b, ei = gv[a] < gv[b] ? b : a;
      const int q[2] = {si, ei};
      out[n++] = prod_dir(q, 2, lam, del, j);
      if (k >= 3) {
        const int c1[3] = {si, si, ei}, c2[3] = {si, ei, ei};
        out[n++] = prod_dir(c1, 3, lam, del, j) - prod_dir(c2, 3, lam, del, j);
      }
    }
  }
  if (k >= 3) {
    const int nf = D == 2 ? 1 : 4;
    for (int f = 0; f < nf; f++) {
      const int t[3] = {D == 2 ? 0 : TET_FACES[f][0], D == 2 ? 1 : TET_FACES[f][1], D == 2 ? 2 : TET_FACES[f][2]};
      out[n++] = prod_dir(t, 3, lam, del, j);
    }
  }
}

// DiffOpDuDnk<D, k>::GenerateMatrix, version 2 (ghostpenalty.cpp:268-340) on an
// affine element: the basis values at x + (i - w) eps n, eps = h * GetOptimalEps,
// h = |det F|^(1/D) (the reference takes sqrt / cbrt of the signed determinant),
// combined with the stencil and scaled by eps^-k.  The back-mapping of the
// shifted points is exact for affine elements (its Newton loop stops at once).
void basis_dn_fd(const Geo& g, int k_fe, const int* gv, const double* x, const double* nside, int k, double* out) {
  const int D = g.D, n = ndof_el(D, k_fe);
  double c[16], epsf;
  const int w = fd_stencil(k, 4, c, &epsf);
  const double h = std::pow(std::fabs(g.det), 1.0 / D);
  const double eps = h * epsf;
  std::fill(out, out + n, 0.0);
  double phi[20], dphi[20][3];
  for (int i = 0; i <= 2 * w; i++) {
    double xi[3] = {0, 0, 0}, lam[4];
    for (int d = 0; d < D; d++) xi[d] = x[d] + (i - w) * eps * nside[d];
    phys_to_lam(g, xi, lam);
    basis(D, k_fe, gv, lam, phi, dphi);
    for (int a = 0; a < n; a++) out[a] += c[i] * phi[a];
  }
  const double fac = std::pow(1.0 / eps, k);
  for (int a = 0; a < n; a++) out[a] *= fac;
}

// the facet rule in the facet's reference coordinates: the plain rule of the
// (D-1)-simplex (ORC_WHOLE) or its straight-cut rule for the domain
int facet_rule(int d, const double* lf, int region, int order, std::vector<double>& pts, std::vector<double>& wts) {
  if (region == ORC_WHOLE) {
    const Rule& r = get_rule(d, order);
    pts = r.p;
    wts = r.w;
    return r.size();
  }
  Geo gd;
  gd.D = d;
  return straight_cut_rule(gd, lf, region, order, pts, wts);
}

bool is_skel(int kind) { return kind >= ORC_TERM_SKEL_JUMP && kind <= ORC_TERM_SKEL_DN3; }

// skeleton terms of facet f added to elmat ((2n)^2, row = test)
int skel_add(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms, int f, int dn_fd,
             double* elmat) {
  const int D = s->D, n = s->nd, n2 = 2 * n, d = D - 1;
  const int e1 = s->facet_els[2 * f], e2 = s->facet_els[2 * f + 1];
  if (e1 < 0 || e2 < 0) return -5;
  Geo g1, g2;
  element_geo(s, e1, g1, nullptr, nullptr);
  element_geo(s, e2, g2, nullptr, nullptr);
  const int* gv1 = &s->elv[(size_t)e1 * (D + 1)];
  const int* gv2 = &s->elv[(size_t)e2 * (D + 1)];
  // the facet: e1's vertices except the one e2 does not have (e1's local order)
  int opp1 = -1, fv[3], nfv = 0;
  for (int i = 0; i <= D; i++) {
    bool shared = false;
    for (int j = 0; j <= D; j++) shared |= gv1[i] == gv2[j];
    if (!shared) opp1 = i;
    else if (nfv < D) fv[nfv++] = gv1[i];
  }
  if (opp1 < 0 || nfv != D) return -5;
  double X[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, lf[3];
  for (int i = 0; i < D; i++) {
    for (int c = 0; c < D; c++) X[i][c] = s->coords[(size_t)fv[i] * D + c];
    lf[i] = lset_vertex ? lset_vertex[fv[i]] : 0.0;
  }
  double meas;
  if (d == 1) {
    const double v[3] = {X[0][0] - X[1][0], X[0][1] - X[1][1], 0.0};
    meas = l2norm3(v);
  } else {
    double a[3], b[3];
    for (int c = 0; c < 3; c++) { a[c] = X[0][c] - X[2][c]; b[c] = X[1][c] - X[2][c]; }
    const double cr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    meas = l2norm3(cr);
  }
  // outward normal of e1: -grad lambda_opp1 / |grad lambda_opp1|
  double nF[3] = {0, 0, 0};
  {
    double gl[3] = {0, 0, 0};
    for (int c = 0; c < D; c++) {
      double v = 0;
      if (opp1 < D) v = g1.Finv[opp1][c];
      else for (int i = 0; i < D; i++) v -= g1.Finv[i][c];
      gl[c] = v;
    }
    const double nn = l2norm3(gl);
    for (int c = 0; c < 3; c++) nF[c] = -gl[c] / nn;
  }
  const double mnF[3] = {-nF[0], -nF[1], -nF[2]};
  double del1[4], del2[4];
  lam_dir(g1, nF, del1);
  lam_dir(g2, nF, del2);
  const double h1 = std::pow(std::fabs(g1.det), 1.0 / D);
  std::vector<double> pts, wts;
  std::vector<double> P((size_t)4 * n2);  // P[j][a]: d^j_nF of function a (a < n: e1, else e2)
  for (int t = 0; t < nterms; t++) {
    const orc_term& T = terms[t];
    if (!is_skel(T.kind)) continue;
    if (T.defined_on && !test_bit(T.defined_on, f)) continue;
    if (T.domain == ORC_IF) return -6;  // codim-2 skeleton rules are not part of the menu
    const int np = facet_rule(d, lf, T.domain, 2 * s->k, pts, wts);
    if (np < -1) return np;
    if (np <= 0) continue;
    double c = T.coef;
    if (T.hpow != 0) c *= std::pow(h1, (double)T.hpow);
    const int kd = T.kind >= ORC_TERM_SKEL_DN1 ? T.kind - ORC_TERM_SKEL_DN1 + 1 : 0;
    for (int q = 0; q < np; q++) {
      const double* xi = &pts[3 * q];
      double x[3] = {0, 0, 0}, rest = 1.0;
      for (int m = 0; m < d; m++) rest -= xi[m];
      for (int c2 = 0; c2 < D; c2++) {
        double v = rest * X[d][c2];
        for (int m = 0; m < d; m++) v += xi[m] * X[m][c2];
        x[c2] = v;
      }
      double lam1[4], lam2[4];
      phys_to_lam(g1, x, lam1);
      phys_to_lam(g2, x, lam2);
      for (int j = 0; j <= 1; j++) {
        basis_dir(D, s->k, gv1, lam1, del1, j, &P[(size_t)j * n2]);
        basis_dir(D, s->k, gv2, lam2, del2, j, &P[(size_t)j * n2 + n]);
      }
      if (kd > 0) {
        double* Pk = &P[(size_t)2 * n2];
        if (!dn_fd) {
          basis_dir(D, s->k, gv1, lam1, del1, kd, Pk);
          basis_dir(D, s->k, gv2, lam2, del2, kd, Pk + n);
        } else {
          // dn(w, k) of each side along its own outward normal, turned to n_F
          basis_dn_fd(g1, s->k, gv1, x, nF, kd, Pk);
          basis_dn_fd(g2, s->k, gv2, x, mnF, kd, Pk + n);
          if (kd & 1)
            for (int a = 0; a < n; a++) Pk[n + a] = -Pk[n + a];
        }
      }
      const double W = wts[q] * meas * c;
      const double* P0 = &P[0];
      const double* P1 = &P[(size_t)n2];
      const double* Pk = &P[(size_t)2 * n2];
      for (int a = 0; a < n2; a++) {  // test
        const double sa = a < n ? 1.0 : -1.0;
        for (int b = 0; b < n2; b++) {  // trial
          const double sb = b < n ? 1.0 : -1.0;
          double v;
          switch (T.kind) {
            case ORC_TERM_SKEL_JUMP: v = sa * P0[a] * sb * P0[b]; break;
            case ORC_TERM_SKEL_FLUX: v = P1[b] * sa * P0[a]; break;
            case ORC_TERM_SKEL_FLUX_T: v = sb * P0[b] * P1[a]; break;
            default: v = sa * Pk[a] * sb * Pk[b]; break;
          }
          elmat[a * n2 + b] += W * v;
        }
      }
    }
  }
  return 0;
}

// patch terms, then skeleton terms, of facet f
// The deformed element map x(xi) = x0 + F (xi + Theta(xi)) (edge shapes
// lambda_a lambda_b, th[6][3] in the reference frame) and its Jacobian F A.
void deformed_map(const Geo& g, const double* th, const double* xi, double* x, double (*FA)[3]) {
  const int D = g.D;
  double lam[4], sl = 0.0;
  for (int k = 0; k < D; k++) {
    lam[k] = xi[k];
    sl += xi[k];
  }
  lam[D] = 1.0 - sl;
  double y[3] = {xi[0], xi[1], D == 3 ? xi[2] : 0.0}, Am[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  const int E2[3][2] = {{0, 1}, {0, 2}, {1, 2}}, E3[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  for (int j = 0; j < (D == 2 ? 3 : 6); j++) {
    const int a = D == 2 ? E2[j][0] : E3[j][0], b = D == 2 ? E2[j][1] : E3[j][1];
    const double ph = lam[a] * lam[b];
    for (int k = 0; k < D; k++) {
      const double da = a < D ? (a == k ? 1.0 : 0.0) : -1.0, db = b < D ? (b == k ? 1.0 : 0.0) : -1.0;
      const double dph = da * lam[b] + lam[a] * db;
      for (int r = 0; r < D; r++) Am[r][k] += th[j * 3 + r] * dph;
    }
    for (int r = 0; r < D; r++) y[r] += th[j * 3 + r] * ph;
  }
  for (int r = 0; r < 3; r++) {
    x[r] = 0.0;
    for (int k = 0; k < 3; k++) FA[r][k] = 0.0;
  }
  for (int r = 0; r < D; r++) {
    double acc = g.x0[r];
    for (int k = 0; k < D; k++) acc += g.F[r][k] * y[k];
    x[r] = acc;
    for (int k = 0; k < D; k++)
      for (int q = 0; q < D; q++) FA[r][k] += g.F[r][q] * Am[q][k];
  }
}

// the D x D matrix as a Geo (for its inverse and determinant)
Geo as_geo(int D, const double (*M)[3]) {
  double elc[12];
  for (int v = 0; v <= D; v++)
    for (int r = 0; r < D; r++) elc[v * D + r] = v < D ? M[r][v] : 0.0;
  Geo g;
  make_geo(D, elc, g);
  return g;
}

// MapPatchIntegrationPoint (symboliccutbfi.cpp:1747-1846) with the deformed
// maps: the point of `from` at xi_from sent into `to`; the low-order guess
// uses the vertex positions (which the deformation leaves in place), the
// Newton steps the deformed Jacobian at the current point.  Returns
// |det| of `from` at the point (the physical weight factor).
double map_patch_point_def(const Geo& from, const double* thf, const Geo& to, const double* tht, const double* xi_from,
                           double* xi_to) {
  const int D = from.D;
  double vec[3], FA[3][3];
  deformed_map(from, thf, xi_from, vec, FA);
  const double det_from = as_geo(D, FA).det;
  const double h = std::sqrt(det_from);  // NaN for a negative determinant, as in the affine statement
  double x00[3] = {0, 0, 0}, f[3];
  for (int i = 0; i < D; i++) f[i] = vec[i] - to.x0[i];
  for (int i = 0; i < D; i++) {
    double sacc = 0;
    for (int k = 0; k < D; k++) sacc += to.Finv[i][k] * f[k];
    x00[i] = sacc;
  }
  double x0[3] = {x00[0], x00[1], x00[2]};
  const double eps = 1e-12;
  const int maxit = 15;
  int its = 0;
  double diffn = 0;
  while (its == 0 || (diffn > eps * h && its < maxit)) {
    double xt[3], Ft[3][3];
    deformed_map(to, tht, x0, xt, Ft);
    const Geo gt = as_geo(D, Ft);
    double diff[3] = {0, 0, 0};
    for (int i = 0; i < D; i++) diff[i] = vec[i] - xt[i];
    diffn = 0;
    for (int i = 0; i < D; i++) diffn += diff[i] * diff[i];
    diffn = std::sqrt(diffn);
    for (int i = 0; i < D; i++) {
      double sacc = 0;
      for (int k = 0; k < D; k++) sacc += gt.Finv[i][k] * diff[k];
      x0[i] += sacc;
    }
    its++;
  }
  double dist = 0;
  for (int i = 0; i < D; i++) dist += (x0[i] - x00[i]) * (x0[i] - x00[i]);
  dist = std::sqrt(dist);
  const bool fail = its >= maxit || diffn > eps * h || dist > 10.0;
  for (int i = 0; i < 3; i++) xi_to[i] = fail ? x00[i] : x0[i];
  return std::fabs(det_from);
}

// the patch terms of facet f on the deformed mesh (theta [ne][6][3]): both
// elements' order-2k rules, each point mapped into the other element, weight
// w |det (J A)| of its own element, coefficient with the first element's h
int patch_matrix_def(const orc_space* s, const orc_term* terms, int nterms, int f, const double* theta,
                     double* elmat) {
  const int D = s->D, n = s->nd, n2 = 2 * n;
  std::fill(elmat, elmat + n2 * n2, 0.0);
  int e1 = s->facet_els[2 * f], e2 = s->facet_els[2 * f + 1];
  if (e1 < 0 || e2 < 0) return -5;
  Geo g1, g2;
  element_geo(s, e1, g1, nullptr, nullptr);
  element_geo(s, e2, g2, nullptr, nullptr);
  const double* th1 = theta + (size_t)e1 * 18;
  const double* th2 = theta + (size_t)e2 * 18;
  const int* gv1 = &s->elv[(size_t)e1 * (D + 1)];
  const int* gv2 = &s->elv[(size_t)e2 * (D + 1)];
  for (int t = 0; t < nterms; t++) {
    const orc_term& T = terms[t];
    if (T.kind != ORC_TERM_GHOST_MASS) continue;
    if (T.defined_on && !test_bit(T.defined_on, f)) continue;
    const int order = T.order >= 0 ? T.order : 2 * s->k;
    const Rule& r = get_rule(D, order);
    const int nq = r.size();
    const double c = hcoef(T, g1);
    double phi1[20], phi2[20], dphi[20][3], sh[40];
    for (int l = 0; l < 2 * nq; l++) {
      const int m = l < nq ? l : l - nq;
      double xi[3] = {r.p[3 * m], r.p[3 * m + 1], r.p[3 * m + 2]}, xo[3];
      double W;
      if (l < nq) {
        W = r.w[m] * map_patch_point_def(g1, th1, g2, th2, xi, xo);
        basis(D, s->k, gv1, xi, phi1, dphi);
        basis(D, s->k, gv2, xo, phi2, dphi);
      } else {
        W = r.w[m] * map_patch_point_def(g2, th2, g1, th1, xi, xo);
        basis(D, s->k, gv1, xo, phi1, dphi);
        basis(D, s->k, gv2, xi, phi2, dphi);
      }
      for (int i = 0; i < n; i++) {
        sh[i] = phi1[i];
        sh[n + i] = -phi2[i];
      }
      W *= c;
      for (int i = 0; i < n2; i++)
        for (int j = 0; j < n2; j++) elmat[i * n2 + j] += W * sh[i] * sh[j];
    }
  }
  return 0;
}

int facet_matrix(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms, int f, int dn_fd,
                 double* elmat, const double* theta = nullptr) {
  const int r = theta ? patch_matrix_def(s, terms, nterms, f, theta, elmat) : patch_matrix(s, terms, nterms, f, elmat);
  if (r) return r;
  return skel_add(s, lset_vertex, terms, nterms, f, dn_fd, elmat);
}

}  // namespace

struct orc_csr {
  std::vector<int64_t> rowptr;
  std::vector<int32_t> cols;
  std::vector<double> vals;
};

// Row-wise gather of element and facet-patch matrices into CSR over all dofs:
// per dof, its adjacent elements ascending, each element's own row then its
// active facets in local order (first element's columns, then the second's).
orc_csr* gather_csr(int64_t ndof, int n, const std::vector<int32_t>& el_dofs, const std::vector<int64_t>& adj_ptr,
                    const std::vector<int32_t>& adj, int nfl, const std::vector<int32_t>& el_facets,
                    const std::vector<int32_t>& facet_els, const std::vector<int32_t>& el_slot,
                    const std::vector<double>& elm, const std::vector<int32_t>& fa_slot, const std::vector<double>& fam,
                    int nthreads) {
  const int n2 = 2 * n;
  auto* csr = new orc_csr();
  csr->rowptr.assign(ndof + 1, 0);
  std::vector<std::vector<int32_t>> rc(ndof);
  std::vector<std::vector<double>> rv(ndof);
  parallel_for(ndof, nthreads, [&](int64_t b, int64_t en) {
    std::vector<std::pair<int32_t, double>> cand;
    for (int64_t r = b; r < en; r++) {
      cand.clear();
      for (int64_t a = adj_ptr[r]; a < adj_ptr[r + 1]; a++) {
        int e = adj[a] >> 5, i = adj[a] & 31;
        const int32_t* de = &el_dofs[(size_t)e * n];
        if (el_slot[e] >= 0) {
          const double* m = &elm[(size_t)el_slot[e] * n * n];
          for (int j = 0; j < n; j++) cand.push_back({de[j], m[i * n + j]});
        }
        for (int lf = 0; lf < nfl; lf++) {
          int f = el_facets[(size_t)e * nfl + lf];
          if (fa_slot[f] < 0) continue;
          int e1 = facet_els[2 * f], e2 = facet_els[2 * f + 1];
          int row = (e == e1) ? i : n + i;
          const double* m = &fam[(size_t)fa_slot[f] * n2 * n2];
          const int32_t* d1 = &el_dofs[(size_t)e1 * n];
          const int32_t* d2 = &el_dofs[(size_t)e2 * n];
          for (int j = 0; j < n; j++) cand.push_back({d1[j], m[row * n2 + j]});
          for (int j = 0; j < n; j++) cand.push_back({d2[j], m[row * n2 + n + j]});
        }
      }
      std::stable_sort(cand.begin(), cand.end(),
                       [](const std::pair<int32_t, double>& x, const std::pair<int32_t, double>& y) { return x.first < y.first; });
      for (size_t c = 0; c < cand.size();) {
        size_t d = c;
        double sacc = 0;
        while (d < cand.size() && cand[d].first == cand[c].first) sacc += cand[d++].second;
        rc[r].push_back(cand[c].first);
        rv[r].push_back(sacc);
        c = d;
      }
    }
  });
  for (int64_t r = 0; r < ndof; r++) csr->rowptr[r + 1] = csr->rowptr[r] + (int64_t)rc[r].size();
  csr->cols.resize(csr->rowptr[ndof]);
  csr->vals.resize(csr->rowptr[ndof]);
  for (int64_t r = 0; r < ndof; r++) {
    std::copy(rc[r].begin(), rc[r].end(), csr->cols.begin() + csr->rowptr[r]);
    std::copy(rv[r].begin(), rv[r].end(), csr->vals.begin() + csr->rowptr[r]);
  }
  return csr;
}

extern "C" {

int orc_cutinfo(const orc_space* s, const double* lset_vertex, uint8_t* dom, double* cut_ratio, uint64_t* bits,
                int nthreads) {
  const int ne = s->ne, D = s->D;
  const int64_t nw = (ne + 63) / 64;
  std::vector<uint8_t> d8(ne);
  std::atomic<int> err(0);
  parallel_for(ne, nthreads, [&](int64_t b, int64_t en) {
    std::vector<double> pts, wts;
    for (int64_t e = b; e < en; e++) {
      Geo g;
      double l[4];
      element_geo(s, (int)e, g, l, lset_vertex);
      double part_vol[2] = {0.0, 0.0};
      for (int np : {POS, NEG}) {
        int n = straight_cut_rule(g, l, np, 0, pts, wts);
        if (n < -1) err = n;
        if (n > 0)
          for (int q = 0; q < n; q++) part_vol[np] += wts[q];
      }
      cut_ratio[e] = part_vol[NEG] / (part_vol[NEG] + part_vol[POS]);
      uint8_t t;
      if (part_vol[NEG] > 0.0) t = (part_vol[POS] > 0.0) ? IF : NEG;
      else t = POS;
      d8[e] = t;
      dom[e] = t;
    }
  });
  std::memset(bits, 0, sizeof(uint64_t) * nw * 8);
  for (int e = 0; e < ne; e++) {
    int cdt = d8[e] == NEG ? 1 : (d8[e] == POS ? 2 : 4);
    for (int c = 0; c < 8; c++)
      if ((c & cdt) || c == 7) bits[c * nw + (e >> 6)] |= (uint64_t)1 << (e & 63);
  }
  (void)D;
  return err.load();
}

// Boundary elements (NGSolve's BND elements): the boundary facets in facet order,
// each with its vertices in ascending global order.
int orc_boundary_elements(const orc_space* s, int32_t* facets, int32_t* verts) {
  const int D = s->D;
  int n = 0;
  for (int64_t f = 0; f < s->nfacets; f++) {
    if (s->facet_els[2 * f + 1] >= 0) continue;
    if (facets) facets[n] = (int32_t)f;
    if (verts) {
      const int e = s->facet_els[2 * f];
      int lf = 0;
      while (s->el_facets[(size_t)e * (D + 1) + lf] != f) lf++;
      int v[3];
      for (int q = 0; q < D; q++)
        v[q] = s->elv[(size_t)e * (D + 1) + (D == 2 ? TRI_EDGES[lf][q] : TET_FACES[lf][q])];
      std::sort(v, v + D);
      for (int q = 0; q < D; q++) verts[(size_t)n * D + q] = v[q];
    }
    n++;
  }
  return n;
}

// CutInformation::Update for BND elements (xfem/cutinfo.cpp:83-131, vb == BND):
// order-0 cut rules of the (D-1)-simplex with its vertices in ascending order.
int orc_cutinfo_bnd(const orc_space* s, const double* lset_vertex, uint8_t* dom, double* cut_ratio,
                    uint64_t* bits) {
  const int D = s->D, SD = D - 1;
  const int nb = orc_boundary_elements(s, nullptr, nullptr);
  std::vector<int32_t> verts((size_t)nb * D);
  orc_boundary_elements(s, nullptr, verts.data());
  const int64_t nw = (nb + 63) / 64;
  std::memset(bits, 0, sizeof(uint64_t) * nw * 8);
  double ref[12] = {0};
  for (int i = 0; i < SD; i++) ref[i * SD + i] = 1.0;  // reference vertices e_i, then the origin
  Geo g;
  make_geo(SD, ref, g);
  std::vector<double> pts, wts;
  int err = 0;
  for (int e = 0; e < nb; e++) {
    double l[4];
    for (int i = 0; i <= SD; i++) l[i] = lset_vertex[verts[(size_t)e * D + i]];
    double part_vol[2] = {0.0, 0.0};
    for (int np : {POS, NEG}) {
      int n = straight_cut_rule(g, l, np, 0, pts, wts);
      if (n < -1) err = n;
      if (n > 0)
        for (int q = 0; q < n; q++) part_vol[np] += wts[q];
    }
    cut_ratio[e] = part_vol[NEG] / (part_vol[NEG] + part_vol[POS]);
    uint8_t t;
    if (part_vol[NEG] > 0.0) t = (part_vol[POS] > 0.0) ? IF : NEG;
    else t = POS;
    dom[e] = t;
    int cdt = t == NEG ? 1 : (t == POS ? 2 : 4);
    for (int c = 0; c < 8; c++)
      if ((c & cdt) || c == 7) bits[c * nw + (e >> 6)] |= (uint64_t)1 << (e & 63);
  }
  return err;
}

// CutInformation::Update, node part (xfem/cutinfo.cpp:134-224): nodes of IF
// elements (vertices, edges, faces, elements) and the domain of every node:
// NEG if it belongs to a NEG element, else POS; elements (cells) by cut ratio > 0.5.
int orc_cutinfo_nodes(const orc_space* s, const uint8_t* dom, const double* cut_ratio, uint64_t* nb_v,
                      uint64_t* nb_e, uint64_t* nb_f, uint64_t* nb_el, uint8_t* dv, uint8_t* de, uint8_t* df,
                      uint8_t* dc) {
  const int D = s->D, ne = s->ne;
  const int nle = D == 2 ? 3 : 6;
  auto setb = [](uint64_t* b, int64_t i) { b[i >> 6] |= (uint64_t)1 << (i & 63); };
  std::memset(nb_v, 0, sizeof(uint64_t) * ((s->nv + 63) / 64));
  std::memset(nb_e, 0, sizeof(uint64_t) * ((s->nedges + 63) / 64));
  if (D == 3) std::memset(nb_f, 0, sizeof(uint64_t) * ((s->nfaces + 63) / 64));
  std::memset(nb_el, 0, sizeof(uint64_t) * ((ne + 63) / 64));
  for (int i = 0; i < s->nv; i++) dv[i] = POS;
  for (int64_t i = 0; i < s->nedges; i++) de[i] = POS;
  if (D == 3)
    for (int64_t i = 0; i < s->nfaces; i++) df[i] = POS;
  for (int e = 0; e < ne; e++) {
    if (dom[e] == IF) {
      for (int i = 0; i <= D; i++) setb(nb_v, s->elv[(size_t)e * (D + 1) + i]);
      for (int j = 0; j < nle; j++) setb(nb_e, s->el_edges[(size_t)e * nle + j]);
      if (D == 3)
        for (int j = 0; j < 4; j++) setb(nb_f, s->el_faces[(size_t)e * 4 + j]);
      setb(nb_el, e);
    } else if (dom[e] == NEG) {
      for (int i = 0; i <= D; i++) dv[s->elv[(size_t)e * (D + 1) + i]] = NEG;
      for (int j = 0; j < nle; j++) de[s->el_edges[(size_t)e * nle + j]] = NEG;
      if (D == 3)
        for (int j = 0; j < 4; j++) df[s->el_faces[(size_t)e * 4 + j]] = NEG;
    }
    dc[e] = cut_ratio[e] > 0.5 ? NEG : POS;
  }
  return 0;
}

int orc_facets_with_neighbor_types(const orc_space* s, const uint64_t* a, const uint64_t* b, int bnd_a,
                                   int bnd_b, int use_and, uint64_t* out) {
  const int64_t nf = s->nfacets;
  std::memset(out, 0, sizeof(uint64_t) * ((nf + 63) / 64));
  for (int64_t f = 0; f < nf; f++) {
    int l = s->facet_els[2 * f], r = s->facet_els[2 * f + 1];
    bool a_left = test_bit(a, l), b_left = test_bit(b, l);
    bool a_right = r >= 0 ? test_bit(a, r) : (bool)bnd_a;
    bool b_right = r >= 0 ? test_bit(b, r) : (bool)bnd_b;
    bool set = use_and ? ((a_left && b_right) || (a_right && b_left)) : ((a_left || b_right) || (a_right || b_left));
    if (set) out[f >> 6] |= (uint64_t)1 << (f & 63);
  }
  return 0;
}

// CutIntegral::T_CutIntegrate (cutint/cutintegral.cpp:126-212) for f = x^ex y^ey z^ez.
double orc_integrate(const orc_space* s, const double* lset_vertex, int dt, int order, int ex, int ey, int ez,
                     const uint64_t* defined_on) {
  const int D = s->D;
  double sum = 0;
  std::vector<double> pts, wts;
  for (int e = 0; e < s->ne; e++) {
    if (defined_on && !test_bit(defined_on, e)) continue;
    Geo g;
    double l[4];
    element_geo(s, e, g, l, lset_vertex);
    int n = straight_cut_rule(g, l, dt, order, pts, wts);
    if (n <= 0) continue;
    double meas = std::fabs(g.det);
    for (int q = 0; q < n; q++) {
      double x[3] = {0, 0, 0};
      for (int i = 0; i < D; i++) {
        double sacc = g.x0[i];
        for (int k = 0; k < D; k++) sacc += g.F[i][k] * pts[3 * q + k];
        x[i] = sacc;
      }
      double fv = std::pow(x[0], ex) * std::pow(x[1], ey) * (D == 3 ? std::pow(x[2], ez) : 1.0);
      sum += wts[q] * meas * fv;
    }
  }
  return sum;
}

// Integrate of a polynomial in coefficient fields and x, y, z over the
// straight cut rule: cutint/cutintegral.cpp:126-212 with a CoefficientFunction
// made of GridFunctions, evaluated at the rule's points (the error norms of
// the reference's demos, e.g. (gfu - gfex)^2, (grad gfu - grad gfex)^2).
// Field i has order f_order[i] and element coefficients f_el[i] [ne][nd_i]
// in this oracle's basis; product m is coef[m] x^e3[3m] y^e3[3m+1]
// z^e3[3m+2] F0 F1, F0 the value of field f0[m] (d0[m] = -1) or its
// derivative along x_d0[m], F1 likewise (f = -1: no factor; d0 / d1 NULL:
// values only).
double orc_integrate_fields(const orc_space* s, const double* lset_vertex, int dt, int order, int nf,
                            const int* f_order, const double* const* f_el, int nm, const double* coef,
                            const int* e3, const int* f0, const int* f1, const int* d0, const int* d1,
                            const uint64_t* defined_on, const double* theta_mesh) {
  const int D = s->D;
  double sum = 0;
  std::vector<double> pts, wts;
  double phi[20], dphi[20][3], fv[8][4];
  Geo gref;
  {
    const double ref2[6] = {1, 0, 0, 1, 0, 0}, ref3[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
    make_geo(D, D == 2 ? ref2 : ref3, gref);
  }
  for (int e = 0; e < s->ne; e++) {
    if (defined_on && !test_bit(defined_on, e)) continue;
    Geo g;
    double l[4];
    element_geo(s, e, g, l, lset_vertex);
    // on the deformed mesh: the rule of the reference element, mapped point by point
    const double* th = theta_mesh ? theta_mesh + (size_t)e * 18 : nullptr;
    const int n = straight_cut_rule(th ? gref : g, l, dt, order, pts, wts);
    if (n <= 0) continue;
    const int* gv = &s->elv[(size_t)e * (D + 1)];
    const double meas = std::fabs(g.det);
    for (int q = 0; q < n; q++) {
      const double* xi = &pts[3 * q];
      double y[3] = {xi[0], xi[1], D == 3 ? xi[2] : 0.0}, wq = wts[q] * meas;
      Geo gd = g;  // the map whose inverse takes the gradients (the point's Jacobian when deformed)
      if (th) {
        // y = xi + Theta(xi), A = I + grad Theta (edge shapes lambda_a lambda_b), F = J A
        double lam[4], sl = 0.0, Am[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int k = 0; k < D; k++) {
          lam[k] = xi[k];
          sl += xi[k];
        }
        lam[D] = 1.0 - sl;
        const int E2[3][2] = {{0, 1}, {0, 2}, {1, 2}}, E3[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
        for (int j = 0; j < (D == 2 ? 3 : 6); j++) {
          const int a = D == 2 ? E2[j][0] : E3[j][0], b = D == 2 ? E2[j][1] : E3[j][1];
          const double ph = lam[a] * lam[b];
          double dph[3];
          for (int k = 0; k < D; k++) {
            const double da = a < D ? (a == k ? 1.0 : 0.0) : -1.0, db = b < D ? (b == k ? 1.0 : 0.0) : -1.0;
            dph[k] = da * lam[b] + lam[a] * db;
          }
          for (int r = 0; r < D; r++) {
            y[r] += th[j * 3 + r] * ph;
            for (int k = 0; k < D; k++) Am[r][k] += th[j * 3 + r] * dph[k];
          }
        }
        double elc[12], F[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int r = 0; r < D; r++)
          for (int k = 0; k < D; k++)
            for (int q2 = 0; q2 < D; q2++) F[r][k] += g.F[r][q2] * Am[q2][k];
        for (int v = 0; v <= D; v++)
          for (int r = 0; r < D; r++) elc[v * D + r] = v < D ? F[r][v] : 0.0;
        make_geo(D, elc, gd);
        wq = wts[q] * std::fabs(gd.det);
        if (dt == ORC_IF) {
          double gr[3] = {0, 0, 0}, gp[3];
          for (int k = 0; k < D; k++) gr[k] = l[k] - l[D];
          phys_grad(gd, gr, gp);
          wq *= l2norm3(gp) / l2norm3(gr);
        }
      }
      double x[3] = {0, 0, 0};
      for (int i = 0; i < D; i++) {
        double sacc = g.x0[i];
        for (int k = 0; k < D; k++) sacc += g.F[i][k] * y[k];
        x[i] = sacc;
      }
      for (int i = 0; i < nf && i < 8; i++) {
        const int k = f_order[i], nd = D == 2 ? (k + 1) * (k + 2) / 2 : (k + 1) * (k + 2) * (k + 3) / 6;
        basis(D, k, gv, xi, phi, dphi);
        double v = 0.0, dr[3] = {0, 0, 0}, dp[3];
        for (int a = 0; a < nd; a++) {
          const double c = f_el[i][(size_t)e * nd + a];
          v += c * phi[a];
          for (int r = 0; r < 3; r++) dr[r] += c * dphi[a][r];
        }
        phys_grad(gd, dr, dp);
        fv[i][0] = v;
        for (int r = 0; r < 3; r++) fv[i][1 + r] = dp[r];
      }
      double val = 0.0;
      for (int m = 0; m < nm; m++) {
        double t = coef[m] * std::pow(x[0], e3[3 * m]) * std::pow(x[1], e3[3 * m + 1]) *
                   (D == 3 ? std::pow(x[2], e3[3 * m + 2]) : 1.0);
        if (f0[m] >= 0) t *= fv[f0[m]][d0 ? 1 + d0[m] : 0];
        if (f1[m] >= 0) t *= fv[f1[m]][d1 ? 1 + d1[m] : 0];
        val += t;
      }
      sum += wq * val;
    }
  }
  return sum;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Subdivision cut rules for a higher-order level set (subdivlvl): the
// reference's CutIntegrationRule (cutint/xintegration.cpp:1626-1754) with
// NumericalIntegrationStrategy<ET_TRIG / ET_TET, ET_POINT>::MakeQuadRule
// (:757-1063).  A simplex (reference coordinates) at refinement level L is
// checked on the lattice of its points with spacing 1/2^L (CheckIfCut,
// :620-751; CutIntegrationRule sets no distance threshold, so the check is
// the sign of the level set at every lattice point, >= 0 counting as
// positive).  An uncut simplex gets the plain rule of its domain; a cut one
// is refined into the reference's children (:820-914) down to level 0,
// where the vertex signs decide (Simplex::CheckIfCut, xdecompose.hpp:34-80:
// a side whose share of sum |l| is below 1e-14 does not count) and a cut
// simplex gets the straight-cut rule of its vertex values (CutSimplex::MakeQuad,
// :1084-1550: the region and interface of the linear interpolant).  Every
// rule is built on the physical image of its simplex, so points are physical
// and weights are physical measures; integrals of polynomials equal the
// reference's up to rounding.
// ---------------------------------------------------------------------------
namespace {

// children of the red refinement, as barycentric weights on the parent's
// vertices (xintegration.cpp:826-833, 896-906) and vertex lists (:836-841, 898-906)
const double SUB_TRI_BARY[6][3] = {{0, 0, 1}, {.5, 0, .5}, {1, 0, 0}, {0, .5, .5}, {.5, .5, 0}, {0, 1, 0}};
const int SUB_TRI_KIDS[4][3] = {{0, 1, 3}, {1, 2, 4}, {1, 3, 4}, {3, 4, 5}};
const double SUB_TET_BARY[10][4] = {{0, 0, 0, 1}, {.5, 0, 0, .5}, {1, 0, 0, 0}, {0, .5, 0, .5}, {.5, .5, 0, 0},
                                    {0, 1, 0, 0}, {0, 0, .5, .5}, {.5, 0, .5, 0}, {0, .5, .5, 0}, {0, 0, 1, 0}};
const int SUB_TET_KIDS[8][4] = {{1, 2, 4, 7}, {3, 4, 5, 8}, {6, 7, 8, 9}, {3, 4, 8, 6},
                                {3, 4, 1, 6}, {0, 1, 3, 6}, {8, 6, 1, 7}, {8, 4, 1, 7}};

struct Subdiv {
  int D, k;
  const int* gv;        // the element's vertex ids (orientation of the basis)
  const double* coef;   // the level set's element coefficients (H1 basis of order k)
  Geo g;                // the element map
  int dt, order;
  std::vector<double> P, W;  // physical points (3 per point) and weights
  int err = 0;
};

double subdiv_lset(const Subdiv& S, const double* xi) {
  double phi[20], dphi[20][3];
  basis(S.D, S.k, S.gv, xi, phi, dphi);
  double v = 0.0;
  const int n = ndof_el(S.D, S.k);
  for (int i = 0; i < n; i++) v += S.coef[i] * phi[i];
  return v;
}

// NumericalIntegrationStrategy::CheckIfCut without a distance threshold
int subdiv_lattice(const Subdiv& S, const double (*v)[3], int L) {
  const int D = S.D, np = 1 << L;
  const double dx = 1.0 / np;
  bool pos = false, neg = false;
  int I[3] = {0, 0, 0};
  for (;;) {
    double xi[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) xi[d] = v[0][d];
    for (int j = 0; j < D; j++)
      for (int d = 0; d < D; d++) xi[d] += I[j] * dx * (v[j + 1][d] - v[0][d]);
    if (subdiv_lset(S, xi) >= 0.0) pos = true;
    else neg = true;
    if (pos && neg) return IF;
    // next lattice index (I[0] fastest, sum <= np)
    I[0]++;
    int c = 0;
    while (c < D) {
      int sum = 0;
      for (int i = 0; i < D; i++) sum += I[i];
      if (sum <= np) break;
      if (c == D - 1) return pos ? POS : NEG;
      I[c] = 0;
      I[c + 1]++;
      c++;
    }
  }
}

// Simplex::CheckIfCut on the vertex values
int subdiv_vertex_domain(const double* l, int n) {
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
  if (pos && neg) return IF;
  return pos ? POS : (neg ? NEG : POS);
}

// a rule on the physical image of the reference-coordinate simplex v: the
// plain rule (cut = false) or the straight cut of the vertex values l
void subdiv_fill(Subdiv& S, const double (*v)[3], const double* l, bool cut) {
  const int D = S.D;
  double elc[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i <= D; i++)
    for (int r = 0; r < D; r++) {
      double x = S.g.x0[r];
      for (int c = 0; c < D; c++) x += S.g.F[r][c] * v[i][c];
      elc[i * D + r] = x;
    }
  Geo gs;
  make_geo(D, elc, gs);
  std::vector<double> p, w;
  int n;
  if (cut) {
    // a vertex value of exactly 0 counts as positive (CutSimplex::MakeQuad,
    // :1140-1180: such a vertex is cut against its negative neighbours at the
    // vertex itself): the smallest positive normal double does the same
    double lc[4];
    for (int i = 0; i <= D; i++) lc[i] = l[i] == 0.0 ? 2.2250738585072014e-308 : l[i];
    n = straight_cut_rule(gs, lc, S.dt, S.order, p, w);
    if (n < -1) {
      S.err = n;
      return;
    }
  } else {
    // FillSimplexWithRule (:218-264): point = (1 - sum ip) X0 + sum ip_m X_{m+1},
    // weight = w |det(X1 - X0, ...)|
    Sub sub;
    sub.np = D + 1;
    for (int i = 0; i <= D; i++)
      for (int r = 0; r < 3; r++) sub.p[i].c[r] = r < D ? elc[i * D + r] : 0.0;
    plain_rule(sub, S.order, p, w);
    for (size_t q = 0; q < w.size(); q++) {
      S.P.insert(S.P.end(), &p[3 * q], &p[3 * q] + 3);
      S.W.push_back(w[q]);
    }
    return;
  }
  const double meas = std::fabs(gs.det);
  for (int q = 0; q < n; q++) {
    double x[3] = {0, 0, 0};
    for (int r = 0; r < D; r++) {
      double s = gs.x0[r];
      for (int c = 0; c < D; c++) s += gs.F[r][c] * p[3 * q + c];
      x[r] = s;
    }
    S.P.insert(S.P.end(), x, x + 3);
    S.W.push_back(w[q] * meas);
  }
}

// NumericalIntegrationStrategy::MakeQuadRule on the simplex v at level L
void subdiv_quad(Subdiv& S, const double (*v)[3], int L) {
  const int D = S.D;
  const int dself = subdiv_lattice(S, v, L);
  if (dself != IF) {
    if (dself == S.dt) subdiv_fill(S, v, nullptr, false);
    return;
  }
  if (L > 0) {
    const int nk = D == 2 ? 4 : 8;
    for (int c = 0; c < nk; c++) {
      double w[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int j = 0; j <= D; j++)
        for (int d = 0; d <= D; d++) {
          const double b = D == 2 ? SUB_TRI_BARY[SUB_TRI_KIDS[c][j]][d] : SUB_TET_BARY[SUB_TET_KIDS[c][j]][d];
          for (int r = 0; r < D; r++) w[j][r] += b * v[d][r];
        }
      subdiv_quad(S, w, L - 1);
    }
    return;
  }
  double l[4];
  for (int i = 0; i <= D; i++) l[i] = subdiv_lset(S, v[i]);
  const int dv = subdiv_vertex_domain(l, D + 1);
  if (dv == IF) subdiv_fill(S, v, l, true);
  else if (dv == S.dt) subdiv_fill(S, v, nullptr, false);
}

// the rule of element e for the level set coefficients of the space s (order k)
int subdiv_rule(const orc_space* s, const double* lset_coefs, int e, int dt, int order, int subdivlvl, Subdiv& S) {
  const int D = s->D;
  S.D = D;
  S.k = s->k;
  S.gv = &s->elv[(size_t)e * (D + 1)];
  double c[20];
  for (int i = 0; i < s->nd; i++) c[i] = lset_coefs[s->el_dofs[(size_t)e * s->nd + i]];
  S.coef = c;
  element_geo(s, e, S.g, nullptr, nullptr);
  S.dt = dt;
  S.order = order;
  S.P.clear();
  S.W.clear();
  S.err = 0;
  double v[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // reference vertices (1,0,0),(0,1,0),(0,0,1),(0,0,0)
  for (int i = 0; i < D; i++) v[i][i] = 1.0;
  subdiv_quad(S, v, subdivlvl);
  S.coef = nullptr;
  return S.err;
}

}  // namespace

extern "C" {

double orc_integrate_subdiv(const orc_space* s, const double* lset_coefs, int dt, int order, int subdivlvl, int ex,
                            int ey, int ez, const uint64_t* defined_on, int* status) {
  const int D = s->D;
  double sum = 0.0;
  Subdiv S;
  if (status) *status = 0;
  for (int e = 0; e < s->ne; e++) {
    if (defined_on && !test_bit(defined_on, e)) continue;
    const int st = subdiv_rule(s, lset_coefs, e, dt, order, subdivlvl, S);
    if (st && status) *status = st;
    for (size_t q = 0; q < S.W.size(); q++) {
      const double* x = &S.P[3 * q];
      const double fv = std::pow(x[0], ex) * std::pow(x[1], ey) * (D == 3 ? std::pow(x[2], ez) : 1.0);
      sum += S.W[q] * fv;
    }
  }
  return sum;
}

int orc_subdiv_rule(const orc_space* s, const double* lset_coefs, int e, int dt, int order, int subdivlvl,
                    double* pts, double* wts, int maxpts) {
  Subdiv S;
  const int st = subdiv_rule(s, lset_coefs, e, dt, order, subdivlvl, S);
  if (st) return st;
  const int n = (int)S.W.size();
  if (n > maxpts) return ERR_CAPACITY;
  std::memcpy(pts, S.P.data(), sizeof(double) * 3 * n);
  std::memcpy(wts, S.W.data(), sizeof(double) * n);
  return n;
}

// NEG moments (x^a y^b z^c, a + b + c <= 4; by degree, then a, then b
// descending) of P2 level sets on the reference tetrahedron, given by their
// values at the vertices and edge midpoints (edges (0,1),(0,2),(0,3),(1,2),
// (1,3),(2,3)), by the subdivision rule of the given level, order 4
int orc_subdiv_moments_p2(int64_t n, const double* vals10, int levels, double* out35, int nthreads) {
  const double ref[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
  const int32_t elv[4] = {0, 1, 2, 3};
  orc_space* s = orc_space_create(3, 4, ref, 1, elv, 2);
  std::atomic<int> err(0);
  parallel_for(n, nthreads, [&](int64_t b, int64_t en) {
    Subdiv S;
    std::vector<double> c(s->ndof);
    for (int64_t e = b; e < en; e++) {
      const double* p = vals10 + e * 10;
      for (int i = 0; i < 4; i++) c[s->el_dofs[i]] = p[i];
      for (int j = 0; j < 6; j++)
        c[s->el_dofs[4 + j]] = 4.0 * p[4 + j] - 2.0 * (p[TET_EDGES[j][0]] + p[TET_EDGES[j][1]]);
      const int st = subdiv_rule(s, c.data(), 0, NEG, 4, levels, S);
      if (st) err = st;
      double* m = out35 + e * 35;
      for (int k = 0; k < 35; k++) m[k] = 0.0;
      for (size_t q = 0; q < S.W.size(); q++) {
        const double x = S.P[3 * q], y = S.P[3 * q + 1], z = S.P[3 * q + 2];
        const double px[5] = {1, x, x * x, x * x * x, x * x * x * x};
        const double py[5] = {1, y, y * y, y * y * y, y * y * y * y};
        const double pz[5] = {1, z, z * z, z * z * z, z * z * z * z};
        int k = 0;
        for (int t = 0; t <= 4; t++)
          for (int a = t; a >= 0; a--)
            for (int bb = t - a; bb >= 0; bb--) m[k++] += S.W[q] * px[a] * py[bb] * pz[t - a - bb];
      }
    }
  });
  orc_space_destroy(s);
  return err.load();
}

int orc_element_matrix(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms, int e,
                       double* elmat) {
  return element_matrix(s, lset_vertex, terms, nterms, e, elmat);
}

int orc_patch_matrix(const orc_space* s, const orc_term* terms, int nterms, int f, double* elmat) {
  return patch_matrix(s, terms, nterms, f, elmat);
}

int orc_facet_matrix(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms, int f,
                     int dn_fd, double* elmat) {
  return facet_matrix(s, lset_vertex, terms, nterms, f, dn_fd, elmat);
}

int orc_fd_stencil(int k, int acc, double* c, double* eps) { return fd_stencil(k, acc, c, eps); }

// CSR over ndof dofs from element matrices alone (no facets): el_dofs
// [ne][n], el_slot[e] the element's matrix in elm or -1; per dof its
// elements ascending (the gather of gather_csr).
orc_csr* orc_csr_from_elements(int64_t ndof, int n, int ne, const int32_t* el_dofs, const int32_t* el_slot,
                               const double* elm, int64_t nslots, int nthreads) {
  std::vector<int32_t> dofs(el_dofs, el_dofs + (size_t)ne * n), slot(el_slot, el_slot + ne);
  std::vector<int64_t> ptr(ndof + 1, 0);
  for (int32_t d : dofs) ptr[d + 1]++;
  for (int64_t r = 0; r < ndof; r++) ptr[r + 1] += ptr[r];
  std::vector<int32_t> adj(dofs.size());
  std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
  for (int e = 0; e < ne; e++)
    for (int i = 0; i < n; i++) adj[fill[dofs[(size_t)e * n + i]]++] = e * 32 + i;
  std::vector<double> m(elm, elm + (size_t)nslots * n * n), none;
  std::vector<int32_t> nof;
  return gather_csr(ndof, n, dofs, ptr, adj, 0, nof, nof, slot, m, nof, none, nthreads);
}

orc_csr* orc_assemble(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms,
                      int nthreads) {
  return orc_assemble_bnd(s, lset_vertex, terms, nterms, nullptr, 0, nthreads, 0);
}

// Bilinear forms on regions of several level sets: SymbolicCutBFI with a
// multi-level-set LevelsetIntegrationDomain (symboliccutbfi.cpp:76-486 with
// CreateMultiLevelsetCutIntegrationRule, cutint/mlsetintegration.cpp:6-180):
// per active element and term the rule of the term's region
// (orc_mlset_cut_rule) and the term's integrand at its points; the patch
// terms as in orc_assemble; summed into a CSR over all dofs.
orc_csr* orc_mlset_assemble(const orc_space* s, int M, const double* lsets, const orc_mlterm* terms, int nterms,
                            const orc_term* patch_terms, int npatch, int nthreads) {
  const int ne = s->ne, n = s->nd, n2 = 2 * n, D = s->D;
  const int64_t nf = s->nfacets, nv = s->nv;
  std::vector<int32_t> el_slot(ne, -1), fa_slot(nf, -1);
  int nact = 0;
  for (int e = 0; e < ne; e++) {
    bool act = false;
    for (int t = 0; t < nterms; t++)
      if (!terms[t].defined_on || test_bit(terms[t].defined_on, e)) act = true;
    if (act) el_slot[e] = nact++;
  }
  int nfa = 0;
  for (int64_t f = 0; f < nf && npatch > 0; f++) {
    if (s->facet_els[2 * f + 1] < 0) continue;
    bool act = false;
    for (int t = 0; t < npatch; t++)
      if (!patch_terms[t].defined_on || test_bit(patch_terms[t].defined_on, f)) act = true;
    if (act) fa_slot[f] = nfa++;
  }
  std::vector<int32_t> el_list(nact), fa_list(nfa);
  for (int e = 0; e < ne; e++) if (el_slot[e] >= 0) el_list[el_slot[e]] = e;
  for (int64_t f = 0; f < nf; f++) if (fa_slot[f] >= 0) fa_list[fa_slot[f]] = (int32_t)f;
  std::vector<double> elm((size_t)nact * n * n, 0.0), fam((size_t)nfa * n2 * n2);
  std::atomic<int> err(0);
  parallel_for(nact, nthreads, [&](int64_t b, int64_t en) {
    std::vector<double> pts(3 * 20000), wts(20000);
    double elc[12], lv[8 * 4], phi[20], dphi[20][3], gp[20][3];
    for (int64_t i = b; i < en; i++) {
      const int e = el_list[i];
      Geo g;
      element_geo(s, e, g, nullptr, nullptr);
      for (int v = 0; v <= D; v++) {
        const int vid = s->elv[(size_t)e * (D + 1) + v];
        for (int c = 0; c < D; c++) elc[v * D + c] = s->coords[(size_t)vid * D + c];
        for (int m = 0; m < M; m++) lv[m * (D + 1) + v] = lsets[(size_t)m * nv + vid];
      }
      const int* gv = &s->elv[(size_t)e * (D + 1)];
      const double meas = std::fabs(g.det);
      double* A = &elm[(size_t)i * n * n];
      for (int t = 0; t < nterms; t++) {
        const orc_mlterm& T = terms[t];
        if (T.defined_on && !test_bit(T.defined_on, e)) continue;
        const int order = T.order >= 0 ? T.order : default_order(T.kind, s->k);
        const int np = orc_mlset_cut_rule(D, elc, M, lv, T.ntup, T.dts, order, pts.data(), wts.data(), 20000);
        if (np < -1) { err = np; continue; }
        if (np <= 0) continue;
        double c = T.coef;
        if (T.hpow != 0) c *= std::pow(meas, (double)T.hpow / D);
        // unit normal of the P1 level set T.normal_lset
        double nrm[3] = {0, 0, 0};
        if (T.kind == ORC_TERM_NGRADU_V || T.kind == ORC_TERM_U_NGRADV) {
          double gr[3] = {0, 0, 0}, gl[3];
          const double* l = &lv[T.normal_lset * (D + 1)];
          for (int k = 0; k < D; k++) gr[k] = l[k] - l[D];
          phys_grad(g, gr, gl);
          const double nn = l2norm3(gl);
          for (int k = 0; k < 3; k++) nrm[k] = gl[k] / nn;
        }
        for (int q = 0; q < np; q++) {
          basis(D, s->k, gv, &pts[3 * q], phi, dphi);
          for (int a = 0; a < n; a++) phys_grad(g, dphi[a], gp[a]);
          const double W = wts[q] * meas * c;
          for (int a = 0; a < n; a++)      // test
            for (int bb = 0; bb < n; bb++) {  // trial
              double v;
              switch (T.kind) {
                case ORC_TERM_MASS: v = phi[a] * phi[bb]; break;
                case ORC_TERM_LAPLACE: v = gp[a][0] * gp[bb][0] + gp[a][1] * gp[bb][1] + gp[a][2] * gp[bb][2]; break;
                case ORC_TERM_NGRADU_V: v = (nrm[0] * gp[bb][0] + nrm[1] * gp[bb][1] + nrm[2] * gp[bb][2]) * phi[a]; break;
                case ORC_TERM_U_NGRADV: v = phi[bb] * (nrm[0] * gp[a][0] + nrm[1] * gp[a][1] + nrm[2] * gp[a][2]); break;
                case ORC_TERM_CONV: v = (T.b[0] * gp[bb][0] + T.b[1] * gp[bb][1] + T.b[2] * gp[bb][2]) * phi[a]; break;
                default: v = 0.0;
              }
              A[a * n + bb] += W * v;
            }
        }
      }
    }
  });
  parallel_for(nfa, nthreads, [&](int64_t b, int64_t en) {
    for (int64_t i = b; i < en; i++) {
      const int r = patch_matrix(s, patch_terms, npatch, fa_list[i], &fam[(size_t)i * n2 * n2]);
      if (r) err = r;
    }
  });
  if (err.load()) return nullptr;
  return gather_csr(s->ndof, n, s->el_dofs, s->dof_adj_ptr, s->dof_adj, s->D + 1, s->el_facets, s->facet_els,
                    el_slot, elm, fa_slot, fam, nthreads);
}

orc_csr* orc_assemble_ex(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms,
                         int nthreads, int dn_fd) {
  return orc_assemble_bnd(s, lset_vertex, terms, nterms, nullptr, 0, nthreads, dn_fd);
}

// orc_assemble with boundary terms: SymbolicCutBFI with vb == BND
// (symboliccutbfi.cpp:76-486 on a boundary element, the rule of
// straightcutrule.cpp:582-677 on the boundary facet): per BND element (the
// boundary facets in facet order) in a term's set, the term's integrand with
// the owning element's basis at the boundary rule's physical points, added
// to the owner's element matrix; the owners join the active elements.
orc_csr* orc_assemble_bnd(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms,
                          const orc_bterm* bterms, int nbterms, int nthreads, int dn_fd) {
  return orc_assemble_full(s, lset_vertex, terms, nterms, bterms, nbterms, nullptr, 0, nullptr, nthreads, dn_fd);
}

// ... and volume terms with a coefficient field (element_matrix_coef), whose
// element sets join the active elements
orc_csr* orc_assemble_full(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms,
                           const orc_bterm* bterms, int nbterms, const orc_cterm* cterms, int ncterms,
                           const double* theta_patch, int nthreads, int dn_fd) {
  const int ne = s->ne, n = s->nd, n2 = 2 * n;
  const int64_t nf = s->nfacets;
  // active elements: in the definedon set of some volume term; active facets:
  // interior facets in the definedon set of some patch or skeleton term
  auto facet_term = [](int kind) { return kind == ORC_TERM_GHOST_MASS || kind >= ORC_TERM_SKEL_JUMP; };
  std::vector<int32_t> el_slot(ne, -1), fa_slot(nf, -1);
  bool any_vol = false, any_patch = false;
  for (int t = 0; t < nterms; t++) (facet_term(terms[t].kind) ? any_patch : any_vol) = true;
  // BND elements (boundary facets in facet order) and their owners
  std::vector<int32_t> bfac, bown;
  std::vector<uint8_t> bnd_act(ne, 0);
  if (nbterms > 0) {
    for (int64_t f = 0; f < nf; f++)
      if (s->facet_els[2 * f + 1] < 0) {
        const int b = (int)bfac.size();
        bfac.push_back((int32_t)f);
        bown.push_back(s->facet_els[2 * f]);
        // the BND element's domain type (CheckIfStraightCut of its vertex values)
        const int e0 = s->facet_els[2 * f], D = s->D;
        int lf = 0;
        while (s->el_facets[(size_t)e0 * (D + 1) + lf] != f) lf++;
        bool hp = false, hn = false;
        for (int q = 0; q < D; q++) {
          const int vq = s->elv[(size_t)e0 * (D + 1) + (D == 2 ? TRI_EDGES[lf][q] : TET_FACES[lf][q])];
          hp |= lset_vertex[vq] > 0.0;
          hn |= lset_vertex[vq] < 0.0;
        }
        const int dom = (hp && hn) || (!hp && !hn) ? ORC_IF : (hn ? ORC_NEG : ORC_POS);
        for (int t = 0; t < nbterms; t++)
          if ((!bterms[t].defined_on || test_bit(bterms[t].defined_on, b)) &&
              (dom == ORC_IF || dom == bterms[t].domain))
            bnd_act[e0] = 1;
      }
  }
  // an element is active for a volume term in whose set it lies if its
  // domain type (CheckIfStraightCut of its vertex values) is the term's
  // domain or IF: elements without a part in the term's domain add nothing
  int nact = 0;
  for (int e = 0; e < ne; e++) {
    bool act = bnd_act[e] != 0;
    double le[4];
    for (int i = 0; i <= s->D; i++) le[i] = lset_vertex[s->elv[(size_t)e * (s->D + 1) + i]];
    const int dom = check_if_straight_cut(le, s->D + 1);
    for (int t = 0; t < nterms && any_vol; t++)
      if (!facet_term(terms[t].kind) && (!terms[t].defined_on || test_bit(terms[t].defined_on, e)) &&
          (dom == ORC_IF || dom == terms[t].domain))
        act = true;
    for (int t = 0; t < ncterms; t++)
      if ((!cterms[t].defined_on || test_bit(cterms[t].defined_on, e)) &&
          (dom == ORC_IF || dom == cterms[t].domain || cterms[t].domain == ORC_WHOLE))
        act = true;
    if (act) el_slot[e] = nact++;
  }
  int nfa = 0;
  for (int64_t f = 0; f < nf && any_patch; f++) {
    if (s->facet_els[2 * f + 1] < 0) continue;
    bool act = false;
    for (int t = 0; t < nterms; t++)
      if (facet_term(terms[t].kind) && (!terms[t].defined_on || test_bit(terms[t].defined_on, f))) act = true;
    if (act) fa_slot[f] = nfa++;
  }
  std::vector<int32_t> el_list(nact), fa_list(nfa);
  for (int e = 0; e < ne; e++) if (el_slot[e] >= 0) el_list[el_slot[e]] = e;
  for (int64_t f = 0; f < nf; f++) if (fa_slot[f] >= 0) fa_list[fa_slot[f]] = (int32_t)f;
  std::vector<double> elm((size_t)nact * n * n), fam((size_t)nfa * n2 * n2);
  std::atomic<int> err(0);
  parallel_for(nact, nthreads, [&](int64_t b, int64_t en) {
    for (int64_t i = b; i < en; i++) {
      int r = element_matrix(s, lset_vertex, terms, nterms, el_list[i], &elm[(size_t)i * n * n]);
      if (!r && ncterms > 0)
        r = element_matrix_coef(s, lset_vertex, cterms, ncterms, el_list[i], &elm[(size_t)i * n * n]);
      if (r) err = r;
    }
  });
  // boundary terms, BND elements ascending
  for (size_t bi = 0; bi < bfac.size(); bi++) {
    const int e = bown[bi], f = bfac[bi], D = s->D;
    double* A = &elm[(size_t)el_slot[e] * n * n];
    Geo g;
    element_geo(s, e, g, nullptr, nullptr);
    const int* gv = &s->elv[(size_t)e * (D + 1)];
    int lf = 0;
    while (s->el_facets[(size_t)e * (D + 1) + lf] != f) lf++;
    int v[3];
    for (int q = 0; q < D; q++) v[q] = gv[D == 2 ? TRI_EDGES[lf][q] : TET_FACES[lf][q]];
    std::sort(v, v + D);
    double xb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, lb[3];
    for (int q = 0; q < D; q++) {
      lb[q] = lset_vertex[v[q]];
      for (int r = 0; r < D; r++) xb[3 * q + r] = s->coords[(size_t)v[q] * D + r];
    }
    double xs[3 * 512], ws[512], phi[20], dphi[20][3];
    for (int t = 0; t < nbterms; t++) {
      const orc_bterm& T = bterms[t];
      if (T.defined_on && !test_bit(T.defined_on, (int64_t)bi)) continue;
      const int order = T.order >= 0 ? T.order : 2 * s->k;
      const int np = orc_bnd_element_rule(D, xb, lb, T.domain, order, xs, ws, 512);
      if (np < 0) {
        err = np == -1 ? ERR_CAPACITY : np;
        continue;
      }
      double c = T.coef;
      if (T.hpow != 0) c *= std::pow(std::pow(std::fabs(g.det), 1.0 / D), (double)T.hpow);
      for (int q = 0; q < np; q++) {
        const double* x = &xs[3 * q];
        double xi[3] = {0, 0, 0};
        for (int k = 0; k < D; k++) {
          double acc = 0.0;
          for (int cc = 0; cc < D; cc++) acc += g.Finv[k][cc] * (x[cc] - g.x0[cc]);
          xi[k] = acc;
        }
        basis(D, s->k, gv, xi, phi, dphi);
        const double w = ws[q] * c;
        for (int a = 0; a < n; a++)
          for (int bb = 0; bb < n; bb++) A[a * n + bb] += w * phi[a] * phi[bb];
      }
    }
  }
  parallel_for(nfa, nthreads, [&](int64_t b, int64_t en) {
    for (int64_t i = b; i < en; i++) {
      int r = facet_matrix(s, lset_vertex, terms, nterms, fa_list[i], dn_fd, &fam[(size_t)i * n2 * n2], theta_patch);
      if (r) err = r;
    }
  });
  if (err.load()) return nullptr;
  return gather_csr(s->ndof, n, s->el_dofs, s->dof_adj_ptr, s->dof_adj, s->D + 1, s->el_facets, s->facet_els,
                    el_slot, elm, fa_slot, fam, nthreads);
}

int64_t orc_csr_nnz(const orc_csr* c) { return c->rowptr.back(); }
void orc_csr_get(const orc_csr* c, int64_t* rowptr, int32_t* cols, double* vals) {
  std::memcpy(rowptr, c->rowptr.data(), sizeof(int64_t) * c->rowptr.size());
  std::memcpy(cols, c->cols.data(), sizeof(int32_t) * c->cols.size());
  std::memcpy(vals, c->vals.data(), sizeof(double) * c->vals.size());
}
void orc_csr_destroy(orc_csr* c) { delete c; }

// CutFEM pipeline as in demos/fictdom.py:95-133: CutInfo -> HASNEG / IF element
// sets -> ghost facets (HASNEG, IF) -> assembly.  Volume terms on NEG get the
// HASNEG set, IF terms the IF set, POS terms the HASPOS set; patch terms get the
// ghost facets.  Skeleton terms (demos/fictdom_dg.py:100-135): on NEG the
// facets between two HASNEG elements, on POS between two HASPOS elements, on
// whole facets the ghost facets.
int64_t orc_pipeline(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms,
                     int ghost_facets, int nthreads) {
  const int ne = s->ne;
  const int64_t nw = (ne + 63) / 64, nfw = (s->nfacets + 63) / 64;
  std::vector<uint8_t> dom(ne);
  std::vector<double> ratio(ne);
  std::vector<uint64_t> bits(8 * nw), fb(nfw);
  if (orc_cutinfo(s, lset_vertex, dom.data(), ratio.data(), bits.data(), nthreads)) return -1;
  const uint64_t* hasneg = &bits[5 * nw];
  const uint64_t* ifb = &bits[4 * nw];
  const uint64_t* haspos = &bits[6 * nw];
  if (ghost_facets) orc_facets_with_neighbor_types(s, hasneg, ifb, 1, 1, 1, fb.data());
  std::vector<uint64_t> fneg(nfw), fpos(nfw);
  orc_facets_with_neighbor_types(s, hasneg, hasneg, 1, 1, 1, fneg.data());
  orc_facets_with_neighbor_types(s, haspos, haspos, 1, 1, 1, fpos.data());
  std::vector<orc_term> t2(terms, terms + nterms);
  for (auto& t : t2) {
    if (t.kind == ORC_TERM_GHOST_MASS) t.defined_on = fb.data();
    else if (t.kind >= ORC_TERM_SKEL_JUMP)
      t.defined_on = t.domain == ORC_NEG ? fneg.data() : (t.domain == ORC_POS ? fpos.data() : fb.data());
    else t.defined_on = t.domain == ORC_NEG ? hasneg : (t.domain == ORC_IF ? ifb : haspos);
  }
  orc_csr* c = orc_assemble(s, lset_vertex, t2.data(), nterms, nthreads);
  if (!c) return -2;
  int64_t nnz = orc_csr_nnz(c);
  orc_csr_destroy(c);
  return nnz;
}

}  // extern "C"

// ===========================================================================
// Space-time: cutint/spacetimecutrule.cpp:8-244 (root_finding,
// SpaceTimeCutIntegrationRule), time basis of spacetime/SpaceTimeFE.cpp:263-281
// (nodal on Gauss-Lobatto points), space-time element and facet-patch
// matrices (T_CalcFacetMatrix with time_order >= 0, symboliccutbfi.cpp:2095-2160).
// ===========================================================================
namespace {

// kt = 0 constant; kt = 1 nodes {0, 1}; kt = 2 nodes {0, 1/2, 1}
void time_basis(int kt, double x, double* psi, double* dpsi) {
  if (kt == 0) { psi[0] = 1.0; dpsi[0] = 0.0; return; }
  if (kt == 1) { psi[0] = 1.0 - x; psi[1] = x; dpsi[0] = -1.0; dpsi[1] = 1.0; return; }
  psi[0] = (1 - x) * (1 - 2 * x);
  psi[1] = 4 * x * (1 - x);
  psi[2] = x * (2 * x - 1);
  dpsi[0] = 4 * x - 3;
  dpsi[1] = 4 - 8 * x;
  dpsi[2] = 4 * x - 1;
}

// spacetimecutrule.cpp:8-48 (orders 0..2)
int time_roots(int kt, const double* li, double* roots) {
  if (kt == 0) return 0;
  if (kt == 1) {
    if ((li[0] >= 0) != (li[1] >= 0)) { roots[0] = -li[0] / (li[1] - li[0]); return 1; }
    return 0;
  }
  const double c = li[0], a = 2 * li[0] + 2 * li[2] - 4. * li[1], b = li[2] - a - c;
  int n = 0;
  if (std::fabs(a) < 1e-12) {
    const double x = -c / b;
    if (x < 1 && x > 0) roots[n++] = x;
  } else {
    const double w = b * b - 4 * a * c;
    if (std::fabs(w) < 1e-12) {
      const double x = -b / (2 * a);
      if (x < 1 && x > 0) roots[n++] = x;
    } else {
      const double x1 = (b + std::sqrt(w)) / (-2.0 * a);
      const double x2 = (b - std::sqrt(w)) / (-2.0 * a);
      if (x1 < 1 && x1 > 0) roots[n++] = x1;
      if (x2 < 1 && x2 > 0) roots[n++] = x2;
    }
  }
  return n;
}

// SpaceTimeCutIntegrationRule (spacetimecutrule.cpp:106-244) for simplices.
// lset_st: (kt+1)*(D+1) time-major; pts4: 4 per point (xi, eta, zeta, tau).
int st_cut_rule(const Geo& g, const double* lset_st, int kt, int dt, int order_space, int order_time,
                std::vector<double>& pts4, std::vector<double>& wts) {
  const int D = g.D, nsp = D + 1;
  pts4.clear();
  wts.clear();
  if (kt < 0 || kt > 2) return ERR_BAD_DECOMP;
  std::vector<double> cut = {0.0, 1.0};
  for (int j = 0; j < nsp; j++) {
    double li[3], r[2];
    for (int i = 0; i <= kt; i++) li[i] = lset_st[i * nsp + j];
    int nr = time_roots(kt, li, r);
    cut.insert(cut.begin(), r, r + nr);
  }
  std::sort(cut.begin(), cut.end());
  const Rule& irt = get_rule(1, order_time);
  if (order_space == -1) order_space = 5;
  const Rule& stdir = get_rule(D, order_space);
  const size_t maxsize = (size_t)5 * stdir.size() * (cut.size() - 1) * irt.size();
  std::vector<double> p3, w3;
  for (size_t i = 0; i + 1 < cut.size(); i++) {
    const double t0 = cut[i], t1 = cut[i + 1];
    for (int q = 0; q < irt.size(); q++) {
      const double t = t0 + irt.p[3 * q] * (t1 - t0);
      double psi[3], dpsi[3], cf[4];
      time_basis(kt, t, psi, dpsi);
      for (int j = 0; j < nsp; j++) {
        double s = 0;
        for (int ii = 0; ii <= kt; ii++) s += lset_st[ii * nsp + j] * psi[ii];
        if (std::fabs(s) < 1e-14) s = s >= 0 ? 1e-14 : -1e-14;  // EPS_STCR_LSET_PERTUBATION
        cf[j] = s;
      }
      const int dom = check_if_straight_cut(cf, nsp);
      if (dom == IF) {
        int n = straight_cut_rule(g, cf, dt, order_space, p3, w3);
        if (n < -1) return n;
        for (int k = 0; k < n; k++) {
          pts4.push_back(p3[3 * k]); pts4.push_back(p3[3 * k + 1]); pts4.push_back(p3[3 * k + 2]); pts4.push_back(t);
          wts.push_back(w3[k] * irt.w[q] * (t1 - t0));
        }
      } else if (dom == dt) {
        for (int k = 0; k < stdir.size(); k++) {
          pts4.push_back(stdir.p[3 * k]); pts4.push_back(stdir.p[3 * k + 1]); pts4.push_back(stdir.p[3 * k + 2]);
          pts4.push_back(t);
          wts.push_back(stdir.w[k] * irt.w[q] * (t1 - t0));
        }
      }
    }
  }
  if (wts.size() > maxsize) return ERR_CAPACITY;
  return wts.empty() ? -1 : (int)wts.size();
}

void lset_trace(const double* lset_st, int kt, int nsp, double tau, double* out) {
  double psi[3], dpsi[3];
  time_basis(kt, tau, psi, dpsi);
  for (int j = 0; j < nsp; j++) {
    double s = 0;
    for (int i = 0; i <= kt; i++) s += lset_st[i * nsp + j] * psi[i];
    if (std::fabs(s) < 1e-14) s = 1e-14;  // InterpolateToP1 perturbation of the trace
    out[j] = s;
  }
}

void element_lset_st(const orc_space* s, int e, const double* lset_st, int kt, double* out) {
  const int nsp = s->D + 1;
  for (int i = 0; i <= kt; i++)
    for (int j = 0; j < nsp; j++) out[i * nsp + j] = lset_st[(size_t)i * s->nv + s->elv[(size_t)e * nsp + j]];
}

double st_coef(const orc_st_term& T, const Geo& g) {
  double c = T.coef;
  if (T.hpow != 0) c *= std::pow(std::pow(std::fabs(g.det), 1.0 / g.D), (double)T.hpow);
  return c;
}

int st_default_order(int kind, int k) {
  switch (kind) {
    case ORC_TERM_LAPLACE: return 2 * k - 2;
    case ORC_TERM_CONV: return 2 * k - 1;
    default: return 2 * k;
  }
}

// element matrix (nd*(kt+1))^2 of the space-time volume terms
int st_element_matrix(const orc_space* s, const double* lset_st, int kt_l, int kt, int order_time,
                      const orc_st_term* terms, int nterms, int e, double* elmat) {
  const int D = s->D, nd = s->nd, nt = kt + 1, N = nd * nt, nsp = D + 1;
  Geo g;
  element_geo(s, e, g, nullptr, nullptr);
  const int* gv = &s->elv[(size_t)e * nsp];
  double lst[12];
  element_lset_st(s, e, lset_st, kt_l, lst);
  std::fill(elmat, elmat + (size_t)N * N, 0.0);
  std::vector<double> pts, wts;
  double phi[20], dphi[20][3], gp[20][3], psi[3], dpsi[3];
  std::vector<double> F(N), GX((size_t)N * 3), FT(N);
  for (int t = 0; t < nterms; t++) {
    const orc_st_term& T = terms[t];
    if (T.kind == ORC_TERM_GHOST_MASS) continue;
    if (T.defined_on && !test_bit(T.defined_on, e)) continue;
    const int order = T.order >= 0 ? T.order : st_default_order(T.kind, s->k);
    int np;
    if (T.tref >= 0) {
      double ls[4];
      lset_trace(lst, kt_l, nsp, T.tref, ls);
      std::vector<double> p3, w3;
      np = straight_cut_rule(g, ls, T.domain, order, p3, w3);
      if (np < -1) return np;
      pts.clear();
      wts.clear();
      for (int k = 0; k < np; k++) {
        pts.push_back(p3[3 * k]); pts.push_back(p3[3 * k + 1]); pts.push_back(p3[3 * k + 2]); pts.push_back(T.tref);
        wts.push_back(w3[k]);
      }
    } else {
      np = st_cut_rule(g, lst, kt_l, T.domain, order, order_time, pts, wts);
      if (np < -1) return np;
    }
    if (np <= 0) continue;
    const double c = st_coef(T, g), meas = std::fabs(g.det);
    for (int q = 0; q < np; q++) {
      const double tau = pts[4 * q + 3];
      basis(D, s->k, gv, &pts[4 * q], phi, dphi);
      for (int i = 0; i < nd; i++) phys_grad(g, dphi[i], gp[i]);
      time_basis(kt, tau, psi, dpsi);
      double b[3] = {T.b[0], T.b[1], T.b[2]};
      if (T.kind == ORC_TERM_CONV && T.omega != 0.0) {
        const double tp = T.t0 + T.dt * tau;
        for (int k = 0; k < 3; k++) b[k] += T.bc[k] * std::cos(T.omega * tp) + T.bs[k] * std::sin(T.omega * tp);
      }
      for (int it = 0; it < nt; it++)
        for (int j = 0; j < nd; j++) {
          const int a = it * nd + j;
          F[a] = psi[it] * phi[j];
          FT[a] = dpsi[it] * phi[j];
          for (int k = 0; k < 3; k++) GX[3 * a + k] = psi[it] * gp[j][k];
        }
      const double w = wts[q] * meas * c;
      for (int p = 0; p < N; p++)
        for (int r = 0; r < N; r++) {
          double v;
          switch (T.kind) {
            case ORC_TERM_MASS: v = F[p] * F[r]; break;
            case ORC_TERM_LAPLACE: v = GX[3 * p] * GX[3 * r] + GX[3 * p + 1] * GX[3 * r + 1] + GX[3 * p + 2] * GX[3 * r + 2]; break;
            case ORC_TERM_CONV: v = (b[0] * GX[3 * r] + b[1] * GX[3 * r + 1] + b[2] * GX[3 * r + 2]) * F[p]; break;
            case ORC_TERM_DT_U_V: v = F[p] * FT[r]; break;
            default: v = 0;
          }
          elmat[(size_t)p * N + r] += w * v;
        }
    }
  }
  return 0;
}

// space-time facet patch: spatial patch rule x time rule (symboliccutbfi.cpp:2095-2160)
int st_patch_matrix(const orc_space* s, int kt, int order_time, const orc_st_term* terms, int nterms, int f,
                    double* elmat) {
  const int D = s->D, nd = s->nd, nt = kt + 1, N = nd * nt, N2 = 2 * N;
  std::fill(elmat, elmat + (size_t)N2 * N2, 0.0);
  const int e1 = s->facet_els[2 * f], e2 = s->facet_els[2 * f + 1];
  if (e1 < 0 || e2 < 0) return -5;
  Geo g1, g2;
  element_geo(s, e1, g1, nullptr, nullptr);
  element_geo(s, e2, g2, nullptr, nullptr);
  const int* gv1 = &s->elv[(size_t)e1 * (D + 1)];
  const int* gv2 = &s->elv[(size_t)e2 * (D + 1)];
  const Rule& irt = get_rule(1, order_time);
  for (int t = 0; t < nterms; t++) {
    const orc_st_term& T = terms[t];
    if (T.kind != ORC_TERM_GHOST_MASS) continue;
    if (T.defined_on && !test_bit(T.defined_on, f)) continue;
    const int order = T.order >= 0 ? T.order : 2 * s->k;
    const Rule& r = get_rule(D, order);
    const int nq = r.size();
    std::vector<double> p1(3 * 2 * nq, 0.0), p2(3 * 2 * nq, 0.0), w1(2 * nq);
    for (int l = 0; l < 2 * nq; l++) {
      if (l < nq) {
        for (int c = 0; c < 3; c++) p1[3 * l + c] = r.p[3 * l + c];
        w1[l] = r.w[l];
        double wd;
        map_patch_point(g1, g2, &p1[3 * l], w1[l], &p2[3 * l], &wd);
      } else {
        const int m = l - nq;
        for (int c = 0; c < 3; c++) p2[3 * l + c] = r.p[3 * m + c];
        map_patch_point(g2, g1, &p2[3 * l], r.w[m], &p1[3 * l], &w1[l]);
      }
    }
    double cc = T.coef;
    if (T.hpow != 0) cc *= std::pow(std::pow(std::fabs(g1.det), 1.0 / D), (double)T.hpow);
    double phi1[20], phi2[20], dphi[20][3], psi[3], dpsi[3];
    std::vector<double> sh(N2);
    for (int it = 0; it < irt.size(); it++) {
      time_basis(kt, irt.p[3 * it], psi, dpsi);
      for (int l = 0; l < 2 * nq; l++) {
        basis(D, s->k, gv1, &p1[3 * l], phi1, dphi);
        basis(D, s->k, gv2, &p2[3 * l], phi2, dphi);
        for (int tt = 0; tt < nt; tt++)
          for (int j = 0; j < nd; j++) {
            sh[tt * nd + j] = psi[tt] * phi1[j];
            sh[N + tt * nd + j] = -psi[tt] * phi2[j];
          }
        const double W = irt.w[it] * w1[l] * std::fabs(g1.det) * cc;
        for (int a = 0; a < N2; a++)
          for (int b = 0; b < N2; b++) elmat[(size_t)a * N2 + b] += W * sh[a] * sh[b];
      }
    }
  }
  return 0;
}

}  // namespace

extern "C" {

int orc_time_basis(int kt, double tau, double* psi, double* dpsi) {
  if (kt < 0 || kt > 2) return -1;
  time_basis(kt, tau, psi, dpsi);
  return kt + 1;
}

int orc_spacetime_cut_rule(int D, const double* elc, const double* lset, int kt, int dt, int order_space,
                           int order_time, double* pts, double* wts, int maxpts) {
  Geo g;
  make_geo(D, elc, g);
  std::vector<double> p, w;
  int n = st_cut_rule(g, lset, kt, dt, order_space, order_time, p, w);
  if (n < 0) return n;
  if (n > maxpts) return ERR_CAPACITY;
  std::memcpy(pts, p.data(), sizeof(double) * 4 * n);
  std::memcpy(wts, w.data(), sizeof(double) * n);
  return n;
}

// CutInformation::Update with a space-time level set and time_order = 0
// (xfem/cutinfo.cpp:83-132 calling SpaceTimeCutIntegrationRule with orders 0, 0)
int orc_cutinfo_st(const orc_space* s, const double* lset_st, int kt, uint8_t* dom, double* ratio, uint64_t* bits,
                   int nthreads) {
  const int ne = s->ne;
  const int64_t nw = (ne + 63) / 64;
  std::vector<uint8_t> d8(ne);
  std::atomic<int> err(0);
  parallel_for(ne, nthreads, [&](int64_t b, int64_t en) {
    std::vector<double> pts, wts;
    double lst[12];
    for (int64_t e = b; e < en; e++) {
      Geo g;
      element_geo(s, (int)e, g, nullptr, nullptr);
      element_lset_st(s, (int)e, lset_st, kt, lst);
      double part_vol[2] = {0.0, 0.0};
      for (int np : {POS, NEG}) {
        int n = st_cut_rule(g, lst, kt, np, 0, 0, pts, wts);
        if (n < -1) err = n;
        for (int q = 0; q < n; q++) part_vol[np] += wts[q];
      }
      ratio[e] = part_vol[NEG] / (part_vol[NEG] + part_vol[POS]);
      uint8_t t = part_vol[NEG] > 0.0 ? (part_vol[POS] > 0.0 ? IF : NEG) : POS;
      d8[e] = t;
      dom[e] = t;
    }
  });
  std::memset(bits, 0, sizeof(uint64_t) * nw * 8);
  for (int e = 0; e < ne; e++) {
    int cdt = d8[e] == NEG ? 1 : (d8[e] == POS ? 2 : 4);
    for (int c = 0; c < 8; c++)
      if ((c & cdt) || c == 7) bits[c * nw + (e >> 6)] |= (uint64_t)1 << (e & 63);
  }
  return err.load();
}

int orc_st_element_matrix(const orc_space* s, const double* lset_st, int kt_l, int kt, int order_time,
                          const orc_st_term* terms, int nterms, int e, double* elmat) {
  return st_element_matrix(s, lset_st, kt_l, kt, order_time, terms, nterms, e, elmat);
}

orc_csr* orc_assemble_st(const orc_space* s, const double* lset_st, int kt_l, int kt, int order_time,
                         const orc_st_term* terms, int nterms, int nthreads) {
  const int ne = s->ne, nd = s->nd, nt = kt + 1, N = nd * nt, N2 = 2 * N;
  const int64_t nf = s->nfacets, ndof = s->ndof * nt;
  std::vector<int32_t> ed((size_t)ne * N);
  for (int e = 0; e < ne; e++)
    for (int it = 0; it < nt; it++)
      for (int j = 0; j < nd; j++) ed[(size_t)e * N + it * nd + j] = (int32_t)(it * s->ndof + s->el_dofs[(size_t)e * nd + j]);
  std::vector<int64_t> ptr(ndof + 1, 0);
  for (size_t i = 0; i < ed.size(); i++) ptr[ed[i] + 1]++;
  for (int64_t i = 0; i < ndof; i++) ptr[i + 1] += ptr[i];
  std::vector<int32_t> adj(ed.size());
  {
    std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
    for (int e = 0; e < ne; e++)
      for (int i = 0; i < N; i++) adj[fill[ed[(size_t)e * N + i]]++] = e * 32 + i;
  }
  std::vector<int32_t> el_slot(ne, -1), fa_slot(nf, -1);
  int nact = 0, nfa = 0;
  for (int e = 0; e < ne; e++) {
    bool act = false;
    for (int t = 0; t < nterms; t++)
      if (terms[t].kind != ORC_TERM_GHOST_MASS && (!terms[t].defined_on || test_bit(terms[t].defined_on, e))) act = true;
    if (act) el_slot[e] = nact++;
  }
  for (int64_t f = 0; f < nf; f++) {
    if (s->facet_els[2 * f + 1] < 0) continue;
    bool act = false;
    for (int t = 0; t < nterms; t++)
      if (terms[t].kind == ORC_TERM_GHOST_MASS && (!terms[t].defined_on || test_bit(terms[t].defined_on, f))) act = true;
    if (act) fa_slot[f] = nfa++;
  }
  std::vector<int32_t> el_list(nact), fa_list(nfa);
  for (int e = 0; e < ne; e++) if (el_slot[e] >= 0) el_list[el_slot[e]] = e;
  for (int64_t f = 0; f < nf; f++) if (fa_slot[f] >= 0) fa_list[fa_slot[f]] = (int32_t)f;
  std::vector<double> elm((size_t)nact * N * N), fam((size_t)nfa * N2 * N2);
  std::atomic<int> err(0);
  parallel_for(nact, nthreads, [&](int64_t b, int64_t en) {
    for (int64_t i = b; i < en; i++) {
      int r = st_element_matrix(s, lset_st, kt_l, kt, order_time, terms, nterms, el_list[i], &elm[(size_t)i * N * N]);
      if (r) err = r;
    }
  });
  parallel_for(nfa, nthreads, [&](int64_t b, int64_t en) {
    for (int64_t i = b; i < en; i++) {
      int r = st_patch_matrix(s, kt, order_time, terms, nterms, fa_list[i], &fam[(size_t)i * N2 * N2]);
      if (r) err = r;
    }
  });
  if (err.load()) return nullptr;
  return gather_csr(ndof, N, ed, ptr, adj, s->D + 1, s->el_facets, s->facet_els, el_slot, elm, fa_slot, fam, nthreads);
}

}  // extern "C"

extern "C" {

// Integrate(1 * dCut(lset_st, dt, order, time_order)) over the space-time slab
// SymbolicCutLinearFormIntegrator::T_CalcElementVector (xfem/symboliccutlfi.cpp:57-180):
// elvec_i = sum_q w_q |det F| g(x_q) phi_i(x_q) over the cut rule of the term's
// domain (order 2k by default, :93-94), g = coef * x^e0 y^e1 z^e2 or coef * u_h
// (u_h a function of the same space); then the vector assembly over the
// elements in ascending order.
int orc_linear_form(const orc_space* s, const double* lset_vertex, const orc_lterm* terms, int nterms, double* out) {
  const int D = s->D, n = s->nd;
  std::fill(out, out + s->ndof, 0.0);
  std::vector<double> pts, wts;
  for (int e = 0; e < s->ne; e++) {
    Geo g;
    double l[4];
    element_geo(s, e, g, l, lset_vertex);
    int gv[4];
    for (int i = 0; i <= D; i++) gv[i] = s->elv[(size_t)e * (D + 1) + i];
    const int32_t* dofs = &s->el_dofs[(size_t)e * n];
    double b[20] = {0};
    for (int t = 0; t < nterms; t++) {
      const orc_lterm& T = terms[t];
      if (T.kind == ORC_LTERM_SOURCE_BND) continue;
      if (T.defined_on && !test_bit(T.defined_on, e)) continue;
      const int order = T.order >= 0 ? T.order : 2 * s->k;
      const int np = straight_cut_rule(g, l, T.domain, order, pts, wts);
      if (np < -1) return np;
      if (np <= 0) continue;
      const double meas = std::fabs(g.det);
      for (int q = 0; q < np; q++) {
        double phi[20], dphi[20][3];
        basis(D, s->k, gv, &pts[3 * q], phi, dphi);
        double gval;
        if (T.kind == ORC_LTERM_SOURCE) {
          double x[3] = {0, 0, 0};
          for (int i = 0; i < D; i++) {
            double sacc = g.x0[i];
            for (int k = 0; k < D; k++) sacc += g.F[i][k] * pts[3 * q + k];
            x[i] = sacc;
          }
          gval = T.coef * std::pow(x[0], T.e[0]) * std::pow(x[1], T.e[1]) * (D == 3 ? std::pow(x[2], T.e[2]) : 1.0);
        } else {
          double u = 0.0;
          for (int j = 0; j < n; j++) u += T.gf[dofs[j]] * phi[j];
          gval = T.coef * u;
        }
        const double w = wts[q] * meas * gval;
        for (int i = 0; i < n; i++) b[i] += w * phi[i];
      }
    }
    for (int i = 0; i < n; i++) out[dofs[i]] += b[i];
  }
  bool bnd_terms = false;
  for (int t = 0; t < nterms; t++) bnd_terms |= terms[t].kind == ORC_LTERM_SOURCE_BND;
  if (!bnd_terms) return 0;
  // boundary terms (dCut(lset, dt, vb=BND)): BND elements = the facets of one
  // element, vertices ascending, in lexicographic order; the trace of the
  // owning element's basis at the boundary rule's physical points
  std::vector<std::pair<std::vector<int>, int>> facets;
  for (int e = 0; e < s->ne; e++)
    for (int skip = 0; skip <= D; skip++) {
      std::vector<int> f;
      for (int v = 0; v <= D; v++)
        if (v != skip) f.push_back(s->elv[(size_t)e * (D + 1) + v]);
      std::sort(f.begin(), f.end());
      facets.push_back({f, e});
    }
  std::sort(facets.begin(), facets.end());
  int64_t b = 0;
  double xs[3 * 512], ws[512];
  for (size_t i = 0; i < facets.size();) {
    size_t j = i;
    while (j < facets.size() && facets[j].first == facets[i].first) j++;
    if (j - i == 1) {
      const int e = facets[i].second;
      Geo g;
      double l[4];
      element_geo(s, e, g, l, lset_vertex);
      int gv[4];
      for (int v = 0; v <= D; v++) gv[v] = s->elv[(size_t)e * (D + 1) + v];
      double xb[9] = {0}, lb[3];
      for (int v = 0; v < D; v++) {
        const int id = facets[i].first[v];
        lb[v] = lset_vertex[id];
        for (int r = 0; r < D; r++) xb[3 * v + r] = s->coords[(size_t)id * D + r];
      }
      const int32_t* dofs = &s->el_dofs[(size_t)e * n];
      double bv[20] = {0};
      for (int t = 0; t < nterms; t++) {
        const orc_lterm& T = terms[t];
        if (T.kind != ORC_LTERM_SOURCE_BND || (T.defined_on && !test_bit(T.defined_on, b))) continue;
        const int order = T.order >= 0 ? T.order : 2 * s->k;
        const int np = orc_bnd_element_rule(D, xb, lb, T.domain, order, xs, ws, 512);
        if (np < 0) return np == -1 ? ERR_CAPACITY : np;
        for (int q = 0; q < np; q++) {
          const double* x = &xs[3 * q];
          double xi[3] = {0, 0, 0};
          for (int k = 0; k < D; k++) {
            double acc = 0.0;
            for (int c = 0; c < D; c++) acc += g.Finv[k][c] * (x[c] - g.x0[c]);
            xi[k] = acc;
          }
          double phi[20], dphi[20][3];
          basis(D, s->k, gv, xi, phi, dphi);
          const double gval =
              T.coef * std::pow(x[0], T.e[0]) * std::pow(x[1], T.e[1]) * (D == 3 ? std::pow(x[2], T.e[2]) : 1.0);
          const double w = ws[q] * gval;
          for (int r = 0; r < n; r++) bv[r] += w * phi[r];
        }
      }
      for (int r = 0; r < n; r++) out[dofs[r]] += bv[r];
      b++;
    }
    i = j;
  }
  return 0;
}

double orc_integrate_st(const orc_space* s, const double* lset_st, int kt, int dt, int order_space, int order_time) {
  double sum = 0;
  std::vector<double> pts, wts;
  double lst[12];
  for (int e = 0; e < s->ne; e++) {
    Geo g;
    element_geo(s, e, g, nullptr, nullptr);
    element_lset_st(s, e, lset_st, kt, lst);
    int n = st_cut_rule(g, lst, kt, dt, order_space, order_time, pts, wts);
    for (int q = 0; q < n; q++) sum += wts[q] * std::fabs(g.det);
  }
  return sum;
}

}  // extern "C"

// Oracle: isoparametric cut rules and NEG-part moments for P2 level sets.
//
// THIS IS TEST INFRASTRUCTURE (see xg_oracle.h): it generates training targets
// and checks for the learned cut quadrature, and is never linked into the
// product.
//
// What it restates, per element (ngsxfem's LevelSetMeshAdaptation workflow):
//  * lset_p1 = InterpolateToP1(lset_ho) with the |v| < 1e-14 -> 1e-14
//    perturbation (utils/p1interpol.cpp:104-107, python/lsetcurv.py:325);
//  * ElementInRelevantBand(vals, 0, 0) (lsetcurving/calcpointshift.cpp:118-135):
//    only elements whose P1 vertex values have both signs (or a zero) are
//    deformed;
//  * ShiftIntegrator<D>::CalcElementVector (lsetcurving/shiftintegrators.cpp:38-122):
//    at each point of the order-2k rule, the search direction is
//    J^-1 qn with qn the physical gradient of lset_ho (the element's own exact
//    gradient: discontinuous_qn), the goal value is lset_p1 at the point, and
//    SearchCorrespondingPoint (calcpointshift.cpp:143-201) runs at most 20
//    Newton steps along the fixed direction until |goal - lset_ho| < 1e-14
//    (no convergence -> no shift); the shift (clipped at `threshold` when
//    threshold >= 0) is tested against the P2 shape functions;
//  * ProjectShift (lsetcurving/projshift.cpp:58-135): the element's mass
//    matrix inverse applied to that vector, then the vertex coefficients set
//    to zero.
//  * the averaging of shared edge dofs over the contributing elements
//    (projshift.cpp:140-197) and the deformed integration of every element,
//    in orc_iso_integrate_mesh.  That mesh-level form is pinned against the
//    reference's curved-circle test (tests/pytests/test_intcurved.py:17-91,
//    order 2: errors < 1e-5 and EOC > 2.75).
// The single-element functions (orc_iso_cut_rule, orc_iso_moments_tet) run the
// same algorithm on a one-element mesh, where the averaging is the identity:
// the rule is then a function of the element's own values (the learned
// quadrature's targets).
// The deformation Theta is expressed in reference coordinates; the deformed
// element map is F(xhat + Theta(xhat)).  The cut rule of the deformed element
// is the straight cut rule of lset_p1 on the reference element, mapped by
// xhat -> xhat + Theta(xhat), with weights times |det(J A)| (A = I + grad Theta)
// and, on the interface, times |(J A)^-T n_ref| (cutint/straightcutrule.cpp:558-578
// evaluated with the deformed transformation).
//
// Shapes and orderings (this project's statement):
//  * reference simplex vertices: trig (1,0),(0,1),(0,0); tet (1,0,0),(0,1,0),
//    (0,0,1),(0,0,0) (straightcutrule.cpp:56-60); lambda_i = x_i for i < D,
//    lambda_D = 1 - sum x;
//  * P2 nodal values: the D+1 vertex values, then the edge-midpoint values of
//    the edges (0,1),(0,2),(1,2) (trig) / (0,1),(0,2),(0,3),(1,2),(1,3),(2,3) (tet);
//  * deformation basis: lambda_i (vertices) and lambda_i lambda_j (edges); the
//    zeroed-vertex projection does not depend on the edge functions' scaling.
//  * moments: x^a y^b z^c with a+b+c <= 4 in graded order (total degree
//    t = 0..4, then a = t..0, then b = t-a..0): 35 in 3D.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "xg_oracle.h"

namespace {

constexpr int TRI_E[3][2] = {{0, 1}, {0, 2}, {1, 2}};
constexpr int TET_E[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

inline int nedges(int D) { return D == 2 ? 3 : 6; }
inline const int (*edges(int D))[2] { return D == 2 ? TRI_E : TET_E; }

void lambdas(int D, const double* x, double* l) {
  double s = 0.0;
  for (int i = 0; i < D; i++) {
    l[i] = x[i];
    s += x[i];
  }
  l[D] = 1.0 - s;
}

// d lambda_i / d x_j
inline double dlam(int D, int i, int j) { return i < D ? (i == j ? 1.0 : 0.0) : -1.0; }

// P2 nodal interpolant: value and reference gradient
double p2_value(int D, const double* v, const double* x, double* grad) {
  double l[4];
  lambdas(D, x, l);
  double val = 0.0;
  for (int j = 0; j < D; j++) grad[j] = 0.0;
  for (int i = 0; i <= D; i++) {
    // N_i = lambda_i (2 lambda_i - 1)
    val += v[i] * l[i] * (2.0 * l[i] - 1.0);
    const double dn = 4.0 * l[i] - 1.0;
    for (int j = 0; j < D; j++) grad[j] += v[i] * dn * dlam(D, i, j);
  }
  const int (*E)[2] = edges(D);
  for (int e = 0; e < nedges(D); e++) {
    const int a = E[e][0], b = E[e][1];
    const double c = v[D + 1 + e];
    val += c * 4.0 * l[a] * l[b];
    for (int j = 0; j < D; j++) grad[j] += c * 4.0 * (dlam(D, a, j) * l[b] + l[a] * dlam(D, b, j));
  }
  return val;
}

// hierarchical P2 shapes (vertex lambda_i, edge lambda_a lambda_b) and reference gradients
void p2h_shape(int D, const double* x, double* phi, double (*dphi)[3]) {
  double l[4];
  lambdas(D, x, l);
  for (int i = 0; i <= D; i++) {
    phi[i] = l[i];
    for (int j = 0; j < D; j++) dphi[i][j] = dlam(D, i, j);
  }
  const int (*E)[2] = edges(D);
  for (int e = 0; e < nedges(D); e++) {
    const int a = E[e][0], b = E[e][1];
    phi[D + 1 + e] = l[a] * l[b];
    for (int j = 0; j < D; j++) dphi[D + 1 + e][j] = dlam(D, a, j) * l[b] + l[a] * dlam(D, b, j);
  }
}

bool invert(int D, const double (*A)[3], double (*Ai)[3], double* det) {
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

// Gaussian elimination with partial pivoting, n <= 10, several right-hand sides
void solve(int n, std::vector<double> M, double* rhs, int nrhs) {
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++)
      if (std::fabs(M[r * n + c]) > std::fabs(M[p * n + c])) p = r;
    if (p != c) {
      for (int k = 0; k < n; k++) std::swap(M[c * n + k], M[p * n + k]);
      for (int k = 0; k < nrhs; k++) std::swap(rhs[c * nrhs + k], rhs[p * nrhs + k]);
    }
    for (int r = c + 1; r < n; r++) {
      const double f = M[r * n + c] / M[c * n + c];
      for (int k = c; k < n; k++) M[r * n + k] -= f * M[c * n + k];
      for (int k = 0; k < nrhs; k++) rhs[r * nrhs + k] -= f * rhs[c * nrhs + k];
    }
  }
  for (int c = n - 1; c >= 0; c--) {
    for (int k = 0; k < nrhs; k++) {
      double s = rhs[c * nrhs + k];
      for (int j = c + 1; j < n; j++) s -= M[c * n + j] * rhs[j * nrhs + k];
      rhs[c * nrhs + k] = s / M[c * n + c];
    }
  }
}

struct Affine {
  int D;
  double J[3][3];
  double Ji[3][3];
  double det;
};

bool make_affine(int D, const double* elc, Affine& a) {
  a.D = D;
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) a.J[r][c] = (r == c && r >= D) ? 1.0 : 0.0;
  for (int j = 0; j < D; j++)
    for (int r = 0; r < D; r++) a.J[r][j] = elc[j * D + r] - elc[D * D + r];
  return invert(D, a.J, a.Ji, &a.det);
}

// per-element deformation: edge coefficients theta[e][d] (reference frame).
// Returns true if the element is in the relevant band; *nonconv counts the
// searches that did not converge.
bool deformation(int D, const Affine& A, const double* p2, const double* p1, double threshold,
                 double (*theta)[3], int* nonconv) {
  const int ne = nedges(D);
  for (int e = 0; e < ne; e++)
    for (int d = 0; d < 3; d++) theta[e][d] = 0.0;
  bool has_neg = false, has_pos = false;
  for (int i = 0; i <= D; i++) {
    if (p1[i] == 0.0) has_neg = has_pos = true;
    if (p1[i] > 0.0) has_pos = true;
    if (p1[i] < 0.0) has_neg = true;
  }
  if (!(has_neg && has_pos)) return false;
  const int nd = D + 1 + ne;
  double pts[3 * 512], wts[512];
  const int nq = orc_base_rule(D, 4, pts, wts, 512);  // 2 * order, order 2
  std::vector<double> M((size_t)nd * nd, 0.0), rhs((size_t)nd * D, 0.0);
  // G = J^-1 J^-T: the search direction J^-1 qn with qn = J^-T grad_ref
  double G[3][3];
  for (int r = 0; r < D; r++)
    for (int c = 0; c < D; c++) {
      double s = 0.0;
      for (int k = 0; k < D; k++) s += A.Ji[r][k] * A.Ji[c][k];
      G[r][c] = s;
    }
  for (int q = 0; q < nq; q++) {
    const double* x0 = &pts[3 * q];
    double phi[10], dphi[10][3];
    p2h_shape(D, x0, phi, dphi);
    for (int i = 0; i < nd; i++)
      for (int j = 0; j < nd; j++) M[i * nd + j] += wts[q] * phi[i] * phi[j];
    double l[4];
    lambdas(D, x0, l);
    double goal = 0.0;
    for (int i = 0; i <= D; i++) goal += p1[i] * l[i];
    double g0[3];
    p2_value(D, p2, x0, g0);
    double s[3];
    for (int r = 0; r < D; r++) {
      s[r] = 0.0;
      for (int c = 0; c < D; c++) s[r] += G[r][c] * g0[c];
    }
    double cur[3] = {x0[0], x0[1], D == 3 ? x0[2] : 0.0};
    int it = 0;
    for (it = 0; it < 20; ++it) {
      double g[3];
      const double val = p2_value(D, p2, cur, g);
      const double defect = goal - val;
      if (std::fabs(defect) < 1e-14) break;
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
      const double n = std::sqrt(n2);
      if (n > threshold)
        for (int r = 0; r < D; r++) dist[r] *= threshold / n;
    }
    for (int i = 0; i < nd; i++)
      for (int r = 0; r < D; r++) rhs[i * D + r] += wts[q] * phi[i] * dist[r];
  }
  solve(nd, M, rhs.data(), D);
  for (int e = 0; e < ne; e++)
    for (int r = 0; r < D; r++) theta[e][r] = rhs[(D + 1 + e) * D + r];
  return true;
}

// deformed point y = x + Theta(x) and A = I + grad Theta (reference frame)
void deform_at(int D, const double (*theta)[3], const double* x, double* y, double (*Am)[3]) {
  double phi[10], dphi[10][3];
  p2h_shape(D, x, phi, dphi);
  const int ne = nedges(D);
  for (int r = 0; r < 3; r++) {
    y[r] = r < D ? x[r] : 0.0;
    for (int c = 0; c < 3; c++) Am[r][c] = r == c ? 1.0 : 0.0;
  }
  for (int e = 0; e < ne; e++) {
    const int k = D + 1 + e;
    for (int r = 0; r < D; r++) {
      y[r] += theta[e][r] * phi[k];
      for (int c = 0; c < D; c++) Am[r][c] += theta[e][r] * dphi[k][c];
    }
  }
}

void perturbed_p1(int D, const double* p2, double* p1) {
  for (int i = 0; i <= D; i++) {
    p1[i] = p2[i];
    if (std::fabs(p1[i]) < 1e-14) p1[i] = 1e-14;
  }
}

const double REF_TRI[6] = {1, 0, 0, 1, 0, 0};
const double REF_TET[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};

// cut rule of lset_p1 on the reference element, mapped by xhat -> xhat + Theta(xhat)
int mapped_rule(int D, const Affine& A, const double* p1, const double (*theta)[3], int dt, int order,
                std::vector<double>& pts, std::vector<double>& wts) {
  const int maxp = 4096;
  std::vector<double> rp(3 * maxp), rw(maxp);
  const int n = orc_straight_cut_rule(D, D == 2 ? REF_TRI : REF_TET, p1, dt, order, rp.data(), rw.data(), maxp);
  pts.clear();
  wts.clear();
  if (n < 0) return n;
  // unit normal of lset_p1 in reference coordinates
  double nref[3] = {0, 0, 0};
  for (int j = 0; j < D; j++) nref[j] = p1[j] - p1[D];
  double nn = 0.0;
  for (int j = 0; j < D; j++) nn += nref[j] * nref[j];
  nn = std::sqrt(nn);
  for (int j = 0; j < D; j++) nref[j] /= nn;
  for (int q = 0; q < n; q++) {
    double y[3], Am[3][3];
    deform_at(D, theta, &rp[3 * q], y, Am);
    // F = J A
    double F[3][3], Fi[3][3], detF;
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) {
        double s = 0.0;
        for (int k = 0; k < 3; k++) s += A.J[r][k] * Am[k][c];
        F[r][c] = s;
      }
    if (!invert(D, F, Fi, &detF)) return -3;
    double w = rw[q] * std::fabs(detF);
    if (dt == ORC_IF) {
      double t2 = 0.0;
      for (int r = 0; r < D; r++) {
        double s = 0.0;
        for (int k = 0; k < D; k++) s += Fi[k][r] * nref[k];
        t2 += s * s;
      }
      w *= std::sqrt(t2);
    }
    pts.push_back(y[0]);
    pts.push_back(y[1]);
    pts.push_back(D == 3 ? y[2] : 0.0);
    wts.push_back(w);
  }
  return n;
}

// single-element (one-element mesh) isoparametric rule
int iso_rule(int D, const double* elc, const double* p2, int dt, int order, double threshold, bool deform,
             std::vector<double>& pts, std::vector<double>& wts, int* nonconv) {
  Affine A;
  if (!make_affine(D, elc, A)) return -2;
  double p1[4];
  perturbed_p1(D, p2, p1);
  double theta[6][3];
  if (deform) {
    deformation(D, A, p2, p1, threshold, theta, nonconv);
  } else {
    for (int e = 0; e < 6; e++)
      for (int r = 0; r < 3; r++) theta[e][r] = 0.0;
  }
  return mapped_rule(D, A, p1, theta, dt, order, pts, wts);
}

void moments_tet(const std::vector<double>& pts, const std::vector<double>& wts, double* out) {
  for (int k = 0; k < 35; k++) out[k] = 0.0;
  for (size_t q = 0; q < wts.size(); q++) {
    const double x = pts[3 * q], y = pts[3 * q + 1], z = pts[3 * q + 2];
    double px[5] = {1, x, x * x, x * x * x, x * x * x * x};
    double py[5] = {1, y, y * y, y * y * y, y * y * y * y};
    double pz[5] = {1, z, z * z, z * z * z, z * z * z * z};
    int k = 0;
    for (int t = 0; t <= 4; t++)
      for (int a = t; a >= 0; a--)
        for (int b = t - a; b >= 0; b--) out[k++] += wts[q] * px[a] * py[b] * pz[t - a - b];
  }
}

template <class F>
void parallel_for(int64_t n, int nthreads, F&& f) {
  nthreads = std::max(1, std::min<int>(nthreads, (int)std::max<int64_t>(1, n / 64)));
  if (nthreads == 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  const int64_t chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    const int64_t b = t * chunk, e = std::min(n, b + chunk);
    if (b < e) th.emplace_back([&, b, e] { f(b, e); });
  }
  for (auto& x : th) x.join();
}

// red refinement of a tetrahedron (Bey): 8 children from the 4 vertices and 6 midpoints
void subdiv_neg_moments(const double (*v)[3], const double* p2, int level, double* out) {
  if (level == 0) {
    double vals[4], elc[12];
    for (int i = 0; i < 4; i++) {
      double g[3];
      vals[i] = p2_value(3, p2, v[i], g);
      for (int r = 0; r < 3; r++) elc[3 * i + r] = v[i][r];
    }
    double pts[3 * 512], wts[512];
    const int n = orc_straight_cut_rule(3, elc, vals, ORC_NEG, 4, pts, wts, 512);
    if (n <= 0) return;
    Affine A;
    if (!make_affine(3, elc, A)) return;
    std::vector<double> P, W;
    for (int q = 0; q < n; q++) {
      double x[3];
      for (int r = 0; r < 3; r++) {
        x[r] = elc[9 + r];
        for (int j = 0; j < 3; j++) x[r] += A.J[r][j] * pts[3 * q + j];
        P.push_back(x[r]);
      }
      W.push_back(wts[q] * std::fabs(A.det));
    }
    double m[35];
    moments_tet(P, W, m);
    for (int k = 0; k < 35; k++) out[k] += m[k];
    return;
  }
  double mid[4][4][3];
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++)
      for (int r = 0; r < 3; r++) mid[a][b][r] = 0.5 * (v[a][r] + v[b][r]);
  const double* C[8][4] = {
      {v[0], mid[0][1], mid[0][2], mid[0][3]}, {mid[0][1], v[1], mid[1][2], mid[1][3]},
      {mid[0][2], mid[1][2], v[2], mid[2][3]}, {mid[0][3], mid[1][3], mid[2][3], v[3]},
      {mid[0][1], mid[0][2], mid[0][3], mid[1][3]}, {mid[0][1], mid[0][2], mid[1][2], mid[1][3]},
      {mid[0][2], mid[0][3], mid[1][3], mid[2][3]}, {mid[0][2], mid[1][2], mid[1][3], mid[2][3]}};
  for (int c = 0; c < 8; c++) {
    double w[4][3];
    for (int i = 0; i < 4; i++)
      for (int r = 0; r < 3; r++) w[i][r] = C[c][i][r];
    subdiv_neg_moments(w, p2, level - 1, out);
  }
}

}  // namespace

extern "C" {

int orc_iso_cut_rule(int D, const double* elc, const double* p2vals, int dt, int order, double threshold,
                     int deform, double* pts, double* wts, int maxpts, int* nonconv) {
  if ((D != 2 && D != 3) || dt < 0 || dt > 2) return -4;
  std::vector<double> p, w;
  int nc = 0;
  const int n = iso_rule(D, elc, p2vals, dt, order, threshold, deform != 0, p, w, &nc);
  if (nonconv) *nonconv = nc;
  if (n < 0) return n;
  if (n > maxpts) return -5;
  std::memcpy(pts, p.data(), sizeof(double) * 3 * n);
  std::memcpy(wts, w.data(), sizeof(double) * n);
  return n;
}

int orc_iso_deformation(int D, const double* elc, const double* p2vals, double threshold, double* theta_out,
                        int* nonconv) {
  Affine A;
  if ((D != 2 && D != 3) || !make_affine(D, elc, A)) return -4;
  double p1[4];
  perturbed_p1(D, p2vals, p1);
  double theta[6][3];
  int nc = 0;
  const bool band = deformation(D, A, p2vals, p1, threshold, theta, &nc);
  for (int e = 0; e < nedges(D); e++)
    for (int r = 0; r < D; r++) theta_out[e * D + r] = theta[e][r];
  if (nonconv) *nonconv = nc;
  return band ? 1 : 0;
}

int orc_iso_moments_tet(int64_t n, const double* vals10, int order, int deform, double* out35, int32_t* nonconv,
                        int nthreads) {
  parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
    std::vector<double> p, w;
    for (int64_t i = b; i < e; i++) {
      int nc = 0;
      const int k = iso_rule(3, REF_TET, vals10 + 10 * i, ORC_NEG, order, -1.0, deform != 0, p, w, &nc);
      if (k < 0) {  // -1: no rule (the element is POS), below: an error
        p.clear();
        w.clear();
      }
      moments_tet(p, w, out35 + 35 * i);
      if (nonconv) nonconv[i] = k < -1 ? -1 : nc;
    }
  });
  return 0;
}

int orc_iso_theta_mesh(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* p2vals,
                       double threshold, double* theta_out, int* nonconv) {
  // the averaging of orc_iso_integrate_mesh, each element's edge
  // coefficients returned in its reference frame
  (void)nv;
  const int nn = (D + 1) * (D + 2) / 2, nle = nedges(D);
  const int (*E)[2] = edges(D);
  std::vector<uint64_t> keys((size_t)ne * nle);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < nle; j++) {
      uint64_t a = (uint32_t)elv[e * (D + 1) + E[j][0]], b = (uint32_t)elv[e * (D + 1) + E[j][1]];
      if (a > b) std::swap(a, b);
      keys[(size_t)e * nle + j] = (a << 32) | b;
    }
  std::vector<uint64_t> uk(keys);
  std::sort(uk.begin(), uk.end());
  uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
  std::vector<int32_t> eid(keys.size());
  for (size_t i = 0; i < keys.size(); i++) eid[i] = (int32_t)(std::lower_bound(uk.begin(), uk.end(), keys[i]) - uk.begin());
  std::vector<double> gdef(uk.size() * 3, 0.0), fac(uk.size(), 0.0);
  std::vector<Affine> aff(ne);
  int nc = 0;
  for (int e = 0; e < ne; e++) {
    double elc[12];
    for (int i = 0; i <= D; i++)
      for (int r = 0; r < D; r++) elc[i * D + r] = coords[(size_t)elv[e * (D + 1) + i] * D + r];
    if (!make_affine(D, elc, aff[e])) return -2;
    double p1[4];
    perturbed_p1(D, p2vals + (size_t)e * nn, p1);
    double theta[6][3];
    if (!deformation(D, aff[e], p2vals + (size_t)e * nn, p1, threshold, theta, &nc)) continue;
    for (int j = 0; j < nle; j++) {
      const int g = eid[(size_t)e * nle + j];
      for (int r = 0; r < D; r++) {
        double acc = 0.0;
        for (int c = 0; c < D; c++) acc += aff[e].J[r][c] * theta[j][c];
        gdef[(size_t)g * 3 + r] += acc;
      }
      fac[g] += 1.0;
    }
  }
  for (size_t g = 0; g < uk.size(); g++)
    if (fac[g] > 0)
      for (int r = 0; r < 3; r++) gdef[g * 3 + r] /= fac[g];
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < 6; j++)
      for (int r = 0; r < 3; r++) {
        double acc = 0.0;
        if (j < nle && r < D) {
          const int g = eid[(size_t)e * nle + j];
          for (int c = 0; c < D; c++) acc += aff[e].Ji[r][c] * gdef[(size_t)g * 3 + c];
        }
        theta_out[((size_t)e * 6 + j) * 3 + r] = acc;
      }
  if (nonconv) *nonconv = nc;
  return 0;
}

double orc_iso_integrate_mesh(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* p2vals,
                              int dt, int order, double threshold, int deform, int* nonconv) {
  // ProjectShift over the band elements (projshift.cpp:58-135): element
  // contributions J * theta_ref summed on the global edge dofs, then divided
  // by the number of contributing elements (projshift.cpp:140-197); every
  // element (cut or not) is then integrated with its deformed map.
  const int nn = (D + 1) * (D + 2) / 2, nle = nedges(D);
  const int (*E)[2] = edges(D);
  std::vector<uint64_t> keys((size_t)ne * nle);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < nle; j++) {
      uint64_t a = (uint32_t)elv[e * (D + 1) + E[j][0]], b = (uint32_t)elv[e * (D + 1) + E[j][1]];
      if (a > b) std::swap(a, b);
      keys[(size_t)e * nle + j] = (a << 32) | b;
    }
  std::vector<uint64_t> uk(keys);
  std::sort(uk.begin(), uk.end());
  uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
  std::vector<int32_t> eid(keys.size());
  for (size_t i = 0; i < keys.size(); i++) eid[i] = (int32_t)(std::lower_bound(uk.begin(), uk.end(), keys[i]) - uk.begin());
  std::vector<double> gdef(uk.size() * 3, 0.0), fac(uk.size(), 0.0);
  std::vector<Affine> aff(ne);
  int nc = 0;
  for (int e = 0; e < ne; e++) {
    double elc[12];
    for (int i = 0; i <= D; i++)
      for (int r = 0; r < D; r++) elc[i * D + r] = coords[(size_t)elv[e * (D + 1) + i] * D + r];
    if (!make_affine(D, elc, aff[e])) return NAN;
    if (!deform) continue;
    double p1[4];
    perturbed_p1(D, p2vals + (size_t)e * nn, p1);
    double theta[6][3];
    if (!deformation(D, aff[e], p2vals + (size_t)e * nn, p1, threshold, theta, &nc)) continue;
    for (int j = 0; j < nle; j++) {
      const int g = eid[(size_t)e * nle + j];
      for (int r = 0; r < D; r++) {
        double s = 0.0;
        for (int c = 0; c < D; c++) s += aff[e].J[r][c] * theta[j][c];
        gdef[(size_t)g * 3 + r] += s;
      }
      fac[g] += 1.0;
    }
  }
  for (size_t g = 0; g < uk.size(); g++)
    if (fac[g] > 0)
      for (int r = 0; r < 3; r++) gdef[g * 3 + r] /= fac[g];
  double total = 0.0;
  std::vector<double> p, w;
  for (int e = 0; e < ne; e++) {
    double theta[6][3] = {};
    for (int j = 0; j < nle; j++) {
      const int g = eid[(size_t)e * nle + j];
      for (int r = 0; r < D; r++) {
        double s = 0.0;
        for (int c = 0; c < D; c++) s += aff[e].Ji[r][c] * gdef[(size_t)g * 3 + c];
        theta[j][r] = s;
      }
    }
    double p1[4];
    perturbed_p1(D, p2vals + (size_t)e * nn, p1);
    if (mapped_rule(D, aff[e], p1, theta, dt, order, p, w) < -1) return NAN;
    for (double x : w) total += x;
  }
  if (nonconv) *nonconv = nc;
  return total;
}

int orc_subdiv_moments_tet(const double* vals10, int levels, double* out35) {
  const double v[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
  for (int k = 0; k < 35; k++) out35[k] = 0.0;
  subdiv_neg_moments(v, vals10, levels, out35);
  return 0;
}

}  // extern "C"

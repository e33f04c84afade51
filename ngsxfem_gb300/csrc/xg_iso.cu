// P2 level sets on tetrahedra: per-element isoparametric NEG-part moments (the
// reference's LevelSetMeshAdaptation workflow on a one-element mesh) and the
// straight-cut moments of the P1 interpolant.  One thread per element, FP64.
//
// Compiled with -fmad=false: the cut geometry follows the CPU statement of
// ngsxfem's straightcutrule.cpp operation by operation (xg_cut.cuh).
//
// Restated algorithm (per element, reference tet, J = I):
//  * lset_p1: the four vertex values with InterpolateToP1's |v| < 1e-14 -> 1e-14
//    (utils/p1interpol.cpp:104-107);
//  * relevant band (lsetcurving/calcpointshift.cpp:118-135): deform only if
//    the P1 values have both signs or a zero;
//  * ShiftIntegrator::CalcElementVector (lsetcurving/shiftintegrators.cpp:38-122)
//    over the order-4 rule: goal = lset_p1(x), search direction = gradient of
//    the P2 function at x, SearchCorrespondingPoint
//    (lsetcurving/calcpointshift.cpp:143-201): at most 20 Newton steps along
//    the fixed direction, stop when |goal - value| < 1e-14, no shift if not
//    converged; the shift is tested against the hierarchical P2 shapes;
//  * ProjectShift (lsetcurving/projshift.cpp:58-135): inverse mass matrix,
//    vertex coefficients set to zero (only the 6 edge coefficients remain);
//  * the straight cut rule of lset_p1 (NEG) mapped by x -> x + Theta(x) with
//    weights times |det(I + grad Theta)|; moments x^a y^b z^c, a+b+c <= 4 in
//    graded order (t = 0..4, a = t..0, b = t-a..0).
#include <cmath>
#include <mutex>
#include <vector>

#include "xg_cut.cuh"
#include "xg_internal.h"

namespace xg {

static __constant__ RuleTable c_rules;
// inverse of the hierarchical P2 mass matrix of the reference tet (order-4 rule)
static __constant__ double c_minv[100];

namespace {

// edges (0,1),(0,2),(0,3),(1,2),(1,3),(2,3)
__host__ __device__ __forceinline__ int edge_a(int e) { return e < 3 ? 0 : (e < 5 ? 1 : 2); }
__host__ __device__ __forceinline__ int edge_b(int e) { return e < 3 ? e + 1 : (e == 3 ? 2 : 3); }

__host__ __device__ __forceinline__ double dlam(int i, int j) { return i < 3 ? (i == j ? 1.0 : 0.0) : -1.0; }

__host__ __device__ __forceinline__ void lambdas(const double* x, double* l) {
  double s = 0.0;
  for (int i = 0; i < 3; i++) {
    l[i] = x[i];
    s += x[i];
  }
  l[3] = 1.0 - s;
}

// P2 nodal function: value and reference gradient
__host__ __device__ __forceinline__ double p2_value(const double* v, const double* x, double* grad) {
  double l[4];
  lambdas(x, l);
  double val = 0.0;
  for (int j = 0; j < 3; j++) grad[j] = 0.0;
  for (int i = 0; i <= 3; i++) {
    val += v[i] * l[i] * (2.0 * l[i] - 1.0);
    const double dn = 4.0 * l[i] - 1.0;
    for (int j = 0; j < 3; j++) grad[j] += v[i] * dn * dlam(i, j);
  }
  for (int e = 0; e < 6; e++) {
    const int a = edge_a(e), b = edge_b(e);
    const double c = v[4 + e];
    val += c * 4.0 * l[a] * l[b];
    for (int j = 0; j < 3; j++) grad[j] += c * 4.0 * (dlam(a, j) * l[b] + l[a] * dlam(b, j));
  }
  return val;
}

__host__ __device__ __forceinline__ void p2h_shape(const double* x, double* phi) {
  double l[4];
  lambdas(x, l);
  for (int i = 0; i < 4; i++) phi[i] = l[i];
  for (int e = 0; e < 6; e++) phi[4 + e] = l[edge_a(e)] * l[edge_b(e)];
}

// y = x + Theta(x), A = I + grad Theta
__device__ __forceinline__ void deform_at(const double (*theta)[3], const double* x, double* y, double (*A)[3]) {
  double l[4];
  lambdas(x, l);
  for (int r = 0; r < 3; r++) {
    y[r] = x[r];
    for (int c = 0; c < 3; c++) A[r][c] = r == c ? 1.0 : 0.0;
  }
  for (int e = 0; e < 6; e++) {
    const int a = edge_a(e), b = edge_b(e);
    const double phi = l[a] * l[b];
    double dphi[3];
    for (int c = 0; c < 3; c++) dphi[c] = dlam(a, c) * l[b] + l[a] * dlam(b, c);
    for (int r = 0; r < 3; r++) {
      y[r] += theta[e][r] * phi;
      for (int c = 0; c < 3; c++) A[r][c] += theta[e][r] * dphi[c];
    }
  }
}

__device__ __forceinline__ double det3(const double (*A)[3]) {
  return A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
         A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
}

__device__ __forceinline__ void add_moments(double* m, double w, const double* y) {
  double px[5], py[5], pz[5];
  px[0] = py[0] = pz[0] = 1.0;
  for (int k = 1; k < 5; k++) {
    px[k] = px[k - 1] * y[0];
    py[k] = py[k - 1] * y[1];
    pz[k] = pz[k - 1] * y[2];
  }
  int k = 0;
  for (int t = 0; t <= 4; t++)
    for (int a = t; a >= 0; a--)
      for (int b = t - a; b >= 0; b--) m[k++] += w * px[a] * py[b] * pz[t - a - b];
}

// the per-element deformation; returns the number of non-converged searches
__device__ int iso_theta(const double* v, const double* p1, double (*theta)[3]) {
  for (int e = 0; e < 6; e++)
    for (int r = 0; r < 3; r++) theta[e][r] = 0.0;
  bool has_neg = false, has_pos = false;
  for (int i = 0; i < 4; i++) {
    if (p1[i] == 0.0) has_neg = has_pos = true;
    if (p1[i] > 0.0) has_pos = true;
    if (p1[i] < 0.0) has_neg = true;
  }
  if (!(has_neg && has_pos)) return 0;
  const int o4 = c_rules.off[3][4], n4 = c_rules.cnt[3][4];
  double rhs[10][3];
  for (int i = 0; i < 10; i++)
    for (int r = 0; r < 3; r++) rhs[i][r] = 0.0;
  int nonconv = 0;
  for (int q = 0; q < n4; q++) {
    const double x0[3] = {c_rules.x[o4 + q][0], c_rules.x[o4 + q][1], c_rules.x[o4 + q][2]};
    const double w = c_rules.w[o4 + q];
    double phi[10];
    p2h_shape(x0, phi);
    double l[4];
    lambdas(x0, l);
    double goal = 0.0;
    for (int i = 0; i < 4; i++) goal += p1[i] * l[i];
    double s[3];
    p2_value(v, x0, s);
    double cur[3] = {x0[0], x0[1], x0[2]};
    int it = 0;
    for (it = 0; it < 20; ++it) {
      double g[3];
      const double val = p2_value(v, cur, g);
      const double defect = goal - val;
      if (fabs(defect) < 1e-14) break;
      const double dn = g[0] * s[0] + g[1] * s[1] + g[2] * s[2];
      for (int r = 0; r < 3; r++) cur[r] += defect / dn * s[r];
    }
    double dist[3] = {0.0, 0.0, 0.0};
    if (it == 20)
      nonconv++;
    else
      for (int r = 0; r < 3; r++) dist[r] = cur[r] - x0[r];
    for (int i = 0; i < 10; i++)
      for (int r = 0; r < 3; r++) rhs[i][r] += w * phi[i] * dist[r];
  }
  for (int e = 0; e < 6; e++)
    for (int r = 0; r < 3; r++) {
      double s = 0.0;
      for (int j = 0; j < 10; j++) s += c_minv[(4 + e) * 10 + j] * rhs[j][r];
      theta[e][r] = s;
    }
  return nonconv;
}

}  // namespace

// NEG-part moments of the reference tet under the P2 values of each element
// (deform = 0: the straight cut rule of the P1 interpolant alone).  With a
// list, element list[i] for i < *count (count on the device).
__global__ void __launch_bounds__(128) k_tet_moments(const double* __restrict__ vals, int64_t n,
                                                      const int32_t* __restrict__ list, const int32_t* count,
                                                      int order, int deform, double* __restrict__ out,
                                                      int32_t* nonconv) {
  const int64_t cnt = count ? (int64_t)*count : n;
  for (int64_t ii = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ii < cnt; ii += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = list ? (int64_t)list[ii] : ii;
    double v[10];
    for (int k = 0; k < 10; k++) v[k] = vals[i * 10 + k];
    double p1[4];
    for (int k = 0; k < 4; k++) p1[k] = fabs(v[k]) < 1e-14 ? 1e-14 : v[k];
    double theta[6][3];
    int nc = 0;
    if (deform) {
      nc = iso_theta(v, p1, theta);
    } else {
      for (int e = 0; e < 6; e++)
        for (int r = 0; r < 3; r++) theta[e][r] = 0.0;
    }
    double m[35];
    for (int k = 0; k < 35; k++) m[k] = 0.0;
    const int p = clamp_order(order);
    const int ob = c_rules.off[3][p], nb = c_rules.cnt[3][p];
    const int dom = check_if_straight_cut(p1, 4);
    Sub subs[3];
    int ns = 0;
    if (dom == XG_IF) {
      ns = decompose<3>(p1, XG_NEG, subs);
      if (ns < 0) {
        nc = -1;
        ns = 0;
      }
    } else if (dom == XG_NEG) {
      ns = 1;  // the whole element with its base rule
      for (int a = 0; a < 4; a++)
        for (int k = 0; k < 3; k++) subs[0].p[a].c[k] = (a < 3 && k == a) ? 1.0 : 0.0;
    }
    for (int s = 0; s < ns; s++) {
      const bool whole = dom == XG_NEG;
      const double trafofac = whole ? 1.0 : simplex_volume(subs[s].p, 4);
      for (int q = 0; q < nb; q++) {
        const double* ip = c_rules.x[ob + q];
        double x[3];
        if (whole) {
          x[0] = ip[0];
          x[1] = ip[1];
          x[2] = ip[2];
        } else {
          plain_point(subs[s], 4, ip, x);
        }
        double y[3], A[3][3];
        deform_at(theta, x, y, A);
        const double w = (whole ? c_rules.w[ob + q] : c_rules.w[ob + q] * trafofac) * fabs(det3(A));
        add_moments(m, w, y);
      }
    }
    for (int k = 0; k < 35; k++) out[i * 35 + k] = m[k];
    if (nonconv) nonconv[i] = nc;
  }
}

namespace {
int upload_iso() {
  static std::mutex mu;
  static std::vector<int> done;
  int dev = 0;
  XG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  for (int d : done)
    if (d == dev) return XG_OK;
  int st = ensure_device_rules();
  if (st) return st;
  // hierarchical P2 mass matrix of the reference tet with the order-4 rule, inverted
  const RuleTable& R = host_rules();
  double M[10][10] = {}, Mi[10][10] = {};
  for (int q = 0; q < R.cnt[3][4]; q++) {
    double phi[10];
    p2h_shape(R.x[R.off[3][4] + q], phi);
    for (int a = 0; a < 10; a++)
      for (int b = 0; b < 10; b++) M[a][b] += R.w[R.off[3][4] + q] * phi[a] * phi[b];
  }
  for (int a = 0; a < 10; a++) Mi[a][a] = 1.0;
  for (int c = 0; c < 10; c++) {
    int piv = c;
    for (int r = c + 1; r < 10; r++)
      if (std::fabs(M[r][c]) > std::fabs(M[piv][c])) piv = r;
    for (int k = 0; k < 10; k++) {
      std::swap(M[c][k], M[piv][k]);
      std::swap(Mi[c][k], Mi[piv][k]);
    }
    const double d = M[c][c];
    for (int k = 0; k < 10; k++) {
      M[c][k] /= d;
      Mi[c][k] /= d;
    }
    for (int r = 0; r < 10; r++)
      if (r != c) {
        const double f = M[r][c];
        for (int k = 0; k < 10; k++) {
          M[r][k] -= f * M[c][k];
          Mi[r][k] -= f * Mi[c][k];
        }
      }
  }
  XG_CUDA(cudaMemcpyToSymbol(c_rules, &R, sizeof(RuleTable)));
  XG_CUDA(cudaMemcpyToSymbol(c_minv, &Mi[0][0], sizeof(Mi)));
  done.push_back(dev);
  return XG_OK;
}
}  // namespace

int tet_moments_launch(const double* d_vals, int64_t n, int order, int deform, double* d_out, int32_t* d_nonconv,
                       cudaStream_t s, const int32_t* d_list, const int32_t* d_count) {
  int st = upload_iso();
  if (st) return st;
  if (n == 0) return XG_OK;
  const int64_t blocks = std::min<int64_t>((n + 127) / 128, 152 * 16);
  k_tet_moments<<<(unsigned)blocks, 128, 0, s>>>(d_vals, n, d_list, d_count, order, deform, d_out, d_nonconv);
  XG_CUDA(cudaGetLastError());
  return XG_OK;
}

}  // namespace xg

extern "C" int xg_iso_moments_tet(const double* d_vals10, int64_t n, int order, int deform, double* d_out35,
                                  int32_t* d_nonconv, void* stream) {
  if (!d_vals10 || !d_out35 || n < 0 || order < 0 || order > xg::kMaxOrder) return XG_ERR_ARG;
  return xg::tet_moments_launch(d_vals10, n, order, deform, d_out35, d_nonconv, (cudaStream_t)stream, nullptr,
                                nullptr);
}

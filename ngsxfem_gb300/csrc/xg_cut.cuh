// Device-side straight-cut geometry on simplices and the H1 basis.
//
// Follows ngsxfem cutint/straightcutrule.cpp:
//   CheckIfStraightCut          :11-24
//   CalcIFPolytopEUsingLset     :41-64
//   SimpleX::GetVolume          :66-72
//   GetPlainIntegrationRule     :80-100
//   LevelsetCutSimplex::Decompose :131-196
//   LevelsetWrapper normal      :509-513, 525-538
// The operation order matches the CPU statement of the same functions so that
// a translation unit compiled with -fmad=false reproduces its bits.
#pragma once
#include <cstdint>

#include "xg_internal.h"

namespace xg {

struct P3 {
  double c[3];
};

// Sign tests of CheckIfStraightCut with epsilon = 0 done on the bit pattern
// (integer pipe; the FP64 pipe of GB300 is narrow): v > 0 <=> sign clear and
// not +0; v < 0 <=> sign set and not -0.  NaN never occurs in valid input.
__device__ __forceinline__ bool d_pos(double v) {
  long long b = __double_as_longlong(v);
  return b > 0;
}
__device__ __forceinline__ bool d_neg(double v) {
  long long b = __double_as_longlong(v);
  return b < 0 && (b & 0x7fffffffffffffffLL) != 0;
}
// (v >= 0) of the edge test in CalcIFPolytopEUsingLset
__device__ __forceinline__ bool d_geq0(double v) { return !d_neg(v); }

__device__ __forceinline__ int check_if_straight_cut(const double* v, int n) {
  bool haspos = false, hasneg = false;
  for (int i = 0; i < n; i++) {
    haspos |= d_pos(v[i]);
    hasneg |= d_neg(v[i]);
  }
  if ((hasneg && haspos) || (!hasneg && !haspos)) return XG_IF;
  return hasneg ? XG_NEG : XG_POS;
}

__device__ __forceinline__ P3 seg_point(const P3& a, const P3& b, double la, double lb) {
  double t = la / (la - lb);
  P3 r;
#pragma unroll
  for (int k = 0; k < 3; k++) r.c[k] = a.c[k] + t * (b.c[k] - a.c[k]);
  return r;
}

__device__ __forceinline__ double l2norm3(double a, double b, double c) { return sqrt(a * a + b * b + c * c); }

// Cut points of the reference simplex of dimension D (D+1 vertices).
// Returns #points or a negative xg error.
template <int D>
__device__ __forceinline__ int calc_if_points(const double* l, P3* out) {
  if (check_if_straight_cut(l, D + 1) != XG_IF) return -XG_ERR_PLAIN_CUT;
  P3 s[D + 1];
#pragma unroll
  for (int i = 0; i <= D; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) s[i].c[k] = (i < D && k == i) ? 1.0 : 0.0;
  int n = 0;
#pragma unroll
  for (int i = 0; i <= D; i++)
#pragma unroll
    for (int j = i + 1; j <= D; j++)
      if (d_geq0(l[i]) != d_geq0(l[j])) {
        // the recursive CheckIfStraightCut on the edge (straightcutrule.cpp:43)
        bool hp = d_pos(l[i]) || d_pos(l[j]);
        bool hn = d_neg(l[i]) || d_neg(l[j]);
        if (!(hp && hn)) return -XG_ERR_PLAIN_CUT;
        out[n++] = seg_point(s[i], s[j], l[i], l[j]);
      }
  return n;
}

struct Sub {
  P3 p[4];
};

// Volume of a simplex with np = dim+1 points (straightcutrule.cpp:66-72).
__device__ __forceinline__ double simplex_volume(const P3* p, int np) {
  if (np == 2) {
    return l2norm3(p[1].c[0] - p[0].c[0], p[1].c[1] - p[0].c[1], p[1].c[2] - p[0].c[2]);
  }
  if (np == 3) {
    double a[3], b[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      a[k] = p[2].c[k] - p[0].c[k];
      b[k] = p[1].c[k] - p[0].c[k];
    }
    return l2norm3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
  }
  double a[3], b[3], c[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    a[k] = p[3].c[k] - p[0].c[k];
    b[k] = p[2].c[k] - p[0].c[k];
    c[k] = p[1].c[k] - p[0].c[k];
  }
  double det = a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) +
               a[2] * (b[0] * c[1] - b[1] * c[0]);
  return fabs(det);
}

// LevelsetCutSimplex::Decompose for the reference simplex of dimension D.
// Writes up to 3 sub-simplices; sub-simplex dimension is D (NEG/POS) or D-1 (IF).
// Returns #sub-simplices or a negative xg error.
template <int D>
__device__ __forceinline__ int decompose_cuts(const double* l, int dt, const P3* cut, int nc, Sub* subs) {
  P3 s[D + 1];
#pragma unroll
  for (int i = 0; i <= D; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) s[i].c[k] = (i < D && k == i) ? 1.0 : 0.0;
  if (dt == XG_IF) {
    if (nc == D) {
      for (int i = 0; i < D; i++) subs[0].p[i] = cut[i];
      return 1;
    }
    if (D == 3 && nc == 4) {
      subs[0].p[0] = cut[0]; subs[0].p[1] = cut[1]; subs[0].p[2] = cut[3];
      subs[1].p[0] = cut[0]; subs[1].p[1] = cut[2]; subs[1].p[2] = cut[3];
      return 2;
    }
    return -XG_ERR_BAD_DECOMP;
  }
  int rel[4], nr = 0;
#pragma unroll
  for (int i = 0; i <= D; i++)
    if ((dt == XG_POS && d_geq0(l[i])) || (dt == XG_NEG && d_neg(l[i]))) rel[nr++] = i;
  if (nr == 1) {
    if (nc != D) return -XG_ERR_BAD_DECOMP;
    for (int i = 0; i < nc; i++) subs[0].p[i] = cut[i];
    subs[0].p[nc] = s[rel[0]];
    return 1;
  }
  if (D == 2 && nr == 2) {
    subs[0].p[0] = s[rel[0]]; subs[0].p[1] = s[rel[1]]; subs[0].p[2] = cut[1];
    subs[1].p[0] = cut[0]; subs[1].p[1] = cut[1]; subs[1].p[2] = s[rel[0]];
    return 2;
  }
  if (D == 3 && nr == 2) {
    if (nc != 4) return -XG_ERR_BAD_DECOMP;
    subs[0].p[0] = s[rel[1]]; subs[0].p[1] = cut[1]; subs[0].p[2] = cut[2]; subs[0].p[3] = cut[3];
    subs[1].p[0] = s[rel[0]]; subs[1].p[1] = s[rel[1]]; subs[1].p[2] = cut[1]; subs[1].p[3] = cut[2];
    subs[2].p[0] = cut[0]; subs[2].p[1] = cut[1]; subs[2].p[2] = cut[2]; subs[2].p[3] = s[rel[0]];
    return 3;
  }
  if (D == 3 && nr == 3) {
    if (nc != 3) return -XG_ERR_BAD_DECOMP;
    subs[0].p[0] = cut[0]; subs[0].p[1] = cut[1]; subs[0].p[2] = cut[2]; subs[0].p[3] = s[rel[2]];
    subs[1].p[0] = s[rel[0]]; subs[1].p[1] = s[rel[1]]; subs[1].p[2] = s[rel[2]]; subs[1].p[3] = cut[1];
    subs[2].p[0] = cut[0]; subs[2].p[1] = cut[1]; subs[2].p[2] = s[rel[0]]; subs[2].p[3] = s[rel[2]];
    return 3;
  }
  return -XG_ERR_BAD_DECOMP;
}

// Decompose with the cut points of the level set (calc_if_points).
template <int D>
__device__ __forceinline__ int decompose(const double* l, int dt, Sub* subs) {
  P3 cut[4];
  const int nc = calc_if_points<D>(l, cut);
  if (nc < 0) return nc;
  return decompose_cuts<D>(l, dt, cut, nc, subs);
}

// Affine element geometry: x(xi) = x_D + F xi with F(:,k) = x_k - x_D.
template <int D>
struct Geo {
  double x0[D];
  double F[D][D];
  double Finv[D][D];
  double det;
};

template <int D>
__device__ __forceinline__ void make_geo(const double (*xv)[3], Geo<D>& g) {
#pragma unroll
  for (int i = 0; i < D; i++) g.x0[i] = xv[D][i];
#pragma unroll
  for (int k = 0; k < D; k++)
#pragma unroll
    for (int i = 0; i < D; i++) g.F[i][k] = xv[k][i] - xv[D][i];
  if (D == 2) {
    double a = g.F[0][0], b = g.F[0][1], c = g.F[1][0], d = g.F[1][1];
    g.det = a * d - b * c;
    double id = 1.0 / g.det;
    g.Finv[0][0] = d * id;
    g.Finv[0][1] = -b * id;
    g.Finv[1][0] = -c * id;
    g.Finv[1][1] = a * id;
  } else {
    const double(*F)[D] = g.F;
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

// |F^-T n_ref| of TransformQuadUntrafoToIRInterface (straightcutrule.cpp:558-578),
// n_ref the normalised constant reference gradient of the P1 level set.
template <int D>
__device__ __forceinline__ double if_factor(const Geo<D>& g, const double* l) {
  double gr[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < D; k++) gr[k] = l[k] - l[D];
  double nn = l2norm3(gr[0], gr[1], gr[2]);
  double inv = 1.0 / nn;
  double nref[3];
#pragma unroll
  for (int k = 0; k < 3; k++) nref[k] = gr[k] * inv;
  double np[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < D; k++) {
    double s = 0;
#pragma unroll
    for (int j = 0; j < D; j++) s += g.Finv[j][k] * nref[j];
    np[k] = s;
  }
  return l2norm3(np[0], np[1], np[2]);
}

// Point q of the plain rule of sub-simplex s (np points) given the base point ip
// (straightcutrule.cpp:80-100).
__device__ __forceinline__ void plain_point(const Sub& s, int np, const double* ip, double* pt) {
  double originweight = 1.0;
  for (int m = 0; m < np - 1; ++m) originweight -= ip[m];
#pragma unroll
  for (int k = 0; k < 3; k++) pt[k] = originweight * s.p[0].c[k];
  for (int m = 0; m < np - 1; ++m)
#pragma unroll
    for (int k = 0; k < 3; k++) pt[k] += ip[m] * s.p[m + 1].c[k];
}

}  // namespace xg

namespace xg {

// ---- space-time ------------------------------------------------------------------
// Nodal time basis on Gauss-Lobatto points (spacetime/SpaceTimeFE.cpp:263-281):
// kt = 0 constant, kt = 1 nodes {0, 1}, kt = 2 nodes {0, 1/2, 1}.
template <typename T>
__host__ __device__ __forceinline__ void time_basis(int kt, T x, T* psi, T* dpsi) {
  if (kt == 0) {
    psi[0] = (T)1;
    dpsi[0] = (T)0;
  } else if (kt == 1) {
    psi[0] = (T)1 - x;
    psi[1] = x;
    dpsi[0] = (T)-1;
    dpsi[1] = (T)1;
  } else {
    psi[0] = ((T)1 - x) * ((T)1 - (T)2 * x);
    psi[1] = (T)4 * x * ((T)1 - x);
    psi[2] = x * ((T)2 * x - (T)1);
    dpsi[0] = (T)4 * x - (T)3;
    dpsi[1] = (T)4 - (T)8 * x;
    dpsi[2] = (T)4 * x - (T)1;
  }
}

// root_finding (cutint/spacetimecutrule.cpp:8-48) for time orders 0..2
__device__ __forceinline__ int time_roots(int kt, const double* li, double* roots) {
  if (kt == 0) return 0;
  if (kt == 1) {
    if (d_geq0(li[0]) != d_geq0(li[1])) {
      roots[0] = -li[0] / (li[1] - li[0]);
      return 1;
    }
    return 0;
  }
  const double c = li[0], a = 2 * li[0] + 2 * li[2] - 4. * li[1], b = li[2] - a - c;
  int n = 0;
  if (fabs(a) < 1e-12) {
    const double x = -c / b;
    if (x < 1 && x > 0) roots[n++] = x;
  } else {
    const double w = b * b - 4 * a * c;
    if (fabs(w) < 1e-12) {
      const double x = -b / (2 * a);
      if (x < 1 && x > 0) roots[n++] = x;
    } else {
      const double x1 = (b + sqrt(w)) / (-2.0 * a);
      const double x2 = (b - sqrt(w)) / (-2.0 * a);
      if (x1 < 1 && x1 > 0) roots[n++] = x1;
      if (x2 < 1 && x2 > 0) roots[n++] = x2;
    }
  }
  return n;
}

// sorted time cut points {0, roots..., 1} of an element (at most 2(D+1)+2)
template <int D>
__device__ __forceinline__ int time_cuts(int kt, const double* lst /* (kt+1)*(D+1) */, double* cut) {
  int n = 0;
  cut[n++] = 0.0;
  cut[n++] = 1.0;
  for (int j = 0; j <= D; j++) {
    double li[3], r[2];
    for (int i = 0; i <= kt; i++) li[i] = lst[i * (D + 1) + j];
    const int nr = time_roots(kt, li, r);
    for (int k = 0; k < nr; k++) cut[n++] = r[k];
  }
  // insertion sort (n <= 8)
  for (int i = 1; i < n; i++) {
    const double v = cut[i];
    int j = i - 1;
    while (j >= 0 && cut[j] > v) {
      cut[j + 1] = cut[j];
      j--;
    }
    cut[j + 1] = v;
  }
  return n;
}

// level set at tau with the space-time perturbation (|d| < 1e-14 -> +-1e-14,
// spacetimecutrule.cpp:167-175)
template <int D>
__device__ __forceinline__ void lset_at(int kt, const double* lst, double tau, double* l) {
  double psi[3], dpsi[3];
  time_basis<double>(kt, tau, psi, dpsi);
#pragma unroll
  for (int j = 0; j <= D; j++) {
    double s = 0;
    for (int i = 0; i <= kt; i++) s += lst[i * (D + 1) + j] * psi[i];
    if (fabs(s) < 1e-14) s = d_geq0(s) ? 1e-14 : -1e-14;
    l[j] = s;
  }
}

// trace at a fixed reference time with the InterpolateToP1 perturbation (+1e-14)
template <int D>
__device__ __forceinline__ void lset_trace(int kt, const double* lst, double tau, double* l) {
  double psi[3], dpsi[3];
  time_basis<double>(kt, tau, psi, dpsi);
#pragma unroll
  for (int j = 0; j <= D; j++) {
    double s = 0;
    for (int i = 0; i <= kt; i++) s += lst[i * (D + 1) + j] * psi[i];
    if (fabs(s) < 1e-14) s = 1e-14;
    l[j] = s;
  }
}

}  // namespace xg

// Straight-cut rules on quadrilaterals and hexahedra, host and device.
//
// Follows ngsxfem cutint/straightcutrule.cpp:
//   LevelsetWrapper (multilinear c[i][j][k])        :503-556
//   Quadrilateral::GetVolume / GetPlainIntegrationRule :73-77, 102-128
//   LevelsetCutQuadrilateral                         :206-501
//     HasTopologyChangeAlongXi, Decompose            :206-249
//     GetTensorProductAlongXiIntegrationRule         :250-301 (c = 0.999 bound)
//     the permuted-quad rules                        :303-350
//     GetSufficientCritsQBound, GetExactCritsQBound2D :352-405
//     GetDimensionSwap                               :407-457
//     GetIntegrationRuleAlongXi / Fallback / GetIntegrationRule :459-501
//   LevelsetCutSimplex on the unit segment and on the fallback's sub-simplices
//     (CalcIFPolytopEUsingLset :41-64, Decompose :131-196)
// The reference builds the rule recursively (a hexahedron's tensor-product
// rule builds a quadrilateral rule at every point of its segment rule).  Here
// the recursion is unrolled into fixed levels (hexahedron -> quadrilateral ->
// segment) and every point is handed to a callback (emit(point, weight)):
// nothing is stored, so one thread builds and consumes the rule of one
// element.  A coordinate permutation (the dimension swaps) is a runtime
// argument and the levels are separate (not inlined) functions, so each level
// is compiled once per callback type.
// The operation order matches the CPU statement of the same functions so
// that a translation unit compiled with -fmad=false reproduces its bits.
#pragma once
#include <cmath>

#include "xg_internal.h"

#ifdef __CUDACC__
#define XG_QHD __host__ __device__ __forceinline__
#define XG_QNI __host__ __device__ __noinline__
#else
#define XG_QHD inline
#define XG_QNI inline
#endif

namespace xg {
namespace qc {

enum { SW_ID = 0, SW_X_Y = 1, SW_X_Z = 2, SW_Y_Z = 3, SW_NONE = 4 };
enum { POL_FIRST_ALLOWED = 0, POL_FIND_OPTIMAL = 1, POL_ALWAYS_NONE = 2 };  // utils/ngsxstd.hpp:10
constexpr double kC = 0.999;

// multilinear level set sum_{ijk} c[i][j][k] x^i y^j z^k on the unit box
struct QL {
  double c[2][2][2];
};

XG_QHD void ql_zero(QL& L) {
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < 2; k++) L.c[i][j][k] = 0.;
}
// ET_QUAD vertex values (0,0),(1,0),(1,1),(0,1)
XG_QHD QL ql_quad(const double* v) {
  QL L;
  ql_zero(L);
  L.c[0][0][0] = v[0];
  L.c[1][0][0] = v[1] - L.c[0][0][0];
  L.c[0][1][0] = v[3] - L.c[0][0][0];
  L.c[1][1][0] = v[2] - L.c[1][0][0] - L.c[0][1][0] - L.c[0][0][0];
  return L;
}
// ET_HEX vertex values: the quadrilateral at z = 0, then at z = 1
XG_QHD QL ql_hex(const double* v) {
  QL L;
  ql_zero(L);
  L.c[0][0][0] = v[0];
  L.c[1][0][0] = v[1] - v[0];
  L.c[0][1][0] = v[3] - v[0];
  L.c[0][0][1] = v[4] - v[0];
  L.c[1][1][0] = v[2] - L.c[1][0][0] - L.c[0][1][0] - L.c[0][0][0];
  L.c[1][0][1] = v[5] - L.c[1][0][0] - L.c[0][0][1] - L.c[0][0][0];
  L.c[0][1][1] = v[7] - L.c[0][1][0] - L.c[0][0][1] - L.c[0][0][0];
  L.c[1][1][1] = v[6] - L.c[1][1][0] - L.c[1][0][1] - L.c[0][1][1] - L.c[1][0][0] - L.c[0][1][0] -
                 L.c[0][0][1] - L.c[0][0][0];
  return L;
}

// value: the terms in (i, j, k) order, each c * x^i * y^j * z^k left to right
// (a factor x^0 = 1 leaves the product unchanged)
XG_QHD double ql_val(const QL& L, double x, double y, double z) {
  double v = 0;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < 2; k++) {
        double t = L.c[i][j][k];
        if (i) t = t * x;
        if (j) t = t * y;
        if (k) t = t * z;
        v += t;
      }
  return v;
}

XG_QHD void ql_grad(const QL& L, const double* p, double* g) {
  g[0] = L.c[1][0][0] + L.c[1][1][0] * p[1] + L.c[1][0][1] * p[2] + L.c[1][1][1] * p[1] * p[2];
  g[1] = L.c[0][1][0] + L.c[1][1][0] * p[0] + L.c[0][1][1] * p[2] + L.c[1][1][1] * p[0] * p[2];
  g[2] = L.c[0][0][1] + L.c[0][1][1] * p[1] + L.c[1][0][1] * p[0] + L.c[1][1][1] * p[0] * p[1];
}

// coefficients in permuted coordinates: new coordinate m = old coordinate perm[m]
XG_QHD QL ql_permute(const QL& L, const int* perm) {
  QL R;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < 2; k++) {
        const int idx[3] = {i, j, k};
        int src[3] = {0, 0, 0};
        for (int m = 0; m < 3; m++) src[perm[m]] = idx[m];
        R.c[i][j][k] = L.c[src[0]][src[1]][src[2]];
      }
  return R;
}

XG_QHD double qnorm3(double a, double b, double c) { return sqrt(a * a + b * b + c * c); }

// CheckIfStraightCut with epsilon (straightcutrule.cpp:11-24)
XG_QHD int qcheck(const double* v, int n, double eps) {
  bool haspos = false, hasneg = false;
  for (int i = 0; i < n; i++) {
    if (v[i] > eps) haspos = true;
    if (v[i] < -eps) hasneg = true;
  }
  if ((hasneg && haspos) || (!hasneg && !haspos)) return XG_IF;
  return hasneg ? XG_NEG : XG_POS;
}

struct Pt {
  double x[3];
};

// Emits a point given in permuted coordinates (perm: new coordinate m = old
// coordinate perm[m]; null = identity) in the original ones.
template <class E>
XG_QHD void emit_perm(E& emit, const int* perm, const double* p, double w) {
  if (!perm) {
    emit(p, w);
    return;
  }
  double o[3];
  for (int m = 0; m < 3; m++) o[perm[m]] = p[m];
  emit(o, w);
}

// ---- simplices with general points (the fallback's sub-simplices) -----------------------
XG_QHD double qsimplex_volume(const Pt* p, int np) {
  if (np == 1) return 1;
  if (np == 2) return qnorm3(p[1].x[0] - p[0].x[0], p[1].x[1] - p[0].x[1], p[1].x[2] - p[0].x[2]);
  if (np == 3) {
    double a[3], b[3];
    for (int k = 0; k < 3; k++) {
      a[k] = p[2].x[k] - p[0].x[k];
      b[k] = p[1].x[k] - p[0].x[k];
    }
    return qnorm3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
  }
  double a[3], b[3], c[3];
  for (int k = 0; k < 3; k++) {
    a[k] = p[3].x[k] - p[0].x[k];
    b[k] = p[2].x[k] - p[0].x[k];
    c[k] = p[1].x[k] - p[0].x[k];
  }
  const double det = a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) +
                     a[2] * (b[0] * c[1] - b[1] * c[0]);
  return fabs(det);
}

// SimpleX::GetPlainIntegrationRule (straightcutrule.cpp:80-100)
template <class E>
XG_QNI void qsimplex_plain(const RuleTable* Rp, const Pt* p, int np, int order, E& emit) {
  const RuleTable& R = *Rp;
  const double trafofac = qsimplex_volume(p, np);
  const int d = np - 1, o = clamp_order(order);
  const int off = R.off[d][o], cnt = R.cnt[d][o];
  for (int q = 0; q < cnt; q++) {
    const double* ip = R.x[off + q];
    double originweight = 1.0;
    for (int m = 0; m < np - 1; ++m) originweight -= ip[m];
    double pt[3];
    for (int k = 0; k < 3; k++) pt[k] = originweight * p[0].x[k];
    for (int m = 0; m < np - 1; ++m)
      for (int k = 0; k < 3; k++) pt[k] += ip[m] * p[m + 1].x[k];
    emit(pt, R.w[off + q] * trafofac);
  }
}

XG_QHD Pt qseg_point(const Pt& a, const Pt& b, double la, double lb) {
  const double t = la / (la - lb);
  Pt r;
  for (int k = 0; k < 3; k++) r.x[k] = a.x[k] + t * (b.x[k] - a.x[k]);
  return r;
}

// LevelsetCutSimplex::GetIntegrationRule on a triangle / tetrahedron with
// points s[0..D] and level set values l (CalcIFPolytopEUsingLset, Decompose,
// plain rules).  Returns 0 or an xg error.
template <int D, class E>
XG_QNI int qcut_simplex(const RuleTable* Rp, const Pt* s, const double* l, int dt, int order, E& emit) {
  if (qcheck(l, D + 1, 0.0) != XG_IF) return XG_ERR_PLAIN_CUT;
  Pt c[4];
  int nc = 0;
  for (int i = 0; i <= D; i++)
    for (int j = i + 1; j <= D; j++)
      if ((l[i] >= 0) != (l[j] >= 0)) {
        const double lij[2] = {l[i], l[j]};
        if (qcheck(lij, 2, 0.0) != XG_IF) return XG_ERR_PLAIN_CUT;
        c[nc++] = qseg_point(s[i], s[j], l[i], l[j]);
      }
  Pt sub[3][4];
  int ns = 0, np = D + 1;
  if (dt == XG_IF) {
    np = D;
    if (nc == D) {
      for (int i = 0; i < D; i++) sub[0][i] = c[i];
      ns = 1;
    } else if (D == 3 && nc == 4) {
      sub[0][0] = c[0]; sub[0][1] = c[1]; sub[0][2] = c[3];
      sub[1][0] = c[0]; sub[1][1] = c[2]; sub[1][2] = c[3];
      ns = 2;
    } else {
      return XG_ERR_BAD_DECOMP;
    }
  } else {
    int rel[4], nr = 0;
    for (int i = 0; i <= D; i++)
      if (((dt == XG_POS) && (l[i] >= 0)) || ((dt == XG_NEG) && (l[i] < 0))) rel[nr++] = i;
    if (nr == 1) {
      if (nc != D) return XG_ERR_BAD_DECOMP;
      for (int i = 0; i < nc; i++) sub[0][i] = c[i];
      sub[0][nc] = s[rel[0]];
      ns = 1;
    } else if (nr == 2 && D == 2) {
      sub[0][0] = s[rel[0]]; sub[0][1] = s[rel[1]]; sub[0][2] = c[1];
      sub[1][0] = c[0]; sub[1][1] = c[1]; sub[1][2] = s[rel[0]];
      ns = 2;
    } else if (nr == 2 && D == 3) {
      if (nc != 4) return XG_ERR_BAD_DECOMP;
      sub[0][0] = s[rel[1]]; sub[0][1] = c[1]; sub[0][2] = c[2]; sub[0][3] = c[3];
      sub[1][0] = s[rel[0]]; sub[1][1] = s[rel[1]]; sub[1][2] = c[1]; sub[1][3] = c[2];
      sub[2][0] = c[0]; sub[2][1] = c[1]; sub[2][2] = c[2]; sub[2][3] = s[rel[0]];
      ns = 3;
    } else if (nr == 3 && D == 3) {
      if (nc != 3) return XG_ERR_BAD_DECOMP;
      sub[0][0] = c[0]; sub[0][1] = c[1]; sub[0][2] = c[2]; sub[0][3] = s[rel[2]];
      sub[1][0] = s[rel[0]]; sub[1][1] = s[rel[1]]; sub[1][2] = s[rel[2]]; sub[1][3] = c[1];
      sub[2][0] = c[0]; sub[2][1] = c[1]; sub[2][2] = s[rel[0]]; sub[2][3] = s[rel[2]];
      ns = 3;
    } else {
      return XG_ERR_BAD_DECOMP;
    }
  }
  for (int k = 0; k < ns; k++) qsimplex_plain(Rp, sub[k], np, order, emit);
  return 0;
}

// LevelsetCutSimplex on the unit segment SimpleX(ET_SEGM) = {(1,0,0), (0,0,0)}
// with the values l0 at (1,0,0) and l1 at (0,0,0).  emit(s, w) receives the
// segment coordinate.  Returns 0 or an xg error.
template <class E>
XG_QNI int qcut_segment(const RuleTable* Rp, double l0, double l1, int dt, int order, E& emit) {
  const RuleTable& R = *Rp;
  const double l[2] = {l0, l1};
  if (qcheck(l, 2, 0.0) != XG_IF) return XG_ERR_PLAIN_CUT;
  const Pt p0 = {{1.0, 0.0, 0.0}}, p1 = {{0.0, 0.0, 0.0}};
  const Pt cp = qseg_point(p0, p1, l0, l1);
  const int o = clamp_order(order);
  if (dt == XG_IF) {
    // the cut point as a 0-simplex: the point rule (weight 1) times volume 1
    const int off = R.off[0][o];
    emit(cp.x[0], R.w[off] * 1.0);
    return 0;
  }
  int rel = -1, nr = 0;
  for (int i = 0; i < 2; i++)
    if (((dt == XG_POS) && (l[i] >= 0)) || ((dt == XG_NEG) && (l[i] < 0))) {
      rel = i;
      nr++;
    }
  if (nr != 1) return XG_ERR_BAD_DECOMP;
  const Pt& v = rel == 0 ? p0 : p1;
  const double trafofac = qnorm3(v.x[0] - cp.x[0], v.x[1] - cp.x[1], v.x[2] - cp.x[2]);
  const int off = R.off[1][o], cnt = R.cnt[1][o];
  for (int q = 0; q < cnt; q++) {
    const double ip = R.x[off + q][0];
    const double originweight = 1.0 - ip;
    const double x = originweight * cp.x[0] + ip * v.x[0];
    emit(x, R.w[off + q] * trafofac);
  }
  return 0;
}

// ---- quadrilaterals (2D) ----------------------------------------------------------------
// Quadrilateral::GetPlainIntegrationRule on [x0,x1] x [y0,y1]: the tensor
// product of the segment rule (x outer), points p0 + A ip, weights w * volume.
template <class E>
XG_QNI void quad_plain(const RuleTable* Rp, double x0, double x1, double y0, double y1, int order, const int* perm,
                      E& emit) {
  const RuleTable& R = *Rp;
  const double p0[3] = {x0, y0, 0.0};
  const double a[3] = {x0 - x0, y1 - y0, 0.0 - 0.0}, b[3] = {x1 - x0, y0 - y0, 0.0 - 0.0};  // p3-p0, p1-p0
  const double trafofac =
      qnorm3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
  const double A[3][3] = {{b[0], a[0], 0.0}, {b[1], a[1], 0.0}, {b[2], a[2], 0.0}};
  const int o = clamp_order(order), off = R.off[1][o], n = R.cnt[1][o];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      const double ip[3] = {R.x[off + i][0], R.x[off + j][0], 0.0};
      const double w = R.w[off + i] * R.w[off + j];
      double pt[3];
      for (int r = 0; r < 3; r++) {
        double acc = A[r][0] * ip[0];
        acc += A[r][1] * ip[1];
        acc += A[r][2] * ip[2];
        pt[r] = p0[r] + acc;
      }
      emit_perm(emit, perm, pt, w * trafofac);
    }
}

// interface scaling |grad phi| / |d phi / dx| of the 2D tensor-product rule
XG_QHD int if_scale_2d(const QL& L, const double* ip, double* fac) {
  double g[3];
  ql_grad(L, ip, g);
  const double f = qnorm3(g[0], g[1], g[2]) / fabs(g[0]);
  const double bound = 1. / sqrt(1 - kC * kC);
  if (f != f || f > bound) return XG_ERR_IF_BOUND;
  *fac = f;
  return 0;
}

// GetTensorProductAlongXiIntegrationRule, D = 2, on [x0,x2] x [e0,e1] (xi = y)
template <class E>
XG_QNI int quad_tensor(const RuleTable* Rp, const QL& L, double x0, double x2, double e0, double e1, int dt,
                       int order, const int* perm, E& emit) {
  const RuleTable& R = *Rp;
  const int o = clamp_order(order), off = R.off[1][o], n = R.cnt[1][o];
  for (int a = 0; a < n; a++) {
    const double xi_ast = e0 + R.x[off + a][0] * (e1 - e0);
    const double wa = R.w[off + a];
    const double l1 = ql_val(L, x0, xi_ast, 0.0);
    const double l0 = ql_val(L, x2, xi_ast, 0.0);
    int st = 0;
    auto on_segment = [&](double s, double w2) {
      const double ip[3] = {x0 + s * (x2 - x0), xi_ast, 0.0};
      double fac = 1;
      if (dt == XG_IF) {
        const int e = if_scale_2d(L, ip, &fac);
        if (e) {
          if (!st) st = e;
          return;
        }
      }
      emit_perm(emit, perm, ip, w2 * wa * (e1 - e0) * fac);
    };
    const int e = qcut_segment(Rp, l0, l1, dt, order, on_segment);
    if (e) return e;
    if (st) return st;
  }
  return 0;
}

// the cut values of the xi-edges ((1,2), (0,3) in 2D; (0,4), (1,5), (2,6),
// (3,7) in 3D) inserted into the sorted set {0, 1} of xi (Decompose).  vb, vt:
// the values at the bottom (xi = 0) and top (xi = 1) ends of each edge.
// Returns the number of breakpoints (2 .. ne + 2) and whether any edge is cut.
XG_QHD int xi_breaks(const double* vb, const double* vt, int ne, double* xs, bool* topo) {
  int n = 2;
  xs[0] = 0.0;
  xs[1] = 1.0;
  *topo = false;
  for (int k = 0; k < ne; k++) {
    const double vals[2] = {vt[k], vb[k]};
    if (qcheck(vals, 2, 0.0) != XG_IF) continue;
    *topo = true;
    // the cut point of the unit segment (1,0,0)-(0,0,0): 1 + t (0 - 1)
    const double t = vals[0] / (vals[0] - vals[1]);
    const double x = 1.0 + t * (0.0 - 1.0);
    if (x != x) continue;
    bool dup = false;
    for (int i = 0; i < n; i++) dup |= xs[i] == x;
    if (dup) continue;
    int j = n++;
    while (j > 0 && xs[j - 1] > x) {
      xs[j] = xs[j - 1];
      j--;
    }
    xs[j] = x;
  }
  return n;
}

// GetIntegrationRuleAlongXi on the unit square (xi = y)
template <class E>
XG_QNI int quad_along_xi(const RuleTable* Rp, const QL& L, int dt, int order, const int* perm, E& emit) {
  const double v[4] = {ql_val(L, 0.0, 0.0, 0.0), ql_val(L, 1.0, 0.0, 0.0), ql_val(L, 1.0, 1.0, 0.0),
                       ql_val(L, 0.0, 1.0, 0.0)};
  const int dq = qcheck(v, 4, 0.0);
  if (dq != XG_IF) {
    if (dq == dt) quad_plain(Rp, 0.0, 1.0, 0.0, 1.0, order, perm, emit);
    return 0;
  }
  // xi-edges (1,2) and (0,3): bottom ends p1, p0, top ends p2, p3
  const double vb[2] = {v[1], v[0]}, vt[2] = {v[2], v[3]};
  double xs[4];
  bool topo;
  const int n = xi_breaks(vb, vt, 2, xs, &topo);
  if (!topo) return quad_tensor(Rp, L, 0.0, 1.0, 0.0, 1.0, dt, order, perm, emit);
  for (int i = 0; i + 1 < n; i++) {
    const double e0 = xs[i], e1 = xs[i + 1];
    const double sv[4] = {ql_val(L, 0.0, e0, 0.0), ql_val(L, 1.0, e0, 0.0), ql_val(L, 1.0, e1, 0.0),
                          ql_val(L, 0.0, e1, 0.0)};
    const int d = qcheck(sv, 4, 1e-15);
    if (d == XG_IF) {
      const int e = quad_tensor(Rp, L, 0.0, 1.0, e0, e1, dt, order, perm, emit);
      if (e) return e;
    } else if (d == dt) {
      quad_plain(Rp, 0.0, 1.0, e0, e1, order, perm, emit);
    }
  }
  return 0;
}

// the fallback: triangles {0,1,3}, {2,1,3} of the unit square with the
// perturbed values of update_initial_coefs
template <class E>
XG_QNI int quad_fallback(const RuleTable* Rp, const QL& L, int dt, int order, E& emit) {
  const Pt c[4] = {{{0.0, 0.0, 0.0}}, {{1.0, 0.0, 0.0}}, {{1.0, 1.0, 0.0}}, {{0.0, 1.0, 0.0}}};
  const int tri[2][3] = {{0, 1, 3}, {2, 1, 3}};
  for (int t = 0; t < 2; t++) {
    Pt s[3];
    double l[3];
    for (int i = 0; i < 3; i++) {
      s[i] = c[tri[t][i]];
      const double d = ql_val(L, s[i].x[0], s[i].x[1], s[i].x[2]);
      l[i] = fabs(d) > 1e-14 ? d : 1e-14;
    }
    const int ds = qcheck(l, 3, 0.0);
    if (ds != XG_IF && ds == dt) {
      qsimplex_plain(Rp, s, 3, order, emit);
    } else if (ds == XG_IF) {
      const int e = qcut_simplex<2>(Rp, s, l, dt, order, emit);
      if (e) return e;
    }
  }
  return 0;
}

// GetExactCritsQBound2D and the 2D branch of GetDimensionSwap
XG_QHD int quad_swap(const QL& L, int pol, bool consider) {
  if (pol == POL_ALWAYS_NONE) return SW_NONE;
  if (!consider) return SW_ID;
  bool allow[2] = {true, true};
  double h_root = -L.c[1][0][0] / L.c[1][1][0];
  if ((h_root > 0) && (h_root < 1)) allow[1] = false;
  h_root = -L.c[0][1][0] / L.c[1][1][0];
  if ((h_root > 0) && (h_root < 1)) allow[0] = false;
  double qm[2] = {0, 0};
  const double cs[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}};
  for (int k = 0; k < 4; k++) {
    double g[3];
    ql_grad(L, cs[k], g);
    const double q_y = fabs(g[1]) / qnorm3(g[0], g[1], g[2]);
    const double q_x = fabs(g[0]) / qnorm3(g[0], g[1], g[2]);
    if (q_y > qm[1]) qm[1] = q_y;
    if (q_x > qm[0]) qm[0] = q_x;
  }
  for (int i = 0; i < 2; i++)
    if (!allow[i]) qm[i] = 2;
  if (pol == POL_FIRST_ALLOWED) {
    if (qm[1] < kC) return SW_ID;
    if (qm[0] < kC) return SW_X_Y;
    return SW_NONE;
  }
  if ((qm[0] < kC) && (qm[1] < kC)) return qm[1] <= qm[0] ? SW_ID : SW_X_Y;
  if (qm[1] < kC) return SW_ID;
  if (qm[0] < kC) return SW_X_Y;
  return SW_NONE;
}

// LevelsetCutQuadrilateral::GetIntegrationRule on the unit square
template <class E>
XG_QNI int quad_rule(const RuleTable* Rp, const QL& L, int dt, int order, int pol, E& emit) {
  const int sw = quad_swap(L, pol, true);
  if (sw == SW_ID) return quad_along_xi(Rp, L, dt, order, (const int*)nullptr, emit);
  if (sw == SW_X_Y) {
    const int perm[3] = {1, 0, 2};
    return quad_along_xi(Rp, ql_permute(L, perm), dt, order, perm, emit);
  }
  return quad_fallback(Rp, L, dt, order, emit);
}

// ---- hexahedra (3D) ---------------------------------------------------------------------
// Quadrilateral::GetPlainIntegrationRule on [x0,x1] x [y0,y1] x [z0,z1]
// (x outermost, z innermost).
template <class E>
XG_QNI void hex_plain(const RuleTable* Rp, double x0, double x1, double y0, double y1, double z0, double z1, int order,
                      const int* perm, E& emit) {
  const RuleTable& R = *Rp;
  const double p0[3] = {x0, y0, z0};
  const double a[3] = {x0 - x0, y0 - y0, z1 - z0};  // p4 - p0
  const double b[3] = {x0 - x0, y1 - y0, z0 - z0};  // p3 - p0
  const double c[3] = {x1 - x0, y0 - y0, z0 - z0};  // p1 - p0
  const double det = a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) +
                     a[2] * (b[0] * c[1] - b[1] * c[0]);
  const double trafofac = fabs(det);
  const double A[3][3] = {{c[0], b[0], a[0]}, {c[1], b[1], a[1]}, {c[2], b[2], a[2]}};
  const int o = clamp_order(order), off = R.off[1][o], n = R.cnt[1][o];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) {
        const double ip[3] = {R.x[off + i][0], R.x[off + j][0], R.x[off + k][0]};
        const double w = R.w[off + i] * R.w[off + j] * R.w[off + k];
        double pt[3];
        for (int r = 0; r < 3; r++) {
          double acc = A[r][0] * ip[0];
          acc += A[r][1] * ip[1];
          acc += A[r][2] * ip[2];
          pt[r] = p0[r] + acc;
        }
        emit_perm(emit, perm, pt, w * trafofac);
      }
}

// GetTensorProductAlongXiIntegrationRule, D = 3, on [x0,x2] x [y0,y2] x [e0,e1]
// (xi = z): at every point of the segment rule the quadrilateral rule of the
// slice (its own level set, dimension swap and fallback included).
template <class E>
XG_QNI int hex_tensor(const RuleTable* Rp, const QL& L, double x0, double x2, double y0, double y2, double e0,
                      double e1, int dt, int order, int pol, const int* perm, E& emit) {
  const RuleTable& R = *Rp;
  const int o = clamp_order(order), off = R.off[1][o], n = R.cnt[1][o];
  const double bound = 1. / sqrt(1 - kC * kC);
  for (int a = 0; a < n; a++) {
    const double xi_ast = e0 + R.x[off + a][0] * (e1 - e0);
    const double wa = R.w[off + a];
    const double lp[4] = {ql_val(L, x0, y0, xi_ast), ql_val(L, x2, y0, xi_ast), ql_val(L, x2, y2, xi_ast),
                          ql_val(L, x0, y2, xi_ast)};
    const QL child = ql_quad(lp);
    int st = 0;
    auto on_slice = [&](const double* p2, double w2) {
      const double ip[3] = {x0 + p2[0] * (x2 - x0), y0 + p2[1] * (y2 - y0), xi_ast};
      double fac = 1;
      if (dt == XG_IF) {
        double g[3];
        ql_grad(L, ip, g);
        fac = qnorm3(g[0], g[1], g[2]) / sqrt(g[0] * g[0] + g[1] * g[1]);
        if (fac != fac || fac > bound) {
          if (!st) st = XG_ERR_IF_BOUND;
          return;
        }
      }
      emit_perm(emit, perm, ip, w2 * wa * (e1 - e0) * fac);
    };
    const int e = quad_rule(Rp, child, dt, order, pol, on_slice);
    if (e) return e;
    if (st) return st;
  }
  return 0;
}

// GetIntegrationRuleAlongXi on the unit cube (xi = z)
template <class E>
XG_QNI int hex_along_xi(const RuleTable* Rp, const QL& L, int dt, int order, int pol, const int* perm, E& emit) {
  const double cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  double v[8];
  for (int k = 0; k < 8; k++) v[k] = ql_val(L, cx[k], cy[k], cz[k]);
  const int dq = qcheck(v, 8, 0.0);
  if (dq != XG_IF) {
    if (dq == dt) hex_plain(Rp, 0.0, 1.0, 0.0, 1.0, 0.0, 1.0, order, perm, emit);
    return 0;
  }
  // xi-edges (0,4), (1,5), (2,6), (3,7)
  const double vb[4] = {v[0], v[1], v[2], v[3]}, vt[4] = {v[4], v[5], v[6], v[7]};
  double xs[6];
  bool topo;
  const int n = xi_breaks(vb, vt, 4, xs, &topo);
  if (!topo) return hex_tensor(Rp, L, 0.0, 1.0, 0.0, 1.0, 0.0, 1.0, dt, order, pol, perm, emit);
  for (int i = 0; i + 1 < n; i++) {
    const double e0 = xs[i], e1 = xs[i + 1];
    double sv[8];
    for (int k = 0; k < 8; k++) sv[k] = ql_val(L, cx[k], cy[k], cz[k] ? e1 : e0);
    const int d = qcheck(sv, 8, 1e-15);
    if (d == XG_IF) {
      const int e = hex_tensor(Rp, L, 0.0, 1.0, 0.0, 1.0, e0, e1, dt, order, pol, perm, emit);
      if (e) return e;
    } else if (d == dt) {
      hex_plain(Rp, 0.0, 1.0, 0.0, 1.0, e0, e1, order, perm, emit);
    }
  }
  return 0;
}

// the fallback: 6 tetrahedra of the unit cube
template <class E>
XG_QNI int hex_fallback(const RuleTable* Rp, const QL& L, int dt, int order, E& emit) {
  const double cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  const int tet[6][4] = {{3, 0, 1, 5}, {3, 1, 2, 5}, {3, 5, 2, 6}, {4, 5, 0, 3}, {4, 7, 5, 3}, {7, 6, 5, 3}};
  for (int t = 0; t < 6; t++) {
    Pt s[4];
    double l[4];
    for (int i = 0; i < 4; i++) {
      const int c = tet[t][i];
      s[i] = Pt{{cx[c], cy[c], cz[c]}};
      const double d = ql_val(L, s[i].x[0], s[i].x[1], s[i].x[2]);
      l[i] = fabs(d) > 1e-14 ? d : 1e-14;
    }
    const int ds = qcheck(l, 4, 0.0);
    if (ds != XG_IF && ds == dt) {
      qsimplex_plain(Rp, s, 4, order, emit);
    } else if (ds == XG_IF) {
      const int e = qcut_simplex<3>(Rp, s, l, dt, order, emit);
      if (e) return e;
    }
  }
  return 0;
}

// GetSufficientCritsQBound and the 3D branch of GetDimensionSwap; returns the
// swap or -(xg error) for a NaN bound
XG_QHD int hex_swap(const QL& L, int pol) {
  if (pol == POL_ALWAYS_NONE) return SW_NONE;
  const double cs[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  double g[8][3];
  for (int k = 0; k < 8; k++) ql_grad(L, cs[k], g[k]);
  double Vsq = 0;
  for (int d = 0; d < 3; d++) {
    double mx = 0;
    for (int k = 0; k < 8; k++) {
      const double v = g[k][d] * g[k][d];
      if (v > mx) mx = v;
    }
    Vsq += mx;
  }
  const double V = sqrt(Vsq);
  double qm[3] = {0, 0, 0};
  for (int k = 0; k < 8; k++)
    for (int d = 0; d < 3; d++) {
      const double q_est = V * V / (V * V - g[k][d] * g[k][d]);
      if (q_est > qm[d]) qm[d] = q_est;
    }
  for (int d = 0; d < 3; d++) {
    qm[d] = sqrt(1 - 1 / qm[d]);
    if (qm[d] != qm[d]) return -XG_ERR_NONFINITE;
  }
  if (pol == POL_FIRST_ALLOWED) {
    if (qm[2] < kC) return SW_ID;
    if (qm[1] < kC) return SW_Y_Z;
    if (qm[0] < kC) return SW_X_Z;
    return SW_NONE;
  }
  int md = 0;  // std::min_element with v1 <= v2: the last of equal minima
  for (int d = 1; d < 3; d++)
    if (qm[d] <= qm[md]) md = d;
  if (qm[md] < kC) return md == 0 ? SW_X_Z : (md == 1 ? SW_Y_Z : SW_ID);
  return SW_NONE;
}

// LevelsetCutQuadrilateral::GetIntegrationRule on the unit cube
template <class E>
XG_QNI int hex_rule(const RuleTable* Rp, const QL& L, int dt, int order, int pol, E& emit) {
  const int sw = hex_swap(L, pol);
  if (sw < 0) return -sw;
  if (sw == SW_ID) return hex_along_xi(Rp, L, dt, order, pol, (const int*)nullptr, emit);
  if (sw == SW_Y_Z || sw == SW_X_Z) {
    const int pyz[3] = {0, 2, 1}, pxz[3] = {2, 1, 0};
    const int* perm = sw == SW_Y_Z ? pyz : pxz;
    return hex_along_xi(Rp, ql_permute(L, perm), dt, order, pol, perm, emit);
  }
  return hex_fallback(Rp, L, dt, order, emit);
}

}  // namespace qc
}  // namespace xg

namespace xg {
namespace qc {

// StraightCutIntegrationRuleUntransformed (straightcutrule.cpp:814-879) for
// ET_QUAD (D = 2, 4 vertex values) and ET_HEX (D = 3, 8 values).  Emits the
// rule on the unit box; returns 0, -1 for "no rule" (an uncut element of the
// other domain) or an xg error.
template <int D, class E>
XG_QHD int tp_cut_rule(const RuleTable* Rp, const double* vals, int dt, int order, int pol, E& emit) {
  constexpr int NV = D == 2 ? 4 : 8;
  const int dom = qcheck(vals, NV, 0.0);
  if (dom != XG_IF && dom != dt) return -1;
  if constexpr (D == 2) {
    if (dom == XG_IF) return quad_rule(Rp, ql_quad(vals), dt, order, pol, emit);
    quad_plain(Rp, 0.0, 1.0, 0.0, 1.0, order, (const int*)nullptr, emit);
  } else {
    if (dom == XG_IF) return hex_rule(Rp, ql_hex(vals), dt, order, pol, emit);
    hex_plain(Rp, 0.0, 1.0, 0.0, 1.0, 0.0, 1.0, order, (const int*)nullptr, emit);
  }
  return 0;
}

}  // namespace qc
}  // namespace xg

// Cut rules on quadrilateral and hexahedral meshes (rule export; Integrate
// is in xg_quad_int.cu).
//
// The rule on the reference box is LevelsetCutQuadrilateral
// (cutint/straightcutrule.cpp:206-501, unrolled in xg_quadcut.cuh); the
// element map is the bilinear (trilinear) interpolation of the vertices, so
// |det J| and the interface factor |J^-T n_ref| vary over the element and are
// evaluated per point (TransformQuadUntrafoToIRInterface,
// straightcutrule.cpp:558-578).  One thread builds the rule of one element;
// a point is written as it is produced (callback).
// Compiled with -fmad=false: points and weights follow the CPU statement
// operation by operation.
#include <cuda_runtime.h>

#include <algorithm>

#include "xg_internal.h"
#include "xg_quadcut.cuh"

namespace xg {

// the rule functions are separate (not inlined) device functions that read the
// table through a pointer: a copy in global memory (generic addressing)
static __device__ RuleTable g_qrules;

int upload_rules_quad() {
  XG_CUDA(cudaMemcpyToSymbol(g_qrules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

// bilinear / trilinear map of the unit box: x = sum_v N_v x_v, J = dx/dxi
template <int D>
__device__ __forceinline__ void tp_map(const double (*xv)[3], const double* xi, double* x, double J[3][3]) {
  constexpr int NV = 1 << D;
  for (int i = 0; i < 3; i++) {
    x[i] = 0;
    for (int k = 0; k < 3; k++) J[i][k] = 0;
  }
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const int cx = (v == 1 || v == 2 || v == 5 || v == 6), cy = (v & 3) >= 2, cz = v >= 4;
    const double fx = cx ? xi[0] : 1 - xi[0], gx = cx ? 1.0 : -1.0;
    const double fy = cy ? xi[1] : 1 - xi[1], gy = cy ? 1.0 : -1.0;
    const double fz = D == 3 ? (cz ? xi[2] : 1 - xi[2]) : 1.0, gz = cz ? 1.0 : -1.0;
    const double N = fx * fy * fz;
    const double dN[3] = {gx * fy * fz, fx * gy * fz, fx * fy * gz};
#pragma unroll
    for (int i = 0; i < D; i++) {
      x[i] += N * xv[v][i];
#pragma unroll
      for (int k = 0; k < D; k++) J[i][k] += xv[v][i] * dN[k];
    }
  }
}

template <int D>
__device__ __forceinline__ double tp_det_inv(const double J[3][3], double Ji[3][3]) {
  if (D == 2) {
    const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double id = 1.0 / det;
    Ji[0][0] = J[1][1] * id;
    Ji[0][1] = -J[0][1] * id;
    Ji[1][0] = -J[1][0] * id;
    Ji[1][1] = J[0][0] * id;
    return det;
  }
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  const double id = 1.0 / det;
  Ji[0][0] = c00 * id;
  Ji[1][0] = c01 * id;
  Ji[2][0] = c02 * id;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  return det;
}

// |J^-T n_ref|, n_ref the normalised gradient of the multilinear level set at xi
template <int D>
__device__ __forceinline__ double tp_if_factor(const qc::QL& L, const double* xi, const double Ji[3][3]) {
  double g[3];
  qc::ql_grad(L, xi, g);
  const double nn = qc::qnorm3(g[0], g[1], g[2]);
  double nr[3];
  for (int k = 0; k < 3; k++) nr[k] = g[k] / nn;
  double np[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < D; k++) {
    double s = 0;
#pragma unroll
    for (int j = 0; j < D; j++) s += Ji[j][k] * nr[j];
    np[k] = s;
  }
  return qc::qnorm3(np[0], np[1], np[2]);
}

template <int D>
__device__ __forceinline__ void gather(int ne, const int32_t* __restrict__ elv, const double* __restrict__ xyz, int nv,
                                       const double* __restrict__ lset, int e, double* l, double (*xv)[3]) {
  constexpr int NV = 1 << D;
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const int vid = elv[(int64_t)v * ne + e];
    l[v] = lset[vid];
#pragma unroll
    for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
  }
}

}  // namespace

// StraightCutIntegrationRule for listed quadrilaterals / hexahedra: rule
// points on the unit box, weights with the interface factor of the element
// map for IF.  counts[i] = -1 for "no rule" (straightcutrule.cpp:669-676 and
// the empty cut rule of :627-628).
template <int D>
__global__ void __launch_bounds__(128) k_quad_rules(int ne, const int32_t* __restrict__ elv,
                                                    const double* __restrict__ xyz, int nv,
                                                    const double* __restrict__ lset, const int32_t* __restrict__ elems,
                                                    int n, int dt, int order, int pol, int max_pts, int32_t* counts,
                                                    double* pts, double* wts, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int e = elems[i];
  if (e < 0 || e >= ne) {
    set_err(err, XG_ERR_ARG);
    counts[i] = 0;
    return;
  }
  constexpr int NV = 1 << D;
  double l[NV], xv[NV][3];
  gather<D>(ne, elv, xyz, nv, lset, e, l, xv);
  const bool cut = qc::qcheck(l, NV, 0.0) == XG_IF;
  const qc::QL L = D == 2 ? qc::ql_quad(l) : qc::ql_hex(l);
  double* P = pts + (int64_t)i * max_pts * 3;
  double* W = wts + (int64_t)i * max_pts;
  int k = 0;
  auto emit = [&](const double* p, double w) {
    if (k < max_pts) {
      if (cut && dt == XG_IF) {
        double x[3], J[3][3], Ji[3][3];
        tp_map<D>(xv, p, x, J);
        tp_det_inv<D>(J, Ji);
        w = w * tp_if_factor<D>(L, p, Ji);
      }
      for (int c = 0; c < 3; c++) P[3 * k + c] = p[c];
      W[k] = w;
    }
    k++;
  };
  const int st = qc::tp_cut_rule<D>(&g_qrules, l, dt, order, pol, emit);
  if (st == -1) {
    counts[i] = -1;
    return;
  }
  if (st > 0 || k > max_pts) {
    set_err(err, st > 0 ? st : XG_ERR_CAPACITY);
    counts[i] = 0;
    return;
  }
  counts[i] = (cut && k == 0) ? -1 : k;
}

// CutInformation::Update (xfem/cutinfo.cpp:61-132) on quadrilaterals /
// hexahedra: the weights of the order-0 NEG and POS rules give the part
// volumes, ratio = NEG / (NEG + POS), the domain type and the combined-domain
// bits (rows: CDOM values; bits set with atomic OR on cleared words).
template <int D>
__global__ void __launch_bounds__(128) k_quad_cutinfo(int ne, const int32_t* __restrict__ elv,
                                                      const double* __restrict__ xyz, int nv,
                                                      const double* __restrict__ lset, int pol, uint8_t* __restrict__ dom,
                                                      double* __restrict__ ratio, unsigned long long* bits, int64_t nw,
                                                      int* err) {
  constexpr int NV = 1 << D;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double l[NV], xv[NV][3];
    gather<D>(ne, elv, xyz, nv, lset, (int)e, l, xv);
    double part[2] = {0.0, 0.0};  // [NEG, POS]
    for (int np : {XG_POS, XG_NEG}) {
      auto emit = [&](const double*, double w) { part[np] += w; };
      const int st = qc::tp_cut_rule<D>(&g_qrules, l, np, 0, pol, emit);
      if (st > 0) set_err(err, st);
    }
    ratio[e] = part[XG_NEG] / (part[XG_NEG] + part[XG_POS]);
    const int d = part[XG_NEG] > 0.0 ? (part[XG_POS] > 0.0 ? XG_IF : XG_NEG) : XG_POS;
    dom[e] = (uint8_t)d;
    const unsigned long long bit = 1ull << (e & 63);
    const int64_t w = e >> 6;
    // NEG: NEG, UNCUT, HASNEG, ANY; POS: POS, UNCUT, HASPOS, ANY; IF: IF, HASNEG, HASPOS, ANY
    const int r0 = d == XG_NEG ? XG_CDOM_NEG : (d == XG_POS ? XG_CDOM_POS : XG_CDOM_IF);
    const int r1 = d == XG_IF ? XG_CDOM_HASNEG : XG_CDOM_UNCUT;
    const int r2 = d == XG_NEG ? XG_CDOM_HASNEG : XG_CDOM_HASPOS;
    atomicOr(bits + r0 * nw + w, bit);
    atomicOr(bits + r1 * nw + w, bit);
    atomicOr(bits + r2 * nw + w, bit);
    atomicOr(bits + XG_CDOM_ANY * nw + w, bit);
  }
}

int quad_cutinfo(xg_mesh* m, const double* d_lset, uint8_t* d_dom, double* d_ratio, uint64_t* d_bits, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nw = ((int64_t)m->ne + 63) / 64;
  XG_CUDA(cudaMemsetAsync(d_bits, 0, sizeof(uint64_t) * 8 * nw, s));
  const unsigned nb = 152 * 8;
  if (m->dim == 2)
    k_quad_cutinfo<2><<<nb, 128, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, qc::POL_FIND_OPTIMAL, d_dom, d_ratio,
                                         (unsigned long long*)d_bits, nw, m->d_err);
  else
    k_quad_cutinfo<3><<<nb, 128, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, qc::POL_FIND_OPTIMAL, d_dom, d_ratio,
                                         (unsigned long long*)d_bits, nw, m->d_err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_quad_cutinfo");
  return XG_OK;
}

// most points a rule of (dim, dt, order) can have: up to 3 (2D) / 5 (3D)
// slabs between the xi breakpoints, each a tensor product over the segment
// rule, or the simplex fallback (2 triangles / 6 tetrahedra, up to 3
// sub-simplices each)
int quad_rule_capacity(int dim, int dt, int order) {
  const RuleTable& R = host_rules();
  const int o = clamp_order(order);
  const int n1 = R.cnt[1][o], n2 = R.cnt[2][o], n3 = R.cnt[3][o];
  const int slice = dt == XG_IF ? 1 : n1;
  const int cap2 = std::max(3 * n1 * std::max(n1, slice), 2 * std::max(2 * n2, n1));
  if (dim == 2) return cap2;
  return std::max(5 * n1 * std::max(n1 * n1, cap2), 6 * std::max(3 * n3, 2 * n2));
}

static int launch_check_q(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return XG_OK;
}

static inline unsigned nblk_q(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

int quad_cut_rules(xg_mesh* m, const double* d_lset, const int32_t* d_elems, int32_t n, int dt, int order, int pol,
                   int32_t max_pts, int32_t* d_counts, double* d_pts, double* d_wts, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (m->dim == 2)
    k_quad_rules<2><<<nblk_q(n, 128), 128, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, d_elems, n, dt, order,
                                                   pol, max_pts, d_counts, d_pts, d_wts, m->d_err);
  else
    k_quad_rules<3><<<nblk_q(n, 128), 128, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, d_elems, n, dt, order,
                                                   pol, max_pts, d_counts, d_pts, d_wts, m->d_err);
  return launch_check_q("k_quad_rules");
}

}  // namespace xg

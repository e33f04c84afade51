// Subdivision cut rules on the GPU (the rule code is xg_subdiv.cuh):
//   xg_integrate_subdiv     Integrate(f * dCut(lset_h, dt, subdivlvl=L)) for a
//                           level set of order 1..3 given as H1 coefficients
//                           (the reference's CutIntegrationRule path for
//                           level sets that are not P1, cutint/xintegration.cpp:
//                           102-116, 1626-1754)
//   xg_subdiv_moments_tet   per element the NEG moments (monomials of degree
//                           <= 4 in reference coordinates) of a P2 level set
//                           given by its values at the vertices and edge
//                           midpoints of the reference tetrahedron
// One thread per element walks the element's refinement tree; the integral
// is summed per thread, per block in a fixed tree and over the blocks in
// order, so repeated calls give the same bits.
#include <cuda_runtime.h>

#include <cstdint>

#include "xg_internal.h"
#include "xg_subdiv.cuh"

namespace xg {

static __device__ RuleTable g_sd_rules;  // the rule code reads its table by pointer

int upload_rules_subdiv() {
  XG_CUDA(cudaMemcpyToSymbol(g_sd_rules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

constexpr int kSdThreads = 128;
constexpr int kSdBlocks = 152 * 8;

__device__ __forceinline__ bool sd_bit(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

__device__ __forceinline__ double sd_ipow(double x, int e) {
  double r = 1.0;
  for (int k = 0; k < e; k++) r *= x;
  return r;
}

template <int D, int K>
__global__ void __launch_bounds__(kSdThreads, 3) k_subdiv_integrate(int ne, int nv, const int32_t* __restrict__ elv,
                                                                     const double* __restrict__ xyz,
                                                                     const int32_t* __restrict__ el_dofs,
                                                                     const double* __restrict__ coefs, int dt,
                                                                     int order, int levels, int ex, int ey, int ez,
                                                                     const uint64_t* __restrict__ defined_on,
                                                                     double* __restrict__ block_sums, int* err) {
  __shared__ double red[kSdThreads];
  constexpr int N = ndof_el(D, K);
  double acc = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    if (defined_on && !sd_bit(defined_on, e)) continue;
    sd::Elem<D, K> el;
    int gv[4] = {0, 0, 0, 0};
    double xv[4][3];
    for (int v = 0; v <= D; v++) {
      gv[v] = elv[(int64_t)v * ne + e];
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + gv[v]] : 0.0;
    }
    for (int r = 0; r < 3; r++) {
      el.x0[r] = xv[D][r];
      for (int c = 0; c < 3; c++) el.F[r][c] = c < D ? xv[c][r] - xv[D][r] : 0.0;
    }
    for (int i = 0; i < N; i++) {
      el.coef[i] = coefs[el_dofs[(int64_t)i * ne + e]];
      el.desc[i] = fn_desc<D, K>(i, gv);
    }
    auto emit = [&](const double* x, double w) {
      acc += w * sd_ipow(x[0], ex) * sd_ipow(x[1], ey) * (D == 3 ? sd_ipow(x[2], ez) : 1.0);
    };
    const int st = sd::element_rule<D, K>(&g_sd_rules, el, dt, order, levels, emit);
    if (st) set_err(err, st);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kSdThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
}

__global__ void k_sd_sum(const double* v, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += v[i];
    out[0] = s;
  }
}

// the 35 NEG moments x^a y^b z^c (a + b + c <= 4, by degree, then a, then b
// descending) of each reference tetrahedron, thread per element (a warp per
// element, with the lattice checks split over its lanes and every lane
// walking the tree, measured about half as fast: the tree walk and the rule
// points, not the checks, are the work)
__global__ void __launch_bounds__(kSdThreads, 3) k_subdiv_moments(int64_t n, const double* __restrict__ vals10,
                                                                  int levels, double* __restrict__ out35,
                                                                  const int32_t* __restrict__ list,
                                                                  const int32_t* __restrict__ count, int* err) {
  const int E[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  const int64_t items = list ? (int64_t)*count : n;
  for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < items;
       it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = list ? (int64_t)list[it] : it;
    if (e < 0 || e >= n) {
      set_err(err, XG_ERR_ARG);
      continue;
    }
    sd::Elem<3, 2> el;
    const int gv[4] = {0, 1, 2, 3};
    for (int r = 0; r < 3; r++) {
      el.x0[r] = 0.0;
      for (int c = 0; c < 3; c++) el.F[r][c] = r == c ? 1.0 : 0.0;
    }
    const double* p = vals10 + e * 10;
    // P2 nodal values -> the H1 coefficients: vertex values, 4 p(mid) - 2 (p_a + p_b)
    for (int i = 0; i < 4; i++) el.coef[i] = p[i];
    for (int j = 0; j < 6; j++) el.coef[4 + j] = 4.0 * p[4 + j] - 2.0 * (p[E[j][0]] + p[E[j][1]]);
    for (int i = 0; i < 10; i++) el.desc[i] = fn_desc<3, 2>(i, gv);
    double m[35];
    for (int k = 0; k < 35; k++) m[k] = 0.0;
    auto emit = [&](const double* x, double w) {
      const double px[5] = {1, x[0], x[0] * x[0], x[0] * x[0] * x[0], x[0] * x[0] * x[0] * x[0]};
      const double py[5] = {1, x[1], x[1] * x[1], x[1] * x[1] * x[1], x[1] * x[1] * x[1] * x[1]};
      const double pz[5] = {1, x[2], x[2] * x[2], x[2] * x[2] * x[2], x[2] * x[2] * x[2] * x[2]};
      int k = 0;
      for (int t = 0; t <= 4; t++)
        for (int a = t; a >= 0; a--)
          for (int b = t - a; b >= 0; b--) m[k++] += w * px[a] * py[b] * pz[t - a - b];
    };
    const int st = sd::element_rule<3, 2>(&g_sd_rules, el, XG_NEG, 4, levels, emit);
    if (st) set_err(err, st);
    for (int k = 0; k < 35; k++) out35[e * 35 + k] = m[k];
  }
}

template <int D, int K>
void launch_int(xg_space* sp, const double* coefs, int dt, int order, int levels, int ex, int ey, int ez,
                const uint64_t* defined_on, double* bs, cudaStream_t s) {
  xg_mesh* m = sp->mesh;
  k_subdiv_integrate<D, K><<<kSdBlocks, kSdThreads, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, sp->d_el_dofs, coefs,
                                                           dt, order, levels, ex, ey, ez, defined_on, bs, m->d_err);
}

}  // namespace

int subdiv_moments_launch(const double* d_vals10, int64_t n, int levels, double* d_out35, const int32_t* d_list,
                          const int32_t* d_count, int* d_err, cudaStream_t s) {
  const int64_t blocks = (n + kSdThreads - 1) / kSdThreads;
  k_subdiv_moments<<<(unsigned)(blocks < kSdBlocks ? (blocks > 0 ? blocks : 1) : kSdBlocks), kSdThreads, 0, s>>>(
      n, d_vals10, levels, d_out35, d_list, d_count, d_err);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_subdiv_moments_tet");
}

}  // namespace xg

using namespace xg;

extern "C" {

int xg_integrate_subdiv(xg_space* sp, const double* d_lset_coefs, int dt, int order, int subdivlvl, int ex, int ey,
                        int ez, const uint64_t* d_defined_on, double* d_result, void* stream) {
  if (!sp || !d_lset_coefs || !d_result || dt < 0 || dt > 2 || order < 0 || order > kMaxOrder || ex < 0 ||
      ey < 0 || ez < 0 || subdivlvl < 0 || subdivlvl > sd::kMaxLevels) {
    set_last_error("xg_integrate_subdiv: bad arguments (subdivlvl 0..6, order 0..8)");
    return XG_ERR_ARG;
  }
  if (sp->kt >= 0 || sp->mesh->tensor || sp->ndof != sp->ndof_s || sp->mesh->dim < 2) {
    set_last_error("xg_integrate_subdiv: the level set lives in an H1 space on a simplex mesh");
    return XG_ERR_UNSUPPORTED;
  }
  int st = ensure_device_rules();
  if (st) return st;
  xg_mesh* m = sp->mesh;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t need = kSdBlocks * sizeof(double);
  if (m->scratch_bytes < need) {
    cudaFree(m->d_scratch);
    m->d_scratch = nullptr;
    m->scratch_bytes = 0;
    XG_CUDA(cudaMalloc(&m->d_scratch, need));
    m->scratch_bytes = need;
  }
  double* bs = (double*)m->d_scratch;
  const int D = m->dim, K = sp->order;
  if (D == 2) {
    if (K == 1) launch_int<2, 1>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
    else if (K == 2) launch_int<2, 2>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
    else launch_int<2, 3>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
  } else {
    if (K == 1) launch_int<3, 1>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
    else if (K == 2) launch_int<3, 2>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
    else launch_int<3, 3>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
  }
  k_sd_sum<<<1, 32, 0, s>>>(bs, kSdBlocks, d_result);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_subdiv_integrate");
}

int xg_subdiv_moments_tet(const double* d_vals10, int64_t n, int subdivlvl, double* d_out35, int* d_err,
                          void* stream) {
  if ((n > 0 && (!d_vals10 || !d_out35)) || n < 0 || subdivlvl < 0 || subdivlvl > sd::kMaxLevels) {
    set_last_error("xg_subdiv_moments_tet: bad arguments (subdivlvl 0..6)");
    return XG_ERR_ARG;
  }
  if (n == 0) return XG_OK;
  int st = ensure_device_rules();
  if (st) return st;
  return subdiv_moments_launch(d_vals10, n, subdivlvl, d_out35, nullptr, nullptr, d_err, (cudaStream_t)stream);
}

}  // extern "C"

// Mesh-level isoparametric integration for P2 level sets on simplex meshes
// (python/lsetcurv.py:281-356 with lsetcurving/projshift.cpp:58-197): the
// per-element steps are xg_isomesh.cuh.  Three launches:
//   k_iso_contrib    thread per element: band test, Newton searches, L2
//                    projection, physical edge contributions J theta;
//   k_iso_average    thread per edge: the contributions of its band elements
//                    summed in element order, divided by their number (the
//                    same order on every run: deterministic);
//   k_iso_integrate  thread per element: the mapped cut rule, fixed-order sums.
// Compiled with -fmad=false (the operation order of the CPU statement).
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "xg_internal.h"
#include "xg_isomesh.cuh"

namespace xg {

static __device__ RuleTable g_isorules;

int upload_rules_isomesh() {
  XG_CUDA(cudaMemcpyToSymbol(g_isorules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

constexpr int kIsoThreads = 128;
constexpr int kIsoBlocks = 152 * 8;

template <int D>
__device__ __forceinline__ void verts_iso(int ne, const int32_t* __restrict__ elv, const double* __restrict__ xyz,
                                          int nv, int e, double (*xv)[3]) {
#pragma unroll
  for (int v = 0; v <= D; v++) {
    const int vid = elv[(int64_t)v * ne + e];
#pragma unroll
    for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
  }
}

__device__ __forceinline__ double ipow_iso(double x, int e) {
  double r = 1.0;
  for (int i = 0; i < e; i++) r *= x;
  return r;
}

}  // namespace

template <int D>
__global__ void __launch_bounds__(kIsoThreads) k_iso_contrib(int ne, const int32_t* __restrict__ elv,
                                                             const double* __restrict__ xyz, int nv,
                                                             const double* __restrict__ p2vals, double threshold,
                                                             double* __restrict__ contrib, uint8_t* __restrict__ band,
                                                             int* nonconv, int* err) {
  constexpr int NE = D == 2 ? 3 : 6, NN = (D + 1) * (D + 2) / 2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double xv[D + 1][3], p2[NN], c[6][3];
    verts_iso<D>(ne, elv, xyz, nv, (int)e, xv);
    for (int i = 0; i < NN; i++) p2[i] = p2vals[e * NN + i];
    bool in_band = false;
    int nc = 0;
    if (!iso::element_contrib<D>(&g_isorules, xv, p2, threshold, c, &in_band, &nc)) {
      set_err(err, XG_ERR_NONFINITE);
      in_band = false;
    }
    if (nc) atomicAdd(nonconv, nc);
    band[e] = in_band ? 1 : 0;
    for (int j = 0; j < NE; j++)
      for (int r = 0; r < 3; r++) contrib[(e * NE + j) * 3 + r] = in_band ? c[j][r] : 0.0;
  }
}

// incidences of edge g: inc[ptr[g] .. ptr[g+1]) = element * 8 + local edge,
// elements ascending
__global__ void __launch_bounds__(kIsoThreads) k_iso_average(int64_t nedges, int nel, const int32_t* __restrict__ ptr,
                                                             const int32_t* __restrict__ inc,
                                                             const double* __restrict__ contrib,
                                                             const uint8_t* __restrict__ band,
                                                             double* __restrict__ gdef) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nedges; g += (int64_t)gridDim.x * blockDim.x) {
    double s[3] = {0.0, 0.0, 0.0}, cnt = 0.0;
    for (int k = ptr[g]; k < ptr[g + 1]; k++) {
      const int e = inc[k] >> 3, j = inc[k] & 7;
      if (!band[e]) continue;
      for (int r = 0; r < 3; r++) s[r] += contrib[((int64_t)e * nel + j) * 3 + r];
      cnt += 1.0;
    }
    for (int r = 0; r < 3; r++) gdef[g * 3 + r] = cnt > 0 ? s[r] / cnt : 0.0;
  }
}

template <int D>
__global__ void __launch_bounds__(kIsoThreads) k_iso_integrate(int ne, const int32_t* __restrict__ elv,
                                                               const double* __restrict__ xyz, int nv,
                                                               const int32_t* __restrict__ el_edges,
                                                               const double* __restrict__ p2vals,
                                                               const double* __restrict__ gdef, int dt, int order,
                                                               int ex, int ey, int ez, double* block_sums, int* err) {
  constexpr int NE = D == 2 ? 3 : 6, NN = (D + 1) * (D + 2) / 2;
  __shared__ double red[kIsoThreads];
  double acc = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double xv[D + 1][3], p2[NN], gl[6][3];
    verts_iso<D>(ne, elv, xyz, nv, (int)e, xv);
    for (int i = 0; i < NN; i++) p2[i] = p2vals[e * NN + i];
    for (int j = 0; j < NE; j++) {
      const int g = el_edges[(int64_t)j * ne + e];
      for (int r = 0; r < 3; r++) gl[j][r] = gdef[(int64_t)g * 3 + r];
    }
    auto emit = [&](const double* x, double w) {
      acc += w * ipow_iso(x[0], ex) * ipow_iso(x[1], ey) * (D == 3 ? ipow_iso(x[2], ez) : 1.0);
    };
    const int st = iso::element_rule<D>(&g_isorules, xv, p2, gl, dt, order, emit);
    if (st) set_err(err, st);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kIsoThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
}

__global__ void k_iso_final(const double* bs, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += bs[i];
    out[0] = s;
  }
}

}  // namespace xg

using namespace xg;

static int iso_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return XG_OK;
}

// edge -> (element, local edge) incidences, elements ascending, built once per mesh
static int iso_incidence(xg_mesh* m) {
  if (m->d_edge_ptr) return XG_OK;
  const int nel = m->dim == 2 ? 3 : 6;
  std::vector<int32_t> ptr((size_t)m->nedges + 1, 0), inc((size_t)m->ne * nel);
  for (size_t i = 0; i < m->h_el_edges.size(); i++) ptr[(size_t)m->h_el_edges[i] + 1]++;
  for (int64_t g = 0; g < m->nedges; g++) ptr[g + 1] += ptr[g];
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
  for (int e = 0; e < m->ne; e++)
    for (int j = 0; j < nel; j++) inc[fill[m->h_el_edges[(size_t)e * nel + j]]++] = e * 8 + j;
  XG_CUDA(cudaMalloc((void**)&m->d_edge_ptr, sizeof(int32_t) * ptr.size()));
  XG_CUDA(cudaMalloc((void**)&m->d_edge_inc, sizeof(int32_t) * inc.size()));
  XG_CUDA(cudaMemcpy(m->d_edge_ptr, ptr.data(), sizeof(int32_t) * ptr.size(), cudaMemcpyHostToDevice));
  XG_CUDA(cudaMemcpy(m->d_edge_inc, inc.data(), sizeof(int32_t) * inc.size(), cudaMemcpyHostToDevice));
  return XG_OK;
}

// the mesh-level deformation alone: d_gdef[edge][3] = the averaged physical
// edge coefficients J theta of the band elements (0 elsewhere)
extern "C" int xg_iso_deformation(xg_mesh* m, const double* d_p2vals, double threshold, double* d_gdef,
                                  int32_t* d_nonconv, void* stream) {
  if (!m || !d_p2vals || !d_gdef || !d_nonconv) return XG_ERR_ARG;
  if (m->tensor) {
    set_last_error("xg_iso_deformation: simplex meshes only");
    return XG_ERR_UNSUPPORTED;
  }
  if (m->ne >= (1 << 28)) return XG_ERR_CAPACITY;
  if (int st = iso_incidence(m)) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int nel = m->dim == 2 ? 3 : 6;
  const size_t n_contrib = (size_t)m->ne * nel * 3;
  const size_t need = sizeof(double) * n_contrib + (size_t)m->ne;
  if (m->iso_bytes < need) {
    cudaFree(m->d_iso);
    m->d_iso = nullptr;
    m->iso_bytes = 0;
    XG_CUDA(cudaMalloc(&m->d_iso, need));
    m->iso_bytes = need;
  }
  double* contrib = (double*)m->d_iso;
  uint8_t* band = (uint8_t*)(contrib + n_contrib);
  XG_CUDA(cudaMemsetAsync(d_nonconv, 0, sizeof(int32_t), s));
  if (m->dim == 2)
    k_iso_contrib<2><<<kIsoBlocks, kIsoThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_p2vals, threshold, contrib,
                                                        band, d_nonconv, m->d_err);
  else
    k_iso_contrib<3><<<kIsoBlocks, kIsoThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_p2vals, threshold, contrib,
                                                        band, d_nonconv, m->d_err);
  k_iso_average<<<kIsoBlocks, kIsoThreads, 0, s>>>(m->nedges, nel, m->d_edge_ptr, m->d_edge_inc, contrib, band,
                                                   d_gdef);
  return iso_check("k_iso_deformation");
}

extern "C" int xg_iso_integrate_mesh(xg_mesh* m, const double* d_p2vals, int dt, int order, double threshold,
                                     int deform, int ex, int ey, int ez, double* d_result, int32_t* d_nonconv,
                                     void* stream) {
  if (!m || !d_p2vals || !d_result || !d_nonconv || dt < 0 || dt > 2 || order < 0 || order > kMaxOrder || ex < 0 ||
      ey < 0 || ez < 0)
    return XG_ERR_ARG;
  if (m->tensor) {
    set_last_error("xg_iso_integrate_mesh: simplex meshes only");
    return XG_ERR_UNSUPPORTED;
  }
  if (m->ne >= (1 << 28)) return XG_ERR_CAPACITY;
  if (int st = iso_incidence(m)) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int nel = m->dim == 2 ? 3 : 6;
  const size_t n_contrib = (size_t)m->ne * nel * 3, n_gdef = (size_t)m->nedges * 3;
  const size_t need = sizeof(double) * (n_contrib + n_gdef + kIsoBlocks) + (size_t)m->ne;
  if (m->iso_bytes < need) {
    cudaFree(m->d_iso);
    m->d_iso = nullptr;
    m->iso_bytes = 0;
    XG_CUDA(cudaMalloc(&m->d_iso, need));
    m->iso_bytes = need;
  }
  double* contrib = (double*)m->d_iso;
  double* gdef = contrib + n_contrib;
  double* bs = gdef + n_gdef;
  uint8_t* band = (uint8_t*)(bs + kIsoBlocks);
  XG_CUDA(cudaMemsetAsync(d_nonconv, 0, sizeof(int32_t), s));
  if (deform) {
    if (m->dim == 2)
      k_iso_contrib<2><<<kIsoBlocks, kIsoThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_p2vals, threshold,
                                                          contrib, band, d_nonconv, m->d_err);
    else
      k_iso_contrib<3><<<kIsoBlocks, kIsoThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_p2vals, threshold,
                                                          contrib, band, d_nonconv, m->d_err);
    k_iso_average<<<kIsoBlocks, kIsoThreads, 0, s>>>(m->nedges, nel, m->d_edge_ptr, m->d_edge_inc, contrib, band,
                                                     gdef);
  } else {
    XG_CUDA(cudaMemsetAsync(gdef, 0, sizeof(double) * n_gdef, s));
  }
  if (m->dim == 2)
    k_iso_integrate<2><<<kIsoBlocks, kIsoThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, m->d_el_edges, d_p2vals,
                                                          gdef, dt, order, ex, ey, ez, bs, m->d_err);
  else
    k_iso_integrate<3><<<kIsoBlocks, kIsoThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, m->d_el_edges, d_p2vals,
                                                          gdef, dt, order, ex, ey, ez, bs, m->d_err);
  k_iso_final<<<1, 32, 0, s>>>(bs, kIsoBlocks, d_result);
  return iso_check("k_iso");
}

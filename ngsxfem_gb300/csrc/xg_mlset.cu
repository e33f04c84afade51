// Several level sets on simplex meshes: Integrate over a union of domain
// tuples and the rule export (cutint/mlsetintegration.cpp:6-180,
// cutint/straightcutrule.cpp:679-812, cutint/cutintegral.cpp:126-212).
// The per-element rule is xg_mlset.cuh; one thread builds and consumes the
// rule of one element.  Compiled with -fmad=false: the exported points and
// weights follow the CPU statement operation by operation.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "xg_internal.h"
#include "xg_mlset.cuh"

namespace xg {

static __device__ RuleTable g_mrules;

int upload_rules_mlset() {
  XG_CUDA(cudaMemcpyToSymbol(g_mrules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

constexpr int kMlThreads = 128;
constexpr int kMlBlocks = 152 * 8;

template <int D>
__device__ __forceinline__ void gather_ml(int ne, const int32_t* __restrict__ elv, const double* __restrict__ xyz, int nv,
                                          const double* __restrict__ lsets, int M, int e, double (*xv)[3],
                                          double (*lv)[D + 1]) {
#pragma unroll
  for (int v = 0; v <= D; v++) {
    const int vid = elv[(int64_t)v * ne + e];
#pragma unroll
    for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
    for (int m = 0; m < M; m++) lv[m][v] = lsets[(int64_t)m * nv + vid];
  }
}

__device__ __forceinline__ double ipow_ml(double x, int e) {
  double r = 1.0;
  for (int i = 0; i < e; i++) r *= x;
  return r;
}

__device__ __forceinline__ bool tbit_ml(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

}  // namespace

template <int D>
__global__ void __launch_bounds__(kMlThreads) k_mlset_integrate(int ne, const int32_t* __restrict__ elv,
                                                                const double* __restrict__ xyz, int nv,
                                                                const double* __restrict__ lsets, const __grid_constant__ ml::MlDesc md,
                                                                int order, int ex, int ey, int ez,
                                                                const uint64_t* __restrict__ defined_on,
                                                                double* block_sums, int* err) {
  __shared__ double red[kMlThreads];
  double acc = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    if (defined_on && !tbit_ml(defined_on, e)) continue;
    double xv[D + 1][3], lv[ml::kMaxLsets][D + 1];
    gather_ml<D>(ne, elv, xyz, nv, lsets, md.M, (int)e, xv, lv);
    ml::AGeo g;
    ml::make_ageo<D>(xv, g);
    const double meas = fabs(g.det);
    auto emit = [&](const double* xi, double w) {
      double x[3] = {0, 0, 0};
      for (int i = 0; i < D; i++) {
        double s = g.x0[i];
        for (int k = 0; k < D; k++) s += g.F[i][k] * xi[k];
        x[i] = s;
      }
      const double fv = ipow_ml(x[0], ex) * ipow_ml(x[1], ey) * (D == 3 ? ipow_ml(x[2], ez) : 1.0);
      acc += w * meas * fv;
    };
    int npts = 0;
    const int st = ml::element_rule<D>(&g_mrules, g, md.M, md.ntup, md.dt, lv, order, emit, &npts);
    if (st) set_err(err, st);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kMlThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
}

__global__ void k_mlset_final(const double* bs, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += bs[i];
    out[0] = s;
  }
}

// rule export for listed elements: points on the reference simplex, weights
// as the reference returns them (codimension transforms included);
// counts[i] = -1 for "no rule"
template <int D>
__global__ void __launch_bounds__(kMlThreads) k_mlset_rules(int ne, const int32_t* __restrict__ elv,
                                                            const double* __restrict__ xyz, int nv,
                                                            const double* __restrict__ lsets, const __grid_constant__ ml::MlDesc md,
                                                            const int32_t* __restrict__ elems, int n, int order,
                                                            int max_pts, int32_t* counts, double* pts, double* wts,
                                                            int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int e = elems[i];
  if (e < 0 || e >= ne) {
    set_err(err, XG_ERR_ARG);
    counts[i] = 0;
    return;
  }
  double xv[D + 1][3], lv[ml::kMaxLsets][D + 1];
  gather_ml<D>(ne, elv, xyz, nv, lsets, md.M, e, xv, lv);
  ml::AGeo g;
  ml::make_ageo<D>(xv, g);
  double* P = pts + (int64_t)i * max_pts * 3;
  double* W = wts + (int64_t)i * max_pts;
  int k = 0;
  auto emit = [&](const double* p, double w) {
    if (k < max_pts) {
      for (int c = 0; c < 3; c++) P[3 * k + c] = p[c];
      W[k] = w;
    }
    k++;
  };
  int npts = 0;
  const int st = ml::element_rule<D>(&g_mrules, g, md.M, md.ntup, md.dt, lv, order, emit, &npts);
  if (st || k > max_pts) {
    set_err(err, st ? st : XG_ERR_CAPACITY);
    counts[i] = 0;
    return;
  }
  counts[i] = k == 0 ? -1 : k;
}

// MultiLevelsetCutInformation markers (xfem/cutinfo.cpp:306-419): mode 0
// marks elements whose level-set domain types equal a tuple, mode 1 those
// whose order-0 rule of the region has a positive weight sum.  bits cleared
// by the caller; bits are set with atomic OR (the result does not depend on
// the order).
template <int D>
__global__ void __launch_bounds__(kMlThreads) k_mlset_mark(int ne, const int32_t* __restrict__ elv,
                                                           const double* __restrict__ xyz, int nv,
                                                           const double* __restrict__ lsets,
                                                           const __grid_constant__ ml::MlDesc md, int mode,
                                                           unsigned long long* bits, int* err) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double xv[D + 1][3], lv[ml::kMaxLsets][D + 1];
    gather_ml<D>(ne, elv, xyz, nv, lsets, md.M, (int)e, xv, lv);
    bool mark = false;
    if (mode == 0) {
      int ldt[ml::kMaxLsets];
      for (int m = 0; m < md.M; m++) ldt[m] = qc::qcheck(lv[m], D + 1, 0.0);
      for (int t = 0; t < md.ntup && !mark; t++) {
        bool match = true;
        for (int m = 0; m < md.M; m++) match &= md.dt[t * md.M + m] == ldt[m];
        mark = match;
      }
    } else {
      ml::AGeo g;
      ml::make_ageo<D>(xv, g);
      double part = 0.0;
      auto emit = [&](const double*, double w) { part += w; };
      int npts = 0;
      const int st = ml::element_rule<D>(&g_mrules, g, md.M, md.ntup, md.dt, lv, 0, emit, &npts);
      if (st) set_err(err, st);
      mark = st == 0 && npts > 0 && part > 0;
    }
    if (mark) atomicOr(bits + (e >> 6), 1ull << (e & 63));
  }
}

// Integrate(x^ex y^ey z^ez * dCut(lset, dt, vb=BND)) over the boundary
// elements (the boundary facets, vertices ascending): thread per boundary
// element, fixed-order block sums.
template <int D>
__global__ void __launch_bounds__(kMlThreads) k_integrate_bnd(int64_t nbnd, const int32_t* __restrict__ bnd_v,
                                                              const double* __restrict__ xyz, int nv,
                                                              const double* __restrict__ lset, int dt, int order,
                                                              int ex, int ey, int ez,
                                                              const uint64_t* __restrict__ defined_on,
                                                              double* block_sums, int* err) {
  __shared__ double red[kMlThreads];
  double acc = 0.0;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbnd; b += (int64_t)gridDim.x * blockDim.x) {
    if (defined_on && !tbit_ml(defined_on, b)) continue;
    double xv[D][3], l[D];
    for (int v = 0; v < D; v++) {
      const int vid = bnd_v[(int64_t)v * nbnd + b];
      l[v] = lset[vid];
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
    }
    auto emit = [&](const double* x, double w, double meas) {
      acc += w * meas * (ipow_ml(x[0], ex) * ipow_ml(x[1], ey) * (D == 3 ? ipow_ml(x[2], ez) : 1.0));
    };
    const int st = ml::bnd_rule<D>(&g_mrules, xv, l, dt, order, emit);
    if (st) set_err(err, st);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kMlThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
}

static int launch_check_ml(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return XG_OK;
}

int mlset_desc(int32_t M, const int8_t* h_domains, int32_t ndom, ml::MlDesc* md) {
  if (M < 1 || M > ml::kMaxLsets || ndom < 1 || ndom > ml::kMaxTuples || !h_domains) {
    set_last_error("multi-level-set domain: 1..8 level sets and 1..256 domain tuples");
    return XG_ERR_ARG;
  }
  md->M = M;
  md->ntup = ndom;
  for (int i = 0; i < M * ndom; i++) {
    if (h_domains[i] != XG_NEG && h_domains[i] != XG_POS && h_domains[i] != XG_IF) {
      set_last_error("multi-level-set domain: entries must be XG_NEG, XG_POS or XG_IF");
      return XG_ERR_ARG;
    }
    md->dt[i] = h_domains[i];
  }
  return XG_OK;
}

int mlset_integrate(xg_mesh* m, const double* d_lsets, const ml::MlDesc& md, int order, int ex, int ey, int ez,
                    const uint64_t* d_defined_on, double* d_result, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const size_t need = sizeof(double) * kMlBlocks;
  if (m->scratch_bytes < need) {
    cudaFree(m->d_scratch);
    m->d_scratch = nullptr;
    m->scratch_bytes = 0;
    XG_CUDA(cudaMalloc(&m->d_scratch, need));
    m->scratch_bytes = need;
  }
  double* bs = (double*)m->d_scratch;
  if (m->dim == 2)
    k_mlset_integrate<2><<<kMlBlocks, kMlThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lsets, md, order, ex,
                                                         ey, ez, d_defined_on, bs, m->d_err);
  else
    k_mlset_integrate<3><<<kMlBlocks, kMlThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lsets, md, order, ex,
                                                         ey, ez, d_defined_on, bs, m->d_err);
  k_mlset_final<<<1, 32, 0, s>>>(bs, kMlBlocks, d_result);
  return launch_check_ml("k_mlset_integrate");
}

int mlset_mark(xg_mesh* m, const double* d_lsets, const ml::MlDesc& md, int mode, uint64_t* d_bits, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  XG_CUDA(cudaMemsetAsync(d_bits, 0, sizeof(uint64_t) * (((size_t)m->ne + 63) / 64), s));
  if (m->dim == 2)
    k_mlset_mark<2><<<kMlBlocks, kMlThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lsets, md, mode,
                                                     (unsigned long long*)d_bits, m->d_err);
  else
    k_mlset_mark<3><<<kMlBlocks, kMlThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lsets, md, mode,
                                                     (unsigned long long*)d_bits, m->d_err);
  return launch_check_ml("k_mlset_mark");
}

int mlset_cut_rules(xg_mesh* m, const double* d_lsets, const ml::MlDesc& md, const int32_t* d_elems, int32_t n,
                    int order, int32_t max_pts, int32_t* d_counts, double* d_pts, double* d_wts, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned nb = (unsigned)((n + kMlThreads - 1) / kMlThreads);
  if (m->dim == 2)
    k_mlset_rules<2><<<nb, kMlThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lsets, md, d_elems, n, order,
                                               max_pts, d_counts, d_pts, d_wts, m->d_err);
  else
    k_mlset_rules<3><<<nb, kMlThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lsets, md, d_elems, n, order,
                                               max_pts, d_counts, d_pts, d_wts, m->d_err);
  return launch_check_ml("k_mlset_rules");
}

}  // namespace xg

using namespace xg;

static int mlset_mesh_ok(const xg_mesh* m, const char* what) {
  if (!m) return XG_ERR_ARG;
  if (m->tensor) {
    set_last_error(std::string(what) + ": several level sets are supported on simplex meshes");
    return XG_ERR_UNSUPPORTED;
  }
  return XG_OK;
}

extern "C" {

int xg_integrate_mlset(xg_mesh* m, const double* d_lsets, int32_t nlsets, const int8_t* h_domains, int32_t ndomains,
                       int order, int ex, int ey, int ez, const uint64_t* d_defined_on, double* d_result,
                       void* stream) {
  if (int st = mlset_mesh_ok(m, "xg_integrate_mlset")) return st;
  if (!d_lsets || !d_result || order < 0 || order > kMaxOrder || ex < 0 || ey < 0 || ez < 0) return XG_ERR_ARG;
  ml::MlDesc md;
  if (int st = mlset_desc(nlsets, h_domains, ndomains, &md)) return st;
  return mlset_integrate(m, d_lsets, md, order, ex, ey, ez, d_defined_on, d_result, stream);
}

int xg_cut_rules_mlset(xg_mesh* m, const double* d_lsets, int32_t nlsets, const int8_t* h_domains, int32_t ndomains,
                       const int32_t* d_elems, int32_t n, int order, int32_t max_pts, int32_t* d_counts,
                       double* d_pts, double* d_wts, void* stream) {
  if (int st = mlset_mesh_ok(m, "xg_cut_rules_mlset")) return st;
  if (!d_lsets || !d_elems || n < 0 || order < 0 || order > kMaxOrder || max_pts <= 0 || !d_counts || !d_pts ||
      !d_wts)
    return XG_ERR_ARG;
  ml::MlDesc md;
  if (int st = mlset_desc(nlsets, h_domains, ndomains, &md)) return st;
  if (n == 0) return XG_OK;
  return mlset_cut_rules(m, d_lsets, md, d_elems, n, order, max_pts, d_counts, d_pts, d_wts, stream);
}

int xg_mlset_mark(xg_mesh* m, const double* d_lsets, int32_t nlsets, const int8_t* h_domains, int32_t ndomains,
                  int mode, uint64_t* d_bits, void* stream) {
  if (int st = mlset_mesh_ok(m, "xg_mlset_mark")) return st;
  if (!d_lsets || !d_bits || (mode != 0 && mode != 1)) return XG_ERR_ARG;
  ml::MlDesc md;
  if (int st = mlset_desc(nlsets, h_domains, ndomains, &md)) return st;
  return mlset_mark(m, d_lsets, md, mode, d_bits, stream);
}

int xg_integrate_bnd(xg_mesh* m, const double* d_lset, int dt, int order, int ex, int ey, int ez,
                     const uint64_t* d_defined_on, double* d_result, void* stream) {
  if (int st = mlset_mesh_ok(m, "xg_integrate_bnd")) return st;
  if (!d_lset || !d_result || dt < 0 || dt > 2 || order < 0 || order > kMaxOrder || ex < 0 || ey < 0 || ez < 0)
    return XG_ERR_ARG;
  if (dt == XG_IF && m->dim == 3) {
    set_last_error("xg_integrate_bnd: the interface on boundary triangles (codimension 2) is not supported");
    return XG_ERR_UNSUPPORTED;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const size_t need = sizeof(double) * kMlBlocks;
  if (m->scratch_bytes < need) {
    cudaFree(m->d_scratch);
    m->d_scratch = nullptr;
    m->scratch_bytes = 0;
    XG_CUDA(cudaMalloc(&m->d_scratch, need));
    m->scratch_bytes = need;
  }
  double* bs = (double*)m->d_scratch;
  if (m->nbnd == 0) {
    XG_CUDA(cudaMemsetAsync(d_result, 0, sizeof(double), s));
    return XG_OK;
  }
  if (m->dim == 2)
    k_integrate_bnd<2><<<kMlBlocks, kMlThreads, 0, s>>>(m->nbnd, m->d_bnd_v, m->d_xyz, m->nv, d_lset, dt, order, ex,
                                                       ey, ez, d_defined_on, bs, m->d_err);
  else
    k_integrate_bnd<3><<<kMlBlocks, kMlThreads, 0, s>>>(m->nbnd, m->d_bnd_v, m->d_xyz, m->nv, d_lset, dt, order, ex,
                                                       ey, ez, d_defined_on, bs, m->d_err);
  k_mlset_final<<<1, 32, 0, s>>>(bs, kMlBlocks, d_result);
  return launch_check_ml("k_integrate_bnd");
}

int xg_mlset_rule_capacity(int dim, int32_t nlsets, int32_t ndomains, int order) {
  if ((dim != 2 && dim != 3) || nlsets < 1 || nlsets > ml::kMaxLsets || ndomains < 1 ||
      ndomains > ml::kMaxTuples || order < 0 || order > kMaxOrder)
    return -1;
  // per tuple at most 3^M final simplices of dimension <= dim
  const RuleTable& R = host_rules();
  const int nq = R.cnt[dim][clamp_order(order)];
  long long leaves = 1;
  for (int i = 0; i < nlsets; i++) leaves *= 3;
  const long long cap = (long long)ndomains * leaves * nq;
  return cap > (1 << 30) ? (1 << 30) : (int)cap;
}

}  // extern "C"

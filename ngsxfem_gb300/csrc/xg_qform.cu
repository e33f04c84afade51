// Bilinear forms of the Q1 space (dofs = vertices) on quadrilateral and
// hexahedral meshes: SymbolicCutBFI on ET_QUAD / ET_HEX
// (xfem/symboliccutbfi.cpp:76-486; the integration order defaults to trial +
// test order there, :107-111, with no derivative reduction on these element
// types) with StraightCutIntegrationRule's quad branch
// (cutint/straightcutrule.cpp:206-501, 582-677: here qc::tp_cut_rule of
// xg_quadcut.cuh on the unit box, the bilinear / trilinear map and the
// interface factor |J^-T n_ref| per point).  The assembly:
//   k_qf_elmat   thread per element: the domain type, whether a term holds the
//                element, its 4x4 / 8x8 matrix (FP64 sums over the terms' rules)
//   k_qf_rows    thread per vertex: the columns its active elements reach, as
//                a bitmask over the vertex's full-pattern row (at most 9 / 27
//                columns, static positions from form creation)
//   scans        compressed row numbers and row offsets
//   k_qf_fill    thread per active vertex: the row's sums over its active
//                elements in ascending order, the compressed columns
// so the values are summed in a fixed order and no atomics touch them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "xg_internal.h"
#include "xg_quadcut.cuh"

namespace xg {

static __device__ RuleTable g_qf_rules;

int upload_rules_qform() {
  XG_CUDA(cudaMemcpyToSymbol(g_qf_rules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

constexpr int kQfMaxTerms = 8;
constexpr int kQfThreads = 128;
constexpr int kScanBlock = 1024;

struct QfTerm {
  int kind, domain, order, hpow;
  double coef, b[3];
  const uint64_t* defined_on;
};
struct QfDesc {
  int n;
  QfTerm t[kQfMaxTerms];
};

__device__ __forceinline__ bool qf_bit(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

// Q1 shape functions of the unit box (corner v at (cx, cy, cz)) and their
// reference gradients
template <int D>
__device__ __forceinline__ void q1_shapes(const double* p, double* N, double (*dN)[3]) {
  constexpr int NV = 1 << D;
  const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const double fx = cx[v] ? p[0] : 1.0 - p[0], gx = cx[v] ? 1.0 : -1.0;
    const double fy = cy[v] ? p[1] : 1.0 - p[1], gy = cy[v] ? 1.0 : -1.0;
    const double fz = D == 3 ? (cz[v] ? p[2] : 1.0 - p[2]) : 1.0, gz = cz[v] ? 1.0 : -1.0;
    N[v] = fx * fy * fz;
    dN[v][0] = gx * fy * fz;
    dN[v][1] = fx * gy * fz;
    dN[v][2] = fx * fy * gz;
  }
}

// J^-1 and det J of a D x D Jacobian
template <int D>
__device__ __forceinline__ double inv_det(const double (*J)[3], double (*Ji)[3]) {
  if (D == 2) {
    const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0], id = 1.0 / det;
    Ji[0][0] = J[1][1] * id;
    Ji[0][1] = -J[0][1] * id;
    Ji[1][0] = -J[1][0] * id;
    Ji[1][1] = J[0][0] * id;
    return det;
  }
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02, id = 1.0 / det;
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

template <int D>
__global__ void __launch_bounds__(kQfThreads) k_qf_elmat(int ne, int nv, const int32_t* __restrict__ elv,
                                                         const double* __restrict__ xyz,
                                                         const double* __restrict__ lset, QfDesc d, int pol,
                                                         uint8_t* __restrict__ act, double* __restrict__ elmat,
                                                         int* err) {
  constexpr int NV = 1 << D;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double l[NV], xv[NV][3];
    for (int v = 0; v < NV; v++) {
      const int id = elv[(int64_t)v * ne + e];
      l[v] = lset[id];
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + id] : 0.0;
    }
    const int dom = qc::qcheck(l, NV, 0.0);
    bool any = false;
    for (int t = 0; t < d.n; t++) {
      const QfTerm& T = d.t[t];
      if ((!T.defined_on || qf_bit(T.defined_on, e)) && (dom == XG_IF || dom == T.domain)) any = true;
    }
    act[e] = any ? 1 : 0;
    if (!any) continue;
    double A[NV * NV];
    for (int k = 0; k < NV * NV; k++) A[k] = 0.0;
    const qc::QL L = D == 2 ? qc::ql_quad(l) : qc::ql_hex(l);
    for (int t = 0; t < d.n; t++) {
      const QfTerm& T = d.t[t];
      if ((T.defined_on && !qf_bit(T.defined_on, e)) || (dom != XG_IF && dom != T.domain)) continue;
      auto emit = [&](const double* p, double wr) {
        double N[NV], dN[NV][3], J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, Ji[3][3];
        q1_shapes<D>(p, N, dN);
        for (int v = 0; v < NV; v++)
          for (int i = 0; i < D; i++)
            for (int k = 0; k < D; k++) J[i][k] += xv[v][i] * dN[v][k];
        const double adet = fabs(inv_det<D>(J, Ji));
        double w = wr * adet;
        double gl[3] = {0, 0, 0}, nrm[3] = {0, 0, 0};
        const bool need_n = T.kind == XG_TERM_NGRADU_V || T.kind == XG_TERM_U_NGRADV;
        if ((dom == XG_IF && T.domain == XG_IF) || need_n) {
          qc::ql_grad(L, p, gl);
          double nn = 0.0, gn = 0.0;
          for (int k = 0; k < D; k++) {
            double s = 0.0;
            for (int j = 0; j < D; j++) s += Ji[j][k] * gl[j];
            nrm[k] = s;
            nn += s * s;
            gn += gl[k] * gl[k];
          }
          nn = sqrt(nn);
          // the interface factor |J^-T n_ref|, n_ref the unit reference gradient
          if (dom == XG_IF && T.domain == XG_IF) w *= nn / sqrt(gn);
          for (int k = 0; k < D; k++) nrm[k] /= nn;
        }
        const double c = T.hpow == 0 ? T.coef : T.coef * int_pow(mesh_h<D>(adet), T.hpow);
        double G[NV][3], dn[NV];
        for (int v = 0; v < NV; v++) {
          double s = 0.0;
          for (int k = 0; k < 3; k++) {
            double g = 0.0;
            if (k < D)
              for (int j = 0; j < D; j++) g += Ji[j][k] * dN[v][j];
            G[v][k] = g;
            s += (T.kind == XG_TERM_CONV ? T.b[k] : nrm[k]) * g;
          }
          dn[v] = s;
        }
        const double W = w * c;
        for (int a = 0; a < NV; a++)      // test
          for (int b = 0; b < NV; b++) {  // trial
            double v;
            switch (T.kind) {
              case XG_TERM_MASS: v = N[a] * N[b]; break;
              case XG_TERM_LAPLACE: v = G[a][0] * G[b][0] + G[a][1] * G[b][1] + G[a][2] * G[b][2]; break;
              case XG_TERM_U_NGRADV: v = N[b] * dn[a]; break;
              default: v = dn[b] * N[a]; break;  // XG_TERM_NGRADU_V, XG_TERM_CONV
            }
            A[a * NV + b] += W * v;
          }
      };
      const int st = qc::tp_cut_rule<D>(&g_qf_rules, l, T.domain, T.order, pol, emit);
      if (st > 0) set_err(err, st);
    }
    for (int k = 0; k < NV * NV; k++) {
      if (!finite_bits(A[k])) set_err(err, XG_ERR_NONFINITE);
      elmat[e * NV * NV + k] = A[k];
    }
  }
}

// per vertex: the positions (in its full-pattern row) that its active
// elements reach, whether it is an active row, and its column count
template <int D>
__global__ void __launch_bounds__(kQfThreads) k_qf_rows(int nv, const int32_t* __restrict__ vptr,
                                                        const int32_t* __restrict__ vadj,
                                                        const uint8_t* __restrict__ pos, const uint8_t* __restrict__ act,
                                                        uint32_t* __restrict__ mask, int64_t* __restrict__ flag,
                                                        int64_t* __restrict__ cnt) {
  constexpr int NV = 1 << D;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = 0;
    for (int k = vptr[v]; k < vptr[v + 1]; k++) {
      const int64_t e = vadj[k] >> 3;
      const int a = vadj[k] & 7;
      if (!act[e]) continue;
      for (int b = 0; b < NV; b++) m |= 1u << pos[(e * NV + a) * NV + b];
    }
    mask[v] = m;
    flag[v] = m ? 1 : 0;
    cnt[v] = __popc(m);
  }
}

// exclusive scan of int64 values: per-block scans, one block over the block
// sums, the offsets added (fixed order)
__global__ void __launch_bounds__(kScanBlock) k_scan_local(const int64_t* __restrict__ in, int64_t n,
                                                           int64_t* __restrict__ out, int64_t* __restrict__ bsum) {
  __shared__ int64_t s[kScanBlock];
  const int64_t i = blockIdx.x * (int64_t)kScanBlock + threadIdx.x;
  const int64_t x = i < n ? in[i] : 0;
  s[threadIdx.x] = x;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    const int64_t y = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += y;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - x;
  if (threadIdx.x == kScanBlock - 1) bsum[blockIdx.x] = s[threadIdx.x];
}
__global__ void k_scan_blocks(int64_t* bsum, int nb, int64_t* total) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int64_t acc = 0;
    for (int b = 0; b < nb; b++) {
      const int64_t x = bsum[b];
      bsum[b] = acc;
      acc += x;
    }
    *total = acc;
  }
}
__global__ void k_scan_add(int64_t* out, int64_t n, const int64_t* bsum) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] += bsum[i / kScanBlock];
}

template <int D>
__global__ void __launch_bounds__(kQfThreads) k_qf_fill(int nv, const int32_t* __restrict__ vptr,
                                                        const int32_t* __restrict__ vadj,
                                                        const uint8_t* __restrict__ pos, const uint8_t* __restrict__ act,
                                                        const double* __restrict__ elmat,
                                                        const uint32_t* __restrict__ mask,
                                                        const int64_t* __restrict__ rowid,
                                                        const int64_t* __restrict__ off,
                                                        const int64_t* __restrict__ full_ptr,
                                                        const int32_t* __restrict__ full_cols,
                                                        int32_t* __restrict__ row_dof, int64_t* __restrict__ rowptr,
                                                        int32_t* __restrict__ cols, double* __restrict__ vals,
                                                        int64_t cap_nnz, int* err) {
  constexpr int NV = 1 << D, W = D == 2 ? 9 : 27;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t m = mask[v];
    if (!m) continue;
    double acc[W];
    for (int p = 0; p < W; p++) acc[p] = 0.0;
    for (int k = vptr[v]; k < vptr[v + 1]; k++) {
      const int64_t e = vadj[k] >> 3;
      const int a = vadj[k] & 7;
      if (!act[e]) continue;
      for (int b = 0; b < NV; b++) acc[pos[(e * NV + a) * NV + b]] += elmat[(e * NV + a) * NV + b];
    }
    const int64_t r = rowid[v], o = off[v];
    row_dof[r] = (int32_t)v;
    rowptr[r] = o;
    if (o + __popc(m) > cap_nnz) {
      set_err(err, XG_ERR_CAPACITY);
      continue;
    }
    int q = 0;
    for (int p = 0; p < W; p++)
      if ((m >> p) & 1u) {
        cols[o + q] = (int32_t)rowid[full_cols[full_ptr[v] + p]];
        vals[o + q] = acc[p];
        q++;
      }
  }
}

__global__ void k_qf_final(const int64_t* tot, int64_t* rowptr, int64_t* counts) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    rowptr[tot[0]] = tot[1];
    counts[0] = tot[0];
    counts[1] = tot[1];
  }
}

int scan_i64(const int64_t* in, int64_t n, int64_t* out, int64_t* bsum, int64_t* total, cudaStream_t s) {
  const int nb = (int)((n + kScanBlock - 1) / kScanBlock);
  if (nb == 0) {
    XG_CUDA(cudaMemsetAsync(total, 0, sizeof(int64_t), s));
    return XG_OK;
  }
  k_scan_local<<<nb, kScanBlock, 0, s>>>(in, n, out, bsum);
  k_scan_blocks<<<1, 32, 0, s>>>(bsum, nb, total);
  k_scan_add<<<nb, kScanBlock, 0, s>>>(out, n, bsum);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_scan");
}

}  // namespace
}  // namespace xg

using namespace xg;

struct xg_quad_form {
  xg_mesh* mesh = nullptr;
  int pol = 1;
  QfDesc desc = {};
  int64_t full_nnz = 0;
  int32_t* d_vptr = nullptr;   // [nv + 1] vertex -> (element * 8 + local vertex), elements ascending
  int32_t* d_vadj = nullptr;
  int64_t* d_full_ptr = nullptr;
  int32_t* d_full_cols = nullptr;  // full-pattern rows (sorted vertices)
  uint8_t* d_pos = nullptr;        // [ne][NV][NV]: column of (a, b) in a's full row
  uint8_t* d_act = nullptr;
  double* d_elmat = nullptr;       // [ne][NV][NV]
  uint32_t* d_mask = nullptr;
  int64_t* d_work = nullptr;       // flag, cnt, rowid, off ([nv] each), block sums, totals
};

extern "C" {

int xg_quad_form_destroy(xg_quad_form* f) {
  if (!f) return XG_OK;
  void* p[] = {f->d_vptr, f->d_vadj, f->d_full_ptr, f->d_full_cols, f->d_pos, f->d_act, f->d_elmat, f->d_mask,
               f->d_work};
  for (void* q : p) cudaFree(q);
  delete f;
  return XG_OK;
}

int xg_quad_form_create(xg_mesh* m, const xg_term* terms, int32_t nterms, int policy, xg_quad_form** out) {
  if (!m || !out || nterms < 0 || nterms > kQfMaxTerms || (nterms > 0 && !terms) || policy < 0 || policy > 2) {
    set_last_error("xg_quad_form_create: bad arguments (at most 8 terms, policy 0..2)");
    return XG_ERR_ARG;
  }
  if (!m->tensor) {
    set_last_error("xg_quad_form_create: quadrilateral / hexahedral meshes (xg_mesh_create_tensor)");
    return XG_ERR_UNSUPPORTED;
  }
  if (m->ne >= (1 << 28)) return XG_ERR_CAPACITY;
  *out = nullptr;
  QfDesc d = {};
  for (int t = 0; t < nterms; t++) {
    const xg_term& T = terms[t];
    const bool kind_ok = T.kind == XG_TERM_MASS || T.kind == XG_TERM_LAPLACE || T.kind == XG_TERM_NGRADU_V ||
                         T.kind == XG_TERM_U_NGRADV || T.kind == XG_TERM_CONV;
    if (!kind_ok || T.domain < XG_NEG || T.domain > XG_IF || T.order > kMaxOrder) {
      set_last_error("xg_quad_form_create: kinds MASS, LAPLACE, NGRADU_V, U_NGRADV, CONV on NEG / POS / IF");
      return XG_ERR_ARG;
    }
    QfTerm& Q = d.t[d.n++];
    Q.kind = T.kind;
    Q.domain = T.domain;
    Q.order = T.order >= 0 ? T.order : 2;  // trial + test order of Q1
    Q.hpow = T.hpow;
    Q.coef = T.coef;
    for (int k = 0; k < 3; k++) Q.b[k] = T.b[k];
    Q.defined_on = T.d_defined_on;
  }
  const int D = m->dim, NV = 1 << D, nv = m->nv, ne = m->ne;
  // vertex -> elements (ascending), full-pattern rows, static positions
  std::vector<int32_t> vptr(nv + 1, 0), vadj((size_t)ne * NV);
  for (size_t i = 0; i < m->h_elv.size(); i++) vptr[m->h_elv[i] + 1]++;
  for (int v = 0; v < nv; v++) vptr[v + 1] += vptr[v];
  {
    std::vector<int32_t> fill(vptr.begin(), vptr.end() - 1);
    for (int e = 0; e < ne; e++)
      for (int a = 0; a < NV; a++) vadj[fill[m->h_elv[(size_t)e * NV + a]]++] = e * 8 + a;
  }
  std::vector<int64_t> fptr(nv + 1, 0);
  std::vector<int32_t> fcols;
  std::vector<int32_t> tmp;
  for (int v = 0; v < nv; v++) {
    tmp.clear();
    for (int k = vptr[v]; k < vptr[v + 1]; k++) {
      const int e = vadj[k] >> 3;
      for (int b = 0; b < NV; b++) tmp.push_back(m->h_elv[(size_t)e * NV + b]);
    }
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    if ((int)tmp.size() > (D == 2 ? 9 : 27)) {
      set_last_error("xg_quad_form_create: a vertex reaches more columns than a conforming Q1 mesh allows");
      return XG_ERR_UNSUPPORTED;
    }
    fcols.insert(fcols.end(), tmp.begin(), tmp.end());
    fptr[v + 1] = (int64_t)fcols.size();
  }
  std::vector<uint8_t> pos((size_t)ne * NV * NV);
  for (int e = 0; e < ne; e++)
    for (int a = 0; a < NV; a++) {
      const int va = m->h_elv[(size_t)e * NV + a];
      const int32_t* row = fcols.data() + fptr[va];
      const int w = (int)(fptr[va + 1] - fptr[va]);
      for (int b = 0; b < NV; b++) {
        const int vb = m->h_elv[(size_t)e * NV + b];
        pos[((size_t)e * NV + a) * NV + b] = (uint8_t)(std::lower_bound(row, row + w, vb) - row);
      }
    }
  auto* f = new xg_quad_form();
  f->mesh = m;
  f->pol = policy;
  f->desc = d;
  f->full_nnz = (int64_t)fcols.size();
  const int nb = (nv + kScanBlock - 1) / kScanBlock;
  auto up = [&](void** p, const void* h, size_t bytes) -> int {
    if (cudaMalloc(p, bytes ? bytes : 8) != cudaSuccess) return XG_ERR_CUDA;
    if (h && bytes && cudaMemcpy(*p, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return XG_ERR_CUDA;
    return XG_OK;
  };
  int st = XG_OK;
  st = st ? st : up((void**)&f->d_vptr, vptr.data(), vptr.size() * 4);
  st = st ? st : up((void**)&f->d_vadj, vadj.data(), vadj.size() * 4);
  st = st ? st : up((void**)&f->d_full_ptr, fptr.data(), fptr.size() * 8);
  st = st ? st : up((void**)&f->d_full_cols, fcols.data(), fcols.size() * 4);
  st = st ? st : up((void**)&f->d_pos, pos.data(), pos.size());
  st = st ? st : up((void**)&f->d_act, nullptr, (size_t)ne);
  st = st ? st : up((void**)&f->d_elmat, nullptr, (size_t)ne * NV * NV * 8);
  st = st ? st : up((void**)&f->d_mask, nullptr, (size_t)nv * 4);
  st = st ? st : up((void**)&f->d_work, nullptr, ((size_t)4 * nv + nb + 2) * 8);
  if (st) {
    xg_quad_form_destroy(f);
    set_last_error("xg_quad_form_create: cudaMalloc failed");
    return st;
  }
  *out = f;
  return XG_OK;
}

int xg_quad_form_capacity(const xg_quad_form* f, int64_t* o) {
  if (!f || !o) return XG_ERR_ARG;
  o[0] = f->mesh->nv;
  o[1] = f->full_nnz;
  return XG_OK;
}

int xg_quad_form_assemble(xg_quad_form* f, const double* d_lset, xg_csr* out, void* stream) {
  if (!f || !d_lset || !out || !out->d_row_dof || !out->d_rowptr || !out->d_cols || !out->d_vals || !out->d_counts)
    return XG_ERR_ARG;
  xg_mesh* m = f->mesh;
  if (out->cap_rows < m->nv) {
    set_last_error("xg_quad_form_assemble: cap_rows below the number of vertices");
    return XG_ERR_CAPACITY;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int nv = m->nv, ne = m->ne;
  const int nb = (nv + kScanBlock - 1) / kScanBlock;
  int64_t* flag = f->d_work;
  int64_t* cnt = flag + nv;
  int64_t* rowid = cnt + nv;
  int64_t* off = rowid + nv;
  int64_t* bsum = off + nv;
  int64_t* tot = bsum + nb;
  const unsigned ge = (unsigned)((ne + kQfThreads - 1) / kQfThreads), gv = (unsigned)((nv + kQfThreads - 1) / kQfThreads);
  if (m->dim == 2) {
    k_qf_elmat<2><<<ge, kQfThreads, 0, s>>>(ne, nv, m->d_elv, m->d_xyz, d_lset, f->desc, f->pol, f->d_act, f->d_elmat,
                                            m->d_err);
    k_qf_rows<2><<<gv, kQfThreads, 0, s>>>(nv, f->d_vptr, f->d_vadj, f->d_pos, f->d_act, f->d_mask, flag, cnt);
  } else {
    k_qf_elmat<3><<<ge, kQfThreads, 0, s>>>(ne, nv, m->d_elv, m->d_xyz, d_lset, f->desc, f->pol, f->d_act, f->d_elmat,
                                            m->d_err);
    k_qf_rows<3><<<gv, kQfThreads, 0, s>>>(nv, f->d_vptr, f->d_vadj, f->d_pos, f->d_act, f->d_mask, flag, cnt);
  }
  int st;
  if ((st = scan_i64(flag, nv, rowid, bsum, tot + 0, s))) return st;
  if ((st = scan_i64(cnt, nv, off, bsum, tot + 1, s))) return st;
  if (m->dim == 2)
    k_qf_fill<2><<<gv, kQfThreads, 0, s>>>(nv, f->d_vptr, f->d_vadj, f->d_pos, f->d_act, f->d_elmat, f->d_mask, rowid,
                                           off, f->d_full_ptr, f->d_full_cols, out->d_row_dof, out->d_rowptr,
                                           out->d_cols, out->d_vals, out->cap_nnz, m->d_err);
  else
    k_qf_fill<3><<<gv, kQfThreads, 0, s>>>(nv, f->d_vptr, f->d_vadj, f->d_pos, f->d_act, f->d_elmat, f->d_mask, rowid,
                                           off, f->d_full_ptr, f->d_full_cols, out->d_row_dof, out->d_rowptr,
                                           out->d_cols, out->d_vals, out->cap_nnz, m->d_err);
  k_qf_final<<<1, 32, 0, s>>>(tot, out->d_rowptr, out->d_counts);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_qf");
}

}  // extern "C"

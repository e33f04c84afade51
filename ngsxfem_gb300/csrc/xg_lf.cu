// Linear forms on cut domains: SymbolicCutLinearFormIntegrator
// (xfem/symboliccutlfi.cpp:57-180) and the vector assembly of
// LinearForm::Assemble.
//
// Per element (thread per element, FP64): for every term whose domain the
// element carries (uncut and matching: the element's own rule; cut: the
// straight cut rule of the term's domain, interface weights with |F^-T n|),
//   elvec_i += w_q |det F| g(x_q) phi_i(x_q),
// g = coef * x^e0 y^e1 z^e2 or coef * u_h (u_h a function of the form's space
// or of another H1 / L2 space of the mesh, by its own basis);
// the default order is 2k (symboliccutlfi.cpp:93-94).  Then thread per dof:
// the sum over the dof's (element, local) adjacency in ascending element
// order -- a fixed order, no atomics.
//
// Boundary terms (dCut(lset, dt, vb=BND)): thread per BND element, the
// boundary rule of xg_mlset.cuh, the owning element's basis at the rule's
// physical points (reference coordinates by F^-1); then thread per dof, the
// sum over its (BND element, local) adjacency in ascending order, added to
// the volume part.
#include <algorithm>
#include <cstring>
#include <vector>

#include "xg_basis.cuh"
#include "xg_cut.cuh"
#include "xg_internal.h"
#include "xg_isomesh.cuh"
#include "xg_lfbnd.cuh"

namespace xg {

static __constant__ RuleTable c_rules;
static __device__ RuleTable g_lfb_rules;  // the boundary rule code reads its table by pointer

int upload_rules_lf() {
  XG_CUDA(cudaMemcpyToSymbol(c_rules, &host_rules(), sizeof(RuleTable)));
  XG_CUDA(cudaMemcpyToSymbol(g_lfb_rules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

constexpr int kMaxLTerms = 8;

struct LfDesc {
  int n;
  xg_lterm t[kMaxLTerms];
  int gf_order[kMaxLTerms];           // XG_LTERM_SOURCE_GF in another space: its order (0: the form's space)
  const int32_t* gf_dofs[kMaxLTerms]; // and its element dofs [nd][ne]
  const double* gdef;        // mesh deformation [nedges][3] of the volume terms, or NULL
  const int32_t* el_edges;   // [nedges per element][ne]
};

namespace {

__device__ __forceinline__ bool tbit64(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

// descriptor of local function i of an H1 element of runtime order k
template <int D>
__device__ __forceinline__ int lf_desc_rt(int k, int i, const int* gv) {
  return k == 1 ? fn_desc<D, 1>(i, gv) : (k == 2 ? fn_desc<D, 2>(i, gv) : fn_desc<D, 3>(i, gv));
}

__device__ __forceinline__ double ipow(double x, int e) {
  double r = 1.0;
  for (int k = 0; k < e; k++) r *= x;
  return r;
}

template <int D, int K>
__global__ void __launch_bounds__(128) k_lf_elvec(int ne, int nv, const int32_t* __restrict__ elv,
                                                   const double* __restrict__ xyz, const double* __restrict__ lset,
                                                   const uint8_t* __restrict__ dom,
                                                   const int32_t* __restrict__ el_dofs, LfDesc d,
                                                   double* __restrict__ elvec, int* err) {
  constexpr int N = ndof_el(D, K);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
    double b[N];
#pragma unroll
    for (int i = 0; i < N; i++) b[i] = 0.0;
    const int de = dom[e];
    double xv[D + 1][3], l[D + 1];
    int gv[4];
#pragma unroll
    for (int v = 0; v <= D; v++) {
      const int vid = elv[(int64_t)v * ne + e];
      gv[v] = vid;
      l[v] = lset[vid];
#pragma unroll
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
    }
    Geo<D> g;
    make_geo<D>(xv, g);
    const double meas = fabs(g.det);
    int desc[N];
#pragma unroll
    for (int i = 0; i < N; i++) desc[i] = fn_desc<D, K>(i, gv);
    // the deformed mesh: theta_j = J^-1 gdef(edge j), the reference frame
    double theta[6][3];
    if (d.gdef) {
      constexpr int NE = D == 2 ? 3 : 6;
      for (int j = 0; j < 6; j++)
        for (int r = 0; r < 3; r++) {
          double sr = 0.0;
          if (j < NE && r < D) {
            const int ed = d.el_edges[(int64_t)j * ne + e];
            for (int k = 0; k < D; k++) sr += g.Finv[r][k] * d.gdef[(int64_t)ed * 3 + k];
          }
          theta[j][r] = sr;
        }
    }
    for (int t = 0; t < d.n; t++) {
      const xg_lterm& T = d.t[t];
      if (T.kind == XG_LTERM_SOURCE_BND) continue;
      if (T.d_defined_on && !tbit64(T.d_defined_on, e)) continue;
      const int dt = T.domain;
      const int p = clamp_order(T.order >= 0 ? T.order : 2 * K);
      Sub subs[3];
      int ns = 0;
      bool whole = false;
      if (de == XG_IF) {
        ns = decompose<D>(l, dt, subs);
        if (ns < 0) {
          set_err(err, -ns);
          continue;
        }
      } else if (de == dt) {
        whole = true;
        ns = 1;
      } else {
        continue;
      }
      const int sd = (dt == XG_IF) ? D - 1 : D;
      const int off = c_rules.off[sd][p], cnt = c_rules.cnt[sd][p];
      const double fac = dt == XG_IF ? if_factor<D>(g, l) : 1.0;
      for (int s = 0; s < ns; s++) {
        const double vol = whole ? 1.0 : simplex_volume(subs[s].p, sd + 1);
        for (int q = 0; q < cnt; q++) {
          double pt[3];
          if (whole) {
#pragma unroll
            for (int k = 0; k < 3; k++) pt[k] = c_rules.x[off + q][k];
          } else {
            plain_point(subs[s], sd + 1, c_rules.x[off + q], pt);
          }
          double lam[D + 1], sl = 0.0;
#pragma unroll
          for (int k = 0; k < D; k++) {
            lam[k] = pt[k];
            sl += pt[k];
          }
          lam[D] = 1.0 - sl;
          double phi[N];
#pragma unroll
          for (int i = 0; i < N; i++) phi[i] = eval_fn_value<D, double>(desc[i], lam);
          double gval;
          // on the deformed mesh: the point y = pt + Theta(pt), the weight
          // |det (J A)| (IF: times |(J A)^-T n_ref|) instead of |det J| fac
          double y[3] = {pt[0], pt[1], pt[2]}, wdef = meas * fac;
          if (d.gdef) {
            double Am[3][3], F[3][3], Fi[3][3], detF;
            iso::deform_at<D>(theta, pt, y, Am);
            for (int r = 0; r < 3; r++)
              for (int k = 0; k < 3; k++) {
                double sr = 0.0;
                if (r < D && k < D)
                  for (int q2 = 0; q2 < D; q2++) sr += g.F[r][q2] * Am[q2][k];
                F[r][k] = r < D && k < D ? sr : (r == k ? 1.0 : 0.0);
              }
            if (!iso::invert<D>(F, Fi, &detF)) {
              set_err(err, XG_ERR_NONFINITE);
              continue;
            }
            wdef = fabs(detF);
            if (dt == XG_IF) {
              double nn = 0.0, gn = 0.0;
              for (int k = 0; k < D; k++) {
                double sr = 0.0;
                for (int j = 0; j < D; j++) sr += Fi[j][k] * (l[j] - l[D]);
                nn += sr * sr;
                gn += (l[k] - l[D]) * (l[k] - l[D]);
              }
              wdef *= sqrt(nn / gn);
            }
          }
          if (T.kind == XG_LTERM_SOURCE) {
            double x[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int i = 0; i < D; i++) {
              double sacc = g.x0[i];
#pragma unroll
              for (int k = 0; k < D; k++) sacc += g.F[i][k] * y[k];
              x[i] = sacc;
            }
            gval = T.coef * ipow(x[0], T.e[0]) * ipow(x[1], T.e[1]) * (D == 3 ? ipow(x[2], T.e[2]) : 1.0);
          } else if (d.gf_order[t] == 0) {
            double u = 0.0;
#pragma unroll
            for (int j = 0; j < N; j++) u += T.d_gf[el_dofs[(int64_t)e * N + j]] * phi[j];
            gval = T.coef * u;
          } else {
            // u_h of another space: its own basis at the point
            const int kg = d.gf_order[t], ng = ndof_el(D, kg);
            double u = 0.0;
            for (int j = 0; j < ng; j++)
              u += T.d_gf[d.gf_dofs[t][(int64_t)j * ne + e]] * eval_fn_value<D, double>(lf_desc_rt<D>(kg, j, gv), lam);
            gval = T.coef * u;
          }
          const double w = c_rules.w[off + q] * vol * wdef * gval;
#pragma unroll
          for (int i = 0; i < N; i++) b[i] += w * phi[i];
        }
      }
    }
#pragma unroll
    for (int i = 0; i < N; i++) {
      if (!isfinite(b[i])) set_err(err, XG_ERR_NONFINITE);
      elvec[(int64_t)e * N + i] = b[i];
    }
  }
}

// boundary terms: bvec[b][i] for BND element b (vertices bnd_v, owner bnd_el[b])
template <int D, int K>
__global__ void __launch_bounds__(128) k_lf_bnd(int64_t nbnd, const int32_t* __restrict__ bnd_v,
                                                 const int32_t* __restrict__ bnd_el, int ne, int nv,
                                                 const int32_t* __restrict__ elv, const double* __restrict__ xyz,
                                                 const double* __restrict__ lset, LfDesc d,
                                                 double* __restrict__ bvec, int* err) {
  constexpr int N = ndof_el(D, K);
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbnd; b += (int64_t)gridDim.x * blockDim.x) {
    double acc[N];
    const int e = bnd_el[b];
    double xv[D + 1][3];
    int gv[4];
#pragma unroll
    for (int v = 0; v <= D; v++) {
      const int vid = elv[(int64_t)v * ne + e];
      gv[v] = vid;
#pragma unroll
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
    }
    double xb[D][3], lb[D];
#pragma unroll
    for (int v = 0; v < D; v++) {
      const int vid = bnd_v[(int64_t)v * nbnd + b];
      lb[v] = lset[vid];
#pragma unroll
      for (int c = 0; c < 3; c++) xb[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
    }
    const int st = lfb::element_vector<D, K>(&g_lfb_rules, xv, gv, xb, lb, d.t, d.n, b, acc);
    if (st) set_err(err, st);
#pragma unroll
    for (int i = 0; i < N; i++) {
      if (!isfinite(acc[i])) set_err(err, XG_ERR_NONFINITE);
      bvec[b * N + i] = acc[i];
    }
  }
}

// out[r] += the boundary contributions of dof r, BND elements ascending
__global__ void k_lf_gather_bnd(int64_t ndof, int nd, const int32_t* __restrict__ adj_ptr,
                                const int32_t* __restrict__ adj, const double* __restrict__ bvec,
                                double* __restrict__ out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < ndof; r += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int a = adj_ptr[r]; a < adj_ptr[r + 1]; a++) {
      const int v = adj[a];
      s += bvec[(int64_t)(v >> 5) * nd + (v & 31)];
    }
    out[r] += s;
  }
}

__global__ void k_lf_gather(int64_t ndof, int nd, const int32_t* __restrict__ adj_ptr, const int32_t* __restrict__ adj,
                            const double* __restrict__ elvec, double* __restrict__ out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < ndof; r += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int a = adj_ptr[r]; a < adj_ptr[r + 1]; a++) {
      const int v = adj[a];
      s += elvec[(int64_t)(v >> 5) * nd + (v & 31)];
    }
    out[r] = s;
  }
}

}  // namespace
}  // namespace xg

using namespace xg;

struct xg_lform {
  xg_space* space = nullptr;
  LfDesc desc;
  double* d_elvec = nullptr;
  int* d_err = nullptr;
  // boundary terms: owner element per BND element, their vectors, and the
  // dof -> (BND element * 32 + local) adjacency, BND elements ascending
  bool has_bnd = false;
  int32_t* d_bnd_el = nullptr;
  double* d_bvec = nullptr;
  int32_t* d_badj_ptr = nullptr;
  int32_t* d_badj = nullptr;
};

static void lform_free(xg_lform* f) {
  cudaFree(f->d_elvec);
  cudaFree(f->d_err);
  cudaFree(f->d_bnd_el);
  cudaFree(f->d_bvec);
  cudaFree(f->d_badj_ptr);
  cudaFree(f->d_badj);
  delete f;
}

static int lform_bnd_setup(xg_lform* f) {
  const xg_space* sp = f->space;
  const xg_mesh* m = sp->mesh;
  const int64_t nbnd = m->nbnd;
  if (nbnd >= (1 << 26)) {
    set_last_error("xg_lform_create: " + std::to_string(nbnd) +
                   " boundary elements; boundary terms take at most 2^26 - 1");
    return XG_ERR_CAPACITY;
  }
  const int nd = sp->nd;
  std::vector<int32_t> owner((size_t)std::max<int64_t>(nbnd, 1), 0), ptr((size_t)sp->ndof + 1, 0);
  for (int64_t b = 0; b < nbnd; b++) {
    owner[b] = m->h_facet_els[2 * (size_t)m->h_bnd_facets[b]];
    for (int i = 0; i < nd; i++) ptr[(size_t)sp->h_el_dofs[(size_t)owner[b] * nd + i] + 1]++;
  }
  for (int64_t r = 0; r < sp->ndof; r++) ptr[r + 1] += ptr[r];
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1), adj((size_t)std::max<int32_t>(ptr.back(), 1), 0);
  for (int64_t b = 0; b < nbnd; b++)
    for (int i = 0; i < nd; i++) adj[fill[sp->h_el_dofs[(size_t)owner[b] * nd + i]]++] = (int32_t)(b * 32 + i);
  XG_CUDA(cudaMalloc((void**)&f->d_bnd_el, sizeof(int32_t) * owner.size()));
  XG_CUDA(cudaMalloc((void**)&f->d_bvec, sizeof(double) * (size_t)std::max<int64_t>(nbnd, 1) * nd));
  XG_CUDA(cudaMalloc((void**)&f->d_badj_ptr, sizeof(int32_t) * ptr.size()));
  XG_CUDA(cudaMalloc((void**)&f->d_badj, sizeof(int32_t) * adj.size()));
  XG_CUDA(cudaMemcpy(f->d_bnd_el, owner.data(), sizeof(int32_t) * owner.size(), cudaMemcpyHostToDevice));
  XG_CUDA(cudaMemcpy(f->d_badj_ptr, ptr.data(), sizeof(int32_t) * ptr.size(), cudaMemcpyHostToDevice));
  XG_CUDA(cudaMemcpy(f->d_badj, adj.data(), sizeof(int32_t) * adj.size(), cudaMemcpyHostToDevice));
  return XG_OK;
}

extern "C" {

int xg_lform_create(xg_space* space, const xg_lterm* terms, int32_t n, xg_lform** out) {
  if (!space || !out || n < 0 || n > kMaxLTerms || (n > 0 && !terms) || space->kt >= 1) {
    set_last_error("xg_lform_create: spatial H1 space and at most 8 terms");
    return XG_ERR_ARG;
  }
  for (int t = 0; t < n; t++) {
    const xg_lterm& T = terms[t];
    if (T.kind == XG_LTERM_SOURCE_BND && T.domain == XG_IF && space->mesh->dim == 3) {
      set_last_error("xg_lform_create: the interface on boundary triangles (codimension 2) is not supported");
      return XG_ERR_UNSUPPORTED;
    }
    const xg_space* gs = T.kind == XG_LTERM_SOURCE_GF ? T.gf_space : nullptr;
    if (gs && gs != space &&
        (gs->mesh != space->mesh || gs->kt >= 0 || gs->order < 1 || gs->order > 3 ||
         gs->nd != ndof_el(space->mesh->dim, gs->order))) {
      set_last_error("xg_lform_create: the source GridFunction needs a spatial H1 / L2 space of order 1..3 on "
                     "the form's mesh");
      return XG_ERR_ARG;
    }
    if ((T.kind != XG_LTERM_SOURCE && T.kind != XG_LTERM_SOURCE_GF && T.kind != XG_LTERM_SOURCE_BND) ||
        T.domain < 0 || T.domain > 2 ||
        T.order > kMaxOrder || (T.kind == XG_LTERM_SOURCE_GF && !T.d_gf) || T.e[0] < 0 || T.e[1] < 0 || T.e[2] < 0) {
      set_last_error("xg_lform_create: invalid term");
      return XG_ERR_ARG;
    }
  }
  *out = nullptr;
  auto* f = new xg_lform();
  f->space = space;
  std::memset(&f->desc, 0, sizeof(f->desc));
  f->desc.n = n;
  for (int t = 0; t < n; t++) {
    f->desc.t[t] = terms[t];
    const xg_space* gs = terms[t].kind == XG_LTERM_SOURCE_GF ? terms[t].gf_space : nullptr;
    if (gs && gs != space) {
      f->desc.gf_order[t] = gs->order;
      f->desc.gf_dofs[t] = gs->d_el_dofs;
    }
  }
  cudaError_t e = cudaMalloc((void**)&f->d_elvec, sizeof(double) * (size_t)space->mesh->ne * space->nd);
  if (!e) e = cudaMalloc((void**)&f->d_err, sizeof(int));
  if (!e) e = cudaMemset(f->d_err, 0, sizeof(int));
  if (e) {
    lform_free(f);
    return cuda_fail(e, "xg_lform_create");
  }
  for (int t = 0; t < n; t++) f->has_bnd |= terms[t].kind == XG_LTERM_SOURCE_BND;
  if (f->has_bnd) {
    if (int st = lform_bnd_setup(f)) {
      lform_free(f);
      return st;
    }
  }
  *out = f;
  return XG_OK;
}

int xg_lform_destroy(xg_lform* f) {
  if (!f) return XG_OK;
  lform_free(f);
  return XG_OK;
}

int xg_lform_check(xg_lform* f) {
  if (!f) return XG_ERR_ARG;
  int h = 0;
  XG_CUDA(cudaMemcpy(&h, f->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  XG_CUDA(cudaMemset(f->d_err, 0, sizeof(int)));
  if (h) set_last_error(std::string("device error: ") + xg_status_string(h));
  return h;
}

int xg_lform_set_deformation(xg_lform* f, const double* d_gdef) {
  if (!f) return XG_ERR_ARG;
  f->desc.gdef = d_gdef;
  f->desc.el_edges = f->space->mesh->d_el_edges;
  return XG_OK;
}

int xg_lform_assemble(xg_lform* f, const double* d_lset, const uint8_t* d_dom, double* d_out, void* stream) {
  if (!f || !d_lset || !d_dom || !d_out) return XG_ERR_ARG;
  xg_space* sp = f->space;
  xg_mesh* m = sp->mesh;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned grid = (unsigned)std::max(1, std::min((m->ne + 127) / 128, 152 * 16));
  const int D = m->dim, K = sp->order;
#define XG_LF(DD, KK)                                                                                            \
  k_lf_elvec<DD, KK><<<grid, 128, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, d_lset, d_dom, sp->d_el_dofs_aos, \
                                          f->desc, f->d_elvec, f->d_err)
  if (D == 2 && K == 1) XG_LF(2, 1);
  else if (D == 2 && K == 2) XG_LF(2, 2);
  else if (D == 2 && K == 3) XG_LF(2, 3);
  else if (D == 3 && K == 1) XG_LF(3, 1);
  else if (D == 3 && K == 2) XG_LF(3, 2);
  else XG_LF(3, 3);
#undef XG_LF
  const unsigned g2 = (unsigned)std::max<int64_t>(1, std::min<int64_t>((sp->ndof + 255) / 256, 152 * 16));
  k_lf_gather<<<g2, 256, 0, s>>>(sp->ndof, sp->nd, sp->d_dof_adj_ptr, sp->d_dof_adj, f->d_elvec, d_out);
  if (f->has_bnd && m->nbnd > 0) {
    const unsigned gb = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m->nbnd + 127) / 128, 152 * 16));
#define XG_LFB(DD, KK)                                                                                      \
  k_lf_bnd<DD, KK><<<gb, 128, 0, s>>>(m->nbnd, m->d_bnd_v, f->d_bnd_el, m->ne, m->nv, m->d_elv, m->d_xyz, d_lset, \
                                      f->desc, f->d_bvec, f->d_err)
    if (D == 2 && K == 1) XG_LFB(2, 1);
    else if (D == 2 && K == 2) XG_LFB(2, 2);
    else if (D == 2 && K == 3) XG_LFB(2, 3);
    else if (D == 3 && K == 1) XG_LFB(3, 1);
    else if (D == 3 && K == 2) XG_LFB(3, 2);
    else XG_LFB(3, 3);
#undef XG_LFB
    k_lf_gather_bnd<<<g2, 256, 0, s>>>(sp->ndof, sp->nd, f->d_badj_ptr, f->d_badj, f->d_bvec, d_out);
  }
  XG_CUDA(cudaGetLastError());
  return XG_OK;
}

}  // extern "C"

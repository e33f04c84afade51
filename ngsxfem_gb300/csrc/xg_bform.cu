// Boundary terms of bilinear forms (dCut(lset, dt, vb=BND)): ngsxfem's
// SymbolicCutBFI on boundary elements (xfem/symboliccutbfi.cpp:76-486 with
// vb == BND; the rule of cutint/straightcutrule.cpp:582-677 on the boundary
// facet, here ml::bnd_rule).  Thread per owning element: its BND elements in
// ascending order, per term the domain part's rule and c * u * v with the
// owner's basis at the rule's physical points (the relations of
// xg_lfbnd.cuh), summed in FP64 and added to the owner's element rows (which
// the volume kernels wrote first); one thread owns an element's rows, so the
// sums need no atomics and are formed in the same order on every run.  An
// owner is active when one of its BND elements has a part in a term's domain.
#include <cuda_runtime.h>

#include <cstdint>

#include "xg_basis.cuh"
#include "xg_internal.h"
#include "xg_lfbnd.cuh"

namespace xg {

static __device__ RuleTable g_bf_rules;  // the boundary rule code reads its table by pointer

int upload_rules_bform() {
  XG_CUDA(cudaMemcpyToSymbol(g_bf_rules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

__device__ __forceinline__ bool bf_bit64(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }
__device__ __forceinline__ bool bf_bit32(const uint32_t* b, int64_t i) { return (b[i >> 5] >> (i & 31)) & 1u; }

// owners of a BND element that has a part in a boundary term's domain (its
// straight-cut domain type, CheckIfStraightCut of its vertex values, is the
// term's domain or IF) join the active elements (as uncut-list elements
// when they are not active already)
__global__ void k_bnd_active(BndFormLaunch L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n_own) return;
  const int e = L.own_el[i];
  bool on = false;
  for (int j = L.own_ptr[i]; j < L.own_ptr[i + 1] && !on; j++) {
    const int b = L.own_bnd[j];
    double l[3];
    for (int v = 0; v < L.dim; v++) l[v] = L.lset[L.bnd_v[(int64_t)v * L.nbnd + b]];
    const int dom = qc::qcheck(l, L.dim, 0.0);
    for (int t = 0; t < L.d.n; t++)
      if ((!L.d.t[t].defined_on || bf_bit64(L.d.t[t].defined_on, b)) && (dom == XG_IF || dom == L.d.t[t].domain))
        on = true;
  }
  if (on && !bf_bit32(L.act_cut, e)) atomicOr(&L.act_un[e >> 5], 1u << (e & 31));
}

template <int D, int K, typename T>
__global__ void __launch_bounds__(128) k_bnd_elmat(BndFormLaunch L) {
  constexpr int N = ndof_el(D, K);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L.n_own; i += gridDim.x * blockDim.x) {
    const int e = L.own_el[i];
    if (!bf_bit32(L.act_un, e) && !bf_bit32(L.act_cut, e)) continue;
    double xv[D + 1][3];
    int gv[4] = {0, 0, 0, 0};
    for (int v = 0; v <= D; v++) {
      gv[v] = L.elv[(int64_t)v * L.ne + e];
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? L.xyz[(int64_t)c * L.nv + gv[v]] : 0.0;
    }
    double x0[3], Finv[3][3];
    lfb::owner_inverse<D>(xv, x0, Finv);
    double det;
    {
      double F[3][3];
      for (int r = 0; r < D; r++)
        for (int c = 0; c < D; c++) F[r][c] = xv[c][r] - xv[D][r];
      det = D == 2 ? F[0][0] * F[1][1] - F[0][1] * F[1][0]
                   : F[0][0] * (F[1][1] * F[2][2] - F[1][2] * F[2][1]) - F[0][1] * (F[1][0] * F[2][2] - F[1][2] * F[2][0]) +
                         F[0][2] * (F[1][0] * F[2][1] - F[1][1] * F[2][0]);
    }
    const double h = mesh_h<D>(fabs(det));
    int desc[N];
    for (int a = 0; a < N; a++) desc[a] = fn_desc<D, K>(a, gv);
    double A[N * N];
    for (int k = 0; k < N * N; k++) A[k] = 0.0;
    for (int j = L.own_ptr[i]; j < L.own_ptr[i + 1]; j++) {
      const int b = L.own_bnd[j];
      double xb[D][3], lb[D];
      for (int v = 0; v < D; v++) {
        const int vid = L.bnd_v[(int64_t)v * L.nbnd + b];
        lb[v] = L.lset[vid];
        for (int c = 0; c < 3; c++) xb[v][c] = c < D ? L.xyz[(int64_t)c * L.nv + vid] : 0.0;
      }
      for (int t = 0; t < L.d.n; t++) {
        const BndTermDev& Tm = L.d.t[t];
        if (Tm.defined_on && !bf_bit64(Tm.defined_on, b)) continue;
        const double c = Tm.hpow == 0 ? Tm.coef : Tm.coef * int_pow(h, Tm.hpow);
        auto emit = [&](const double* x, double w, double meas) {
          double lam[D + 1], sl = 0.0;
          for (int k = 0; k < D; k++) {
            double s = 0.0;
            for (int cc = 0; cc < D; cc++) s += Finv[k][cc] * (x[cc] - x0[cc]);
            lam[k] = s;
            sl += s;
          }
          lam[D] = 1.0 - sl;
          double phi[N];
          for (int a = 0; a < N; a++) phi[a] = eval_fn_value<D, double>(desc[a], lam);
          const double W = w * meas * c;
          for (int a = 0; a < N; a++)
            for (int bb = 0; bb < N; bb++) A[a * N + bb] += W * phi[a] * phi[bb];
        };
        const int st = ml::bnd_rule<D>(&g_bf_rules, xb, lb, Tm.domain, Tm.order, emit);
        if (st) set_err(L.err, st);
      }
    }
    for (int a = 0; a < N; a++) {
      T* row = (T*)L.elmat + (int64_t)L.rowslot[(int64_t)e * N + a] * N;
      for (int bb = 0; bb < N; bb++) {
        const double v = (double)row[bb] + A[a * N + bb];
        if (!finite_bits(v)) set_err(L.err, XG_ERR_NONFINITE);
        row[bb] = (T)v;
      }
    }
  }
}

template <int D, int K, typename T>
int launch_t(const BndFormLaunch& L, cudaStream_t s) {
  k_bnd_elmat<D, K, T><<<152 * 4, 128, 0, s>>>(L);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_bnd_elmat");
}

template <typename T>
int launch_k(const BndFormLaunch& L, cudaStream_t s) {
  if (L.dim == 2) {
    if (L.order == 1) return launch_t<2, 1, T>(L, s);
    if (L.order == 2) return launch_t<2, 2, T>(L, s);
    return launch_t<2, 3, T>(L, s);
  }
  if (L.order == 1) return launch_t<3, 1, T>(L, s);
  if (L.order == 2) return launch_t<3, 2, T>(L, s);
  return launch_t<3, 3, T>(L, s);
}

}  // namespace

int bnd_active_launch(const BndFormLaunch& L, cudaStream_t s) {
  if (L.n_own <= 0) return XG_OK;
  k_bnd_active<<<(L.n_own + 127) / 128, 128, 0, s>>>(L);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_bnd_active");
}

int bnd_elmat_launch(const BndFormLaunch& L, cudaStream_t s) {
  if (L.n_own <= 0 || L.d.n <= 0) return XG_OK;
  if (L.dim < 2 || L.dim > 3 || L.order < 1 || L.order > 3) return XG_ERR_UNSUPPORTED;
  return L.fp64 ? launch_k<double>(L, s) : launch_k<float>(L, s);
}

}  // namespace xg

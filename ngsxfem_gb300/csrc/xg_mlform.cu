// Element matrices of bilinear-form terms on regions of several level sets:
// ngsxfem's SymbolicCutBilinearFormIntegrator with a multi-level-set
// LevelsetIntegrationDomain (xfem/symboliccutbfi.cpp:76-486; the rule of
// CreateMultiLevelsetCutIntegrationRule, cutint/mlsetintegration.cpp:6-180,
// here ml::element_rule of xg_mlset.cuh).  Per active element (thread per
// element): for every term whose element set holds it, the rule of the term's
// region (a union of domain tuples) and the term's integrand at its points
// (mass, Laplace, the Nitsche normal-derivative terms with the normal of one
// of the level sets, convection), summed in FP64 and written as the element's
// rows at their static row slots (the layout of xg_rows.h).
#include <cuda_runtime.h>

#include <cstdint>

#include "xg_basis.cuh"
#include "xg_internal.h"
#include "xg_mlset.cuh"

namespace xg {

static __device__ RuleTable g_mf_rules;  // the rule code reads its table by pointer

int upload_rules_mlform() {
  XG_CUDA(cudaMemcpyToSymbol(g_mf_rules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

__device__ __forceinline__ bool mf_bit(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

template <int D, int K, typename T>
__global__ void __launch_bounds__(128) k_mlform(int ne, int nv, const int32_t* __restrict__ elv,
                                                const double* __restrict__ xyz, int M,
                                                const double* __restrict__ lsets, const MlTermDev* __restrict__ terms,
                                                int nterms, const int8_t* __restrict__ tuples,
                                                const int32_t* __restrict__ list, const int* __restrict__ counts,
                                                const int32_t* __restrict__ rowslot, T* __restrict__ elmat,
                                                int* __restrict__ err) {
  constexpr int N = ndof_el(D, K);
  const int n = counts[1];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int e = list[i];
    int gv[4] = {0, 0, 0, 0};
    double xv[D + 1][3], lv[ml::kMaxLsets][D + 1];
    for (int v = 0; v <= D; v++) {
      gv[v] = elv[(int64_t)v * ne + e];
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + gv[v]] : 0.0;
      for (int m = 0; m < M; m++) lv[m][v] = lsets[(int64_t)m * nv + gv[v]];
    }
    ml::AGeo g;
    ml::make_ageo<D>(xv, g);
    const double meas = fabs(g.det), h = mesh_h<D>(meas);
    // physical gradients of the barycentrics
    double gl[D + 1][D];
    for (int k = 0; k < D; k++) {
      double s = 0.0;
      for (int a = 0; a < D; a++) {
        gl[a][k] = g.Finv[a][k];
        s += g.Finv[a][k];
      }
      gl[D][k] = -s;
    }
    int desc[N];
    for (int a = 0; a < N; a++) desc[a] = fn_desc<D, K>(a, gv);
    double A[N * N];
    for (int k = 0; k < N * N; k++) A[k] = 0.0;
    for (int t = 0; t < nterms; t++) {
      const MlTermDev& Tm = terms[t];
      if (Tm.defined_on && !mf_bit(Tm.defined_on, e)) continue;
      const double c = Tm.hpow == 0 ? Tm.coef : Tm.coef * int_pow(h, Tm.hpow);
      double nrm[D];
      for (int k = 0; k < D; k++) nrm[k] = 0.0;
      if (Tm.kind == XG_TERM_NGRADU_V || Tm.kind == XG_TERM_U_NGRADV) {
        double nn = 0.0;
        for (int k = 0; k < D; k++) {
          double s = 0.0;
          for (int v = 0; v <= D; v++) s += lv[Tm.normal_lset][v] * gl[v][k];
          nrm[k] = s;
          nn += s * s;
        }
        const double inv = 1.0 / sqrt(nn);
        for (int k = 0; k < D; k++) nrm[k] *= inv;
      }
      auto emit = [&](const double* xi, double w) {
        double lam[D + 1], sl = 0.0;
        for (int k = 0; k < D; k++) {
          lam[k] = xi[k];
          sl += xi[k];
        }
        lam[D] = 1.0 - sl;
        double phi[N], gr[N][D], dn[N];
        for (int a = 0; a < N; a++) {
          eval_fn<D, double>(desc[a], lam, gl, phi[a], gr[a]);
          double s = 0.0;
          if (Tm.kind == XG_TERM_CONV) {
            for (int k = 0; k < D; k++) s += Tm.b[k] * gr[a][k];
          } else {
            for (int k = 0; k < D; k++) s += nrm[k] * gr[a][k];
          }
          dn[a] = s;
        }
        const double W = w * meas * c;
        for (int a = 0; a < N; a++)      // test
          for (int b = 0; b < N; b++) {  // trial
            double v;
            switch (Tm.kind) {
              case XG_TERM_MASS: v = phi[a] * phi[b]; break;
              case XG_TERM_LAPLACE: {
                v = 0.0;
                for (int k = 0; k < D; k++) v += gr[a][k] * gr[b][k];
                break;
              }
              case XG_TERM_NGRADU_V: v = dn[b] * phi[a]; break;
              case XG_TERM_U_NGRADV: v = phi[b] * dn[a]; break;
              default: v = dn[b] * phi[a]; break;  // XG_TERM_CONV
            }
            A[a * N + b] += W * v;
          }
      };
      int npts = 0;
      const int st = ml::element_rule<D>(&g_mf_rules, g, M, Tm.ntup, tuples + Tm.tup_off, lv, Tm.order, emit, &npts);
      if (st) set_err(err, st);
    }
    for (int a = 0; a < N; a++) {
      T* row = elmat + (int64_t)rowslot[(int64_t)e * N + a] * N;
      for (int b = 0; b < N; b++) {
        const double v = A[a * N + b];
        if (!finite_bits(v)) set_err(err, XG_ERR_NONFINITE);
        row[b] = (T)v;
      }
    }
  }
}

template <int D, int K, typename T>
int launch_t(const MlFormLaunch& L, cudaStream_t s) {
  k_mlform<D, K, T><<<152 * 8, 128, 0, s>>>(L.ne, L.nv, L.elv, L.xyz, L.M, L.lsets, L.terms, L.nterms, L.tuples,
                                           L.list, L.counts, L.rowslot, (T*)L.elmat, L.err);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_mlform");
}

template <typename T>
int launch_k(const MlFormLaunch& L, cudaStream_t s) {
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

int mlform_launch(const MlFormLaunch& L, cudaStream_t s) {
  if (L.dim < 2 || L.dim > 3 || L.order < 1 || L.order > 3 || L.M < 1 || L.M > ml::kMaxLsets)
    return XG_ERR_UNSUPPORTED;
  return L.fp64 ? launch_k<double>(L, s) : launch_k<float>(L, s);
}

}  // namespace xg

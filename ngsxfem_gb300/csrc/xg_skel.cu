// Skeleton terms on interior facets (XG_TERM_SKEL_*): the facet matrices of
// ngsxfem's SymbolicCutFacetBilinearFormIntegrator (xfem/symboliccutbfi.cpp:
// 886-1572, the facet cut to a domain by the P1 level set) and of
// SymbolicFacetBilinearFormIntegrator2 (:1574-1735, the whole facet), for the
// discontinuous-Galerkin jump / flux terms and the derivative-jump ghost
// penalty (normal derivatives of DiffOpDuDnk, xfem/ghostpenalty.cpp:221-365).
//
// Per active facet slot (the form's facet list, shared with the facet-patch
// terms) one 2n x 2n matrix, rows = test functions [element 1, element 2],
// columns = trial functions, full rows (the layout the row scatter reads):
//   A[a][b] = sum_q w_q ( cJ  s_a s_b P0_a P0_b  +  cF  s_a P0_a P1_b
//                        + cFT P1_a s_b P0_b      +  sum_k cDk s_a s_b Pk_a Pk_b )
// with Pj_a the j-th derivative of function a along n_F (the unit normal out
// of element 1) at point q, s_a = +1 on element 1 and -1 on element 2.  The
// facet rule is the straight-cut rule of the facet simplex (ml::bnd_rule, the
// reference's StraightCutIntegrationRuleUntransformed on the facet, order
// 2 * order of the space, :947-1042) or its plain rule; the weights carry the
// facet measure (:1126-1130).  The derivatives are exact (the reference's
// finite differences are exact on these polynomials up to rounding).
//
// One block handles FPB facets: one thread per facet builds the facet's
// geometry and rule into shared memory, the block evaluates the derivative
// vectors of all 2n functions at a chunk of points, and each thread sums its
// entries over the chunk in FP64 (fixed order: deterministic).  When the form
// has facet-patch terms their kernel has written the facet matrices first and
// this kernel adds to them.
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>

#include "xg_basis.cuh"
#include "xg_cut.cuh"
#include "xg_internal.h"
#include "xg_mlset.cuh"

namespace xg {

static __device__ RuleTable g_sk_rules;  // the facet rule code reads its table by pointer

int upload_rules_skel() {
  XG_CUDA(cudaMemcpyToSymbol(g_sk_rules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

__device__ __forceinline__ bool sk_bit(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

template <int D, int K>
struct SkCfg {
  static constexpr int N = ndof_el(D, K), N2 = 2 * N, E = N2 * N2, NT = 256;
  static constexpr int FPB = E >= 512 ? 1 : 512 / E;  // facets per block
  static constexpr int NACC = (FPB * E + NT - 1) / NT;
  // points of one facet rule of order 2K: 2D one segment piece of K + 1
  // points; 3D up to three triangle pieces of 3 / 6 / 16 points
  static constexpr int PMAX = D == 2 ? K + 1 : (K == 1 ? 9 : (K == 2 ? 18 : 48));
  static constexpr int CH = PMAX < 16 ? PMAX : 16;  // points per pass
  static constexpr int L = K + 1;                   // derivative orders 0..K
};

template <int D, int K>
struct SkSmem {
  using C = SkCfg<D, K>;
  double lam[C::FPB][C::PMAX][2][D + 1];  // barycentrics of the rule points in both elements
  double w[C::FPB][C::PMAX];              // rule weight x facet measure
  double V[C::FPB][C::CH][C::L][C::N2];   // derivatives along n_F of all functions
  double del[C::FPB][2][D + 1];           // d lambda_i / d n_F in both elements
  double x0[C::FPB][2][D];                // element maps: lambda = Finv (x - x0)
  double Finv[C::FPB][2][D][D];
  double X[C::FPB][D][3];                 // facet vertices
  double lf[C::FPB][D];                   // their level-set values
  double h1[C::FPB];
  double coef[C::FPB][kSkelKinds];        // the group's coefficients on this facet (0: not defined on)
  int desc[C::FPB][C::N2];
  int facet[C::FPB];
  int idx[C::FPB];
  int npts[C::FPB];
  int maxpts;
};

// geometry of the facet of slot idx into the block's shared memory; false if
// the facet has no second element
template <int D, int K>
__device__ bool skel_geometry(SkSmem<D, K>& sm, int fl, int f, int ne, int nv, const int32_t* __restrict__ elv,
                              const double* __restrict__ xyz, int64_t nf, const int32_t* __restrict__ fel,
                              const double* __restrict__ lset) {
  constexpr int N = SkCfg<D, K>::N;
  const int e1 = fel[f], e2 = fel[nf + f];
  if (e1 < 0 || e2 < 0) return false;
  int gv[2][D + 1];
  double xv[2][D + 1][3];
#pragma unroll
  for (int s = 0; s < 2; s++)
#pragma unroll
    for (int v = 0; v <= D; v++) {
      gv[s][v] = elv[(int64_t)v * ne + (s == 0 ? e1 : e2)];
#pragma unroll
      for (int c = 0; c < 3; c++) xv[s][v][c] = c < D ? xyz[(int64_t)c * nv + gv[s][v]] : 0.0;
    }
  Geo<D> g[2];
  make_geo<D>(xv[0], g[0]);
  make_geo<D>(xv[1], g[1]);
  // the facet: e1's vertices shared with e2 (e1's local order)
  int opp = -1, nfv = 0;
#pragma unroll
  for (int i = 0; i <= D; i++) {
    bool shared = false;
#pragma unroll
    for (int j = 0; j <= D; j++) shared |= gv[0][i] == gv[1][j];
    if (!shared) {
      opp = i;
    } else if (nfv < D) {
#pragma unroll
      for (int c = 0; c < 3; c++) sm.X[fl][nfv][c] = xv[0][i][c];
      sm.lf[fl][nfv] = lset ? lset[gv[0][i]] : -1.0;
      nfv++;
    }
  }
  if (opp < 0 || nfv != D) return false;
  // n_F = -grad lambda_opp / |grad lambda_opp| (outward of e1)
  double gl[D], nn = 0.0;
#pragma unroll
  for (int c = 0; c < D; c++) {
    double v = 0.0;
    if (opp < D) {
      v = g[0].Finv[opp][c];
    } else {
#pragma unroll
      for (int i = 0; i < D; i++) v -= g[0].Finv[i][c];
    }
    gl[c] = v;
    nn += v * v;
  }
  const double inv = -1.0 / sqrt(nn);
#pragma unroll
  for (int s = 0; s < 2; s++) {
    double sum = 0.0;
#pragma unroll
    for (int i = 0; i < D; i++) {
      double v = 0.0;
#pragma unroll
      for (int c = 0; c < D; c++) v += g[s].Finv[i][c] * (gl[c] * inv);
      sm.del[fl][s][i] = v;
      sum += v;
#pragma unroll
      for (int c = 0; c < D; c++) sm.Finv[fl][s][i][c] = g[s].Finv[i][c];
      sm.x0[fl][s][i] = g[s].x0[i];
    }
    sm.del[fl][s][D] = -sum;
  }
  for (int a = 0; a < N; a++) {
    sm.desc[fl][a] = fn_desc<D, K>(a, gv[0]);
    sm.desc[fl][N + a] = fn_desc<D, K>(a, gv[1]);
  }
  sm.h1[fl] = mesh_h<D>(fabs(g[0].det));
  return true;
}

template <int D, int K, typename T>
__global__ void __launch_bounds__(256) k_skel(const __grid_constant__ FormDesc form, int ne, int nv, const int32_t* __restrict__ elv,
                                              const double* __restrict__ xyz, int64_t nf,
                                              const int32_t* __restrict__ fel, const double* __restrict__ lset,
                                              const int32_t* __restrict__ l_fa, const int* __restrict__ counts,
                                              T* __restrict__ famat, int64_t cap_fa, int accumulate,
                                              int* __restrict__ err) {
  using C = SkCfg<D, K>;
  constexpr int N = C::N, N2 = C::N2, E = C::E, FPB = C::FPB, NT = C::NT, NACC = C::NACC, PMAX = C::PMAX,
                CH = C::CH, L = C::L;
  extern __shared__ __align__(16) unsigned char sk_raw[];
  SkSmem<D, K>& sm = *reinterpret_cast<SkSmem<D, K>*>(sk_raw);
  const int count = counts[2];
  for (int batch = blockIdx.x; batch * FPB < count; batch += gridDim.x) {
    __syncthreads();
    if (threadIdx.x < FPB) {
      const int fl = threadIdx.x, idx = batch * FPB + fl;
      sm.idx[fl] = -1;
      if (idx < count) {
        if (idx >= cap_fa) {
          set_err(err, XG_ERR_CAPACITY);
        } else {
          const int f = l_fa[idx];
          sm.facet[fl] = f;
          if (skel_geometry<D, K>(sm, fl, f, ne, nv, elv, xyz, nf, fel, lset)) sm.idx[fl] = idx;
          else set_err(err, XG_ERR_ARG);
        }
      }
    }
    Acc<double> acc[NACC];
#pragma unroll
    for (int m = 0; m < NACC; m++) acc[m].init();

    for (int gq = 0; gq < form.nskel; gq++) {
      const SkelDesc& G = form.s[gq];
      __syncthreads();
      // ---- the group's rule and coefficients on each facet (thread per facet)
      if (threadIdx.x == 0) sm.maxpts = 0;
      __syncthreads();
      if (threadIdx.x < FPB) {
        const int fl = threadIdx.x;
        int np = 0;
        const bool on = sm.idx[fl] >= 0 && (!G.defined_on || sk_bit(G.defined_on, sm.facet[fl]));
#pragma unroll
        for (int k = 0; k < kSkelKinds; k++)
          sm.coef[fl][k] = on && ((G.used >> k) & 1)
                               ? (G.hpow[k] == 0 ? G.c[k] : G.c[k] * int_pow(sm.h1[fl], G.hpow[k]))
                               : 0.0;
        if (on) {
          double xs[D][3], ls[D];
#pragma unroll
          for (int i = 0; i < D; i++) {
#pragma unroll
            for (int c = 0; c < 3; c++) xs[i][c] = sm.X[fl][i][c];
            ls[i] = G.region == XG_WHOLE ? -1.0 : sm.lf[fl][i];  // whole facet: the plain rule
          }
          auto emit = [&](const double* x, double w, double meas) {
            if (np >= PMAX) {
              set_err(err, XG_ERR_CAPACITY);
              return;
            }
            sm.w[fl][np] = w * meas;
#pragma unroll
            for (int s = 0; s < 2; s++) {
              double sum = 0.0;
#pragma unroll
              for (int i = 0; i < D; i++) {
                double v = 0.0;
#pragma unroll
                for (int c = 0; c < D; c++) v += sm.Finv[fl][s][i][c] * (x[c] - sm.x0[fl][s][c]);
                sm.lam[fl][np][s][i] = v;
                sum += v;
              }
              sm.lam[fl][np][s][D] = 1.0 - sum;
            }
            np++;
          };
          const int st = ml::bnd_rule<D>(&g_sk_rules, xs, ls, G.region == XG_WHOLE ? XG_NEG : G.region, 2 * K, emit);
          if (st) set_err(err, st);
        }
        sm.npts[fl] = np;
        atomicMax(&sm.maxpts, np);
      }
      __syncthreads();
      const int maxpts = sm.maxpts;
      for (int q0 = 0; q0 < maxpts; q0 += CH) {
        // ---- derivative vectors of all functions at the chunk's points
        for (int t = threadIdx.x; t < FPB * CH * N2; t += NT) {
          const int fl = t / (CH * N2), qq = (t / N2) % CH, a = t % N2;
          const int q = q0 + qq;
          double out[4] = {0.0, 0.0, 0.0, 0.0};
          if (q < sm.npts[fl]) {
            const int s = a < N ? 0 : 1;
            eval_fn_dir<K, double>(sm.desc[fl][a], sm.lam[fl][q][s], sm.del[fl][s], out);
          }
#pragma unroll
          for (int j = 0; j < L; j++) sm.V[fl][qq][j][a] = out[j];
        }
        __syncthreads();
        // ---- entries: thread t sums entries t, t + NT, ... over the chunk
#pragma unroll
        for (int m = 0; m < NACC; m++) {
          const int t = threadIdx.x + m * NT;
          if (t < FPB * E) {
            const int fl = t / E, e = t % E, a = e / N2, b = e % N2;
            const int nq = min(CH, sm.npts[fl] - q0);
            const double sa = a < N ? 1.0 : -1.0, sb = b < N ? 1.0 : -1.0, sab = sa * sb;
            const double cJ = sab * sm.coef[fl][0], cF = sa * sm.coef[fl][1], cFT = sb * sm.coef[fl][2];
            double cD[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int k = 1; k <= K; k++) cD[k - 1] = sab * sm.coef[fl][2 + k];
            double v = 0.0;
            for (int qq = 0; qq < nq; qq++) {
              const double* Va = &sm.V[fl][qq][0][a];
              const double* Vb = &sm.V[fl][qq][0][b];
              double s = cJ * Va[0] * Vb[0] + cF * Va[0] * Vb[N2] + cFT * Va[N2] * Vb[0];
#pragma unroll
              for (int k = 1; k <= K; k++) s += cD[k - 1] * Va[k * N2] * Vb[k * N2];
              v += sm.w[fl][q0 + qq] * s;
            }
            acc[m].add(v);
          }
        }
        __syncthreads();
      }
    }
    // ---- store (or add to the facet-patch terms' matrix)
#pragma unroll
    for (int m = 0; m < NACC; m++) {
      const int t = threadIdx.x + m * NT;
      if (t < FPB * E) {
        const int fl = t / E, e = t % E;
        const int idx = sm.idx[fl];
        if (idx >= 0) {
          T* dst = famat + (int64_t)idx * E + e;
          const double v = acc[m].get() + (accumulate ? (double)*dst : 0.0);
          if (!finite_bits(v)) set_err(err, XG_ERR_NONFINITE);
          *dst = (T)v;
        }
      }
    }
  }
}

template <int D, int K, typename T>
int launch_t(const SkelLaunch& A, const FormDesc& form, cudaStream_t s) {
  auto k = k_skel<D, K, T>;
  const size_t smem = sizeof(SkSmem<D, K>);
  static std::mutex mu;
  static std::map<int, int> grids;  // per device: blocks per SM x SMs
  int dev = 0;
  XG_CUDA(cudaGetDevice(&dev));
  int grid;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = grids.find(dev);
    if (it == grids.end()) {
      if (smem > 48 * 1024) XG_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      int occ = 0, sms = 0;
      XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, SkCfg<D, K>::NT, smem));
      XG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      it = grids.emplace(dev, (occ > 0 ? occ : 1) * sms).first;
    }
    grid = it->second;
  }
  k<<<grid, SkCfg<D, K>::NT, smem, s>>>(form, A.ne, A.nv, A.elv, A.xyz, A.nf, A.fel, A.lset, A.l_fa, A.counts,
                                        (T*)A.famat, A.cap_fa, A.accumulate, A.err);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_skel");
}

template <typename T>
int launch_k(const SkelLaunch& A, const FormDesc& form, cudaStream_t s) {
  if (A.dim == 2) {
    if (A.order == 1) return launch_t<2, 1, T>(A, form, s);
    if (A.order == 2) return launch_t<2, 2, T>(A, form, s);
    return launch_t<2, 3, T>(A, form, s);
  }
  if (A.order == 1) return launch_t<3, 1, T>(A, form, s);
  if (A.order == 2) return launch_t<3, 2, T>(A, form, s);
  return launch_t<3, 3, T>(A, form, s);
}

}  // namespace

int skel_launch(const SkelLaunch& A, const FormDesc& form, cudaStream_t s) {
  if (form.nskel <= 0) return XG_OK;
  if (A.dim < 2 || A.dim > 3 || A.order < 1 || A.order > 3) return XG_ERR_UNSUPPORTED;
  return A.fp64 ? launch_k<double>(A, form, s) : launch_k<float>(A, form, s);
}

}  // namespace xg

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
// One block takes SB facets at a time: one warp builds their geometry and
// rules into shared memory (lane per facet), then, FPB facets per pass, the
// block evaluates the derivatives of all 2n functions at a chunk of points,
// folds weights, signs and coefficients into one test-side and one
// trial-side vector per distinct trial factor (two for the DG form: s P0 and
// P1), and each thread sums its entries over the chunk in FP64 with one FMA
// per point and factor (fixed order: deterministic).  Each skeleton group
// writes (the first, without patch terms) or adds its matrix.  When the form
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
  static constexpr int N = ndof_el(D, K), N2 = 2 * N, E = N2 * N2, ET = N2 * (N2 + 1) / 2, NT = 256;
  static constexpr int FPB = E >= 512 ? 1 : 512 / E;  // facets per entry pass
  static constexpr int NACC = (FPB * E + NT - 1) / NT;
  // facets whose geometry and rules one warp builds at once (lane per facet),
  // a multiple of FPB
  static constexpr int SB = (D == 3 && K == 3) ? 16 : FPB * (32 / FPB > 0 ? 32 / FPB : 1);
  // points of one facet rule of order 2K: 2D one segment piece of K + 1
  // points; 3D up to three triangle pieces of 3 / 6 / 16 points
  static constexpr int PMAX = D == 2 ? K + 1 : (K == 1 ? 9 : (K == 2 ? 18 : 48));
  static constexpr int CH = PMAX < 16 ? PMAX : 16;  // points per pass
  static constexpr int L = K + 1;                   // derivative orders 0..K (vector kinds: L + 1)
};

template <int D, int K>
struct SkSmem {
  using C = SkCfg<D, K>;
  double lam[C::SB][C::PMAX][2][D + 1];       // barycentrics of the rule points in both elements
  double w[C::SB][C::PMAX];                   // rule weight x facet measure
  double TV[C::FPB][C::CH][C::L + 1][C::N2];  // test-side vectors per point and kind
  double SV[C::FPB][C::CH][C::L + 1][C::N2];  // trial-side vectors
  double del[C::SB][2][D + 1];                // d lambda_i / d n_F in both elements
  double x0[C::SB][2][D];                     // element maps: lambda = Finv (x - x0)
  double Finv[C::SB][2][D][D];
  double X[C::SB][D][3];                      // facet vertices
  double lf[C::SB][D];                        // their level-set values
  double h1[C::SB];
  double coef[C::SB][kSkelKinds];             // the group's coefficients on this facet (0: not defined on)
  int desc[C::SB][C::N2];
  unsigned char ep[C::ET], eq[C::ET];  // upper-triangle entry k -> (row, column)
  int facet[C::SB];
  int idx[C::SB];
  int npts[C::SB];
};

// geometry of facet f into slot fl of the block's shared memory; false if
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

// the group's facet rule of slot fl (its points as barycentrics of both
// elements) and its coefficients on that facet; returns the point count
template <int D, int K>
__device__ int skel_rule(SkSmem<D, K>& sm, int fl, const SkelDesc& G, int* err) {
  constexpr int PMAX = SkCfg<D, K>::PMAX;
  int np = 0;
  const bool on = sm.idx[fl] >= 0 && (!G.defined_on || sk_bit(G.defined_on, sm.facet[fl]));
#pragma unroll
  for (int k = 0; k < kSkelKinds; k++)
    sm.coef[fl][k] =
        on && ((G.used >> k) & 1) ? (G.hpow[k] == 0 ? G.c[k] : G.c[k] * int_pow(sm.h1[fl], G.hpow[k])) : 0.0;
  if (!on) return 0;
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
  return np;
}

template <int D, int K, typename T>
__global__ void __launch_bounds__(256) k_skel(const __grid_constant__ FormDesc form, int ne, int nv,
                                              const int32_t* __restrict__ elv, const double* __restrict__ xyz,
                                              int64_t nf, const int32_t* __restrict__ fel,
                                              const double* __restrict__ lset, const int32_t* __restrict__ l_fa,
                                              const int* __restrict__ counts, T* __restrict__ famat, int64_t cap_fa,
                                              int accumulate, int* __restrict__ err) {
  using C = SkCfg<D, K>;
  constexpr int N = C::N, N2 = C::N2, E = C::E, ET = C::ET, FPB = C::FPB, NT = C::NT, NACC = C::NACC,
                CH = C::CH, SB = C::SB;
  extern __shared__ __align__(16) unsigned char sk_raw[];
  SkSmem<D, K>& sm = *reinterpret_cast<SkSmem<D, K>*>(sk_raw);
  const int count = counts[2];
  if (threadIdx.x == 0) {
    int k = 0;
    for (int a = 0; a < N2; a++)
      for (int b = a; b < N2; b++) {
        sm.ep[k] = (unsigned char)a;
        sm.eq[k] = (unsigned char)b;
        k++;
      }
  }
  for (int sbatch = blockIdx.x; sbatch * SB < count; sbatch += gridDim.x) {
    __syncthreads();
    // ---- geometry of the super-batch's facets (lane per facet)
    if (threadIdx.x < SB) {
      const int fl = threadIdx.x, idx = sbatch * SB + fl;
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
    for (int gq = 0; gq < form.nskel; gq++) {
      const SkelDesc& G = form.s[gq];
      const bool add = gq > 0 || accumulate;  // later groups and the patch terms' matrices: add
      __syncthreads();
      // ---- the group's rule and coefficients on each facet (lane per facet)
      if (threadIdx.x < SB) sm.npts[threadIdx.x] = skel_rule<D, K>(sm, threadIdx.x, G, err);
      __syncthreads();
      // the group's trial-side vector kinds (block uniform): 0 = s P0 (the
      // jump and the transposed flux), 1 = P1 (the flux), 1 + k = s Pk (the
      // k-th derivative jump); each with its test-side combination
      int kinds[2 + K], nk = 0;
      if (G.used & 5) kinds[nk++] = 0;
      if (G.used & 2) kinds[nk++] = 1;
#pragma unroll
      for (int k = 1; k <= K; k++)
        if ((G.used >> (2 + k)) & 1) kinds[nk++] = 1 + k;
      // symmetric group (no flux term, or both fluxes with one coefficient):
      // the upper triangle, mirrored
      const bool sym = (G.used & 6) == 0 || ((G.used & 6) == 6 && G.c[1] == G.c[2] && G.hpow[1] == G.hpow[2]);
      const int EE = sym ? ET : E;
      for (int fb = 0; fb < SB; fb += FPB) {
        int maxpts = 0;
#pragma unroll
        for (int i = 0; i < FPB; i++) maxpts = max(maxpts, sm.npts[fb + i]);
        Acc<double> acc[NACC];
#pragma unroll
        for (int m = 0; m < NACC; m++) acc[m].init();
        for (int q0 = 0; q0 < maxpts; q0 += CH) {
          const int nqc = min(CH, maxpts - q0);
          // ---- per point and function the test / trial vectors of every kind:
          //   kind 0: T = w (cJ s P0 + cFT P1), S = s P0
          //   kind 1: T = w cF s P0,            S = P1
          //   kind 1+k: T = w cDk s Pk,         S = s Pk
          // so that A[a][b] = sum over points and kinds of T[a] S[b]
          for (int t = threadIdx.x; t < FPB * nqc * N2; t += NT) {
            const int fi = t / (nqc * N2), qq = (t / N2) % nqc, a = t % N2;
            const int fl = fb + fi, q = q0 + qq;
            double out[4] = {0.0, 0.0, 0.0, 0.0};
            double w = 0.0;
            if (q < sm.npts[fl]) {
              const int sd = a < N ? 0 : 1;
              eval_fn_dir<K, double>(sm.desc[fl][a], sm.lam[fl][q][sd], sm.del[fl][sd], out);
              w = sm.w[fl][q];
            }
            const double sa = a < N ? 1.0 : -1.0;
            const double* c = sm.coef[fl];
            for (int j = 0; j < nk; j++) {
              const int kd = kinds[j];
              double tv, sv;
              if (kd == 0) {
                tv = w * (c[0] * sa * out[0] + c[2] * out[1]);
                sv = sa * out[0];
              } else if (kd == 1) {
                tv = w * c[1] * sa * out[0];
                sv = out[1];
              } else {
                const double pk = sa * out[kd - 1];
                tv = w * c[kd + 1] * pk;
                sv = pk;
              }
              sm.TV[fi][qq][j][a] = tv;
              sm.SV[fi][qq][j][a] = sv;
            }
          }
          __syncthreads();
          // ---- entries: thread t sums entries t, t + NT, ... over the chunk
#pragma unroll
          for (int m = 0; m < NACC; m++) {
            const int t = threadIdx.x + m * NT;
            if (t < FPB * EE) {
              const int fi = t / EE, e = t % EE;
              const int a = sym ? sm.ep[e] : e / N2, b = sym ? sm.eq[e] : e % N2;
              const int nq = min(nqc, sm.npts[fb + fi] - q0);
              double v = 0.0;
              for (int qq = 0; qq < nq; qq++)
                for (int j = 0; j < nk; j++) v += sm.TV[fi][qq][j][a] * sm.SV[fi][qq][j][b];
              acc[m].add(v);
            }
          }
          __syncthreads();
        }
        // ---- store (or add to what an earlier group or the patch terms wrote)
#pragma unroll
        for (int m = 0; m < NACC; m++) {
          const int t = threadIdx.x + m * NT;
          if (t < FPB * EE) {
            const int fi = t / EE, e = t % EE;
            const int a = sym ? sm.ep[e] : e / N2, b = sym ? sm.eq[e] : e % N2;
            const int idx = sm.idx[fb + fi];
            if (idx >= 0) {
              T* base = famat + (int64_t)idx * E;
              const double r = acc[m].get();
              const double v = r + (add ? (double)base[a * N2 + b] : 0.0);
              if (!finite_bits(v)) set_err(err, XG_ERR_NONFINITE);
              base[a * N2 + b] = (T)v;
              if (sym && a != b) {
                const double v2 = r + (add ? (double)base[b * N2 + a] : 0.0);
                base[b * N2 + a] = (T)v2;
              }
            }
          }
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

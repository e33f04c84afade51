// Space-time element matrices (dCut(lset_st, dt, time_order=...) forms of
// ngsxfem's space-time discretisations, e.g. demos/spacetime/spacetimeDG_unfitted.py:143-168).
//
// Per element the space-time rule of cutint/spacetimecutrule.cpp:106-244 is
// generated on the fly: time cut points (root_finding per vertex), per time
// interval and time quadrature point the level set at that time (with the
// +-1e-14 perturbation), its straight-cut rule or the standard rule.  A
// fixed-time term (tref >= 0, dCut(..., tref=...)) uses the spatial rule of the
// level-set trace at tref.  Space-time shape functions are products
// psi_i(tau) phi_j(x) with the nodal Gauss-Lobatto time basis; local index
// i * nd_space + j.  Terms: c u v, c grad u . grad v, c (b(t) . grad u) v with
// b(t) = b + bc cos(omega t) + bs sin(omega t), t = t0 + dt tau, and
// c v d/dtau u.
#include <mutex>

#include "xg_basis.cuh"
#include "xg_cut.cuh"
#include "xg_internal.h"

namespace xg {

static __constant__ RuleTable c_rules;

int upload_rules_st() {
  XG_CUDA(cudaMemcpyToSymbol(c_rules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

__device__ __forceinline__ bool tbit64(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

template <int D, int K, int KT>
struct StCfg {
  static constexpr int NS = ndof_el(D, K);
  static constexpr int N = NS * (KT + 1);
  static constexpr int EPB = N <= 8 ? 8 : (N <= 20 ? 4 : 2);
  static constexpr int NTF = N * EPB;              // threads of the per-function phases
  static constexpr int NT = (NTF + 31) / 32 * 32;  // whole warps for the contraction
  static constexpr int CH = 4;
  static constexpr int MAXC = (2 * (D + 1) + 1) * 4;  // time intervals x time points
  static constexpr int NACC = (EPB * N * N + NT - 1) / NT;
};

struct StCombo {
  double t, wt;   // reference time and time weight w_t (t1 - t0)
  double l[4];    // level set at t
  int cls;        // CheckIfStraightCut at t
  int npts;
};

template <int D>
struct StGeoS {
  double g[4][3];
  double meas;
  double lst[3 * 4];
  double cut[2 * 4 + 2];
  int ncut;
  int gv[4];
  int elem, slot;
  double coef[kMaxGroups][7];
};

// number of sub-simplices of Decompose for the sign pattern (no FP work)
template <int D>
__device__ __forceinline__ int n_subs(const double* l, int dt) {
  if (dt == XG_IF) {
    int nc = 0;
    for (int i = 0; i <= D; i++)
      for (int j = i + 1; j <= D; j++) nc += d_geq0(l[i]) != d_geq0(l[j]);
    return (D == 3 && nc == 4) ? 2 : 1;
  }
  int nr = 0;
  for (int i = 0; i <= D; i++) nr += (dt == XG_POS && d_geq0(l[i])) || (dt == XG_NEG && d_neg(l[i]));
  if (nr == 1) return 1;
  return D == 2 ? 2 : 3;
}

template <int D, int K, int KT, typename T>
__global__ void __launch_bounds__(StCfg<D, K, KT>::NT) k_st_elmat(int ne, int nv, const int32_t* __restrict__ elv,
                                                                   const double* __restrict__ xyz,
                                                                   const double* __restrict__ lset_st, StFormDesc form,
                                                                   const int32_t* __restrict__ list,
                                                                   const int* __restrict__ count_ptr,
                                                                   const int* __restrict__ slot_base,
                                                                   T* __restrict__ elmat, int* err) {
  using C = StCfg<D, K, KT>;
  constexpr int NS = C::NS, N = C::N, EPB = C::EPB, NT = C::NT, CH = C::CH, MAXC = C::MAXC, NACC = C::NACC;
  constexpr int NF = D + 4;  // Phi, grad Phi (D), dtau Phi, b . grad Phi
  __shared__ StGeoS<D> geo[EPB];
  __shared__ StCombo combo[EPB][MAXC];
  __shared__ int coff[EPB][MAXC + 1];
  __shared__ int ncombo_s[EPB];
  __shared__ double pts[EPB][CH][D + 6];  // lambda (D+1), tau, w, b(t) (3)
  __shared__ T tr[EPB][CH][N][NF];
  __shared__ T te[EPB][CH][N][4];        // w*cM*Phi, w*cL*grad(as factor), w*cC*Phi, w*cT*Phi
  __shared__ int maxpts_s;
  const int count = *count_ptr;
  const int sbase = slot_base ? *slot_base : 0;
  // threads beyond N * EPB only join the contraction
  const bool fth = threadIdx.x < C::NTF;
  const int le = fth ? threadIdx.x / N : 0, a = fth ? threadIdx.x % N : N;
  const int kl = form.kt_l;

  for (int batch = blockIdx.x; batch * EPB < count; batch += gridDim.x) {
    __syncthreads();
    if (threadIdx.x < EPB) {
      StGeoS<D>& G = geo[threadIdx.x];
      const int idx = batch * EPB + threadIdx.x;
      G.elem = idx < count ? list[idx] : -1;
      G.slot = sbase + idx;
      if (G.elem >= 0) {
        const int e = G.elem;
        double xv[D + 1][3];
        for (int v = 0; v <= D; v++) {
          const int vid = elv[(int64_t)v * ne + e];
          G.gv[v] = vid;
          for (int i = 0; i <= kl; i++) G.lst[i * (D + 1) + v] = lset_st[(int64_t)i * nv + vid];
#pragma unroll
          for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
        }
        Geo<D> g;
        make_geo<D>(xv, g);
        G.meas = fabs(g.det);
        double gs[3] = {0, 0, 0};
        for (int aa = 0; aa < D; aa++)
          for (int k = 0; k < 3; k++) {
            G.g[aa][k] = k < D ? g.Finv[aa][k] : 0.0;
            gs[k] += G.g[aa][k];
          }
        for (int k = 0; k < 3; k++) G.g[D][k] = -gs[k];
        G.ncut = time_cuts<D>(kl, G.lst, G.cut);
        double h = -1.0;
        for (int q = 0; q < form.ngroups; q++)
          for (int k = 0; k < 7; k++) {
            const int hp = form.g[q].hpow[k];
            if (hp != 0 && h < 0) h = mesh_h<D>(G.meas);
            G.coef[q][k] = hp == 0 ? form.g[q].c[k] : form.g[q].c[k] * int_pow(h, hp);
          }
      }
    }
    __syncthreads();
    const StGeoS<D>& G = geo[le];
    const int sidx = fth ? a % NS : 0, tidx = fth ? a / NS : 0;
    const int desc = G.elem >= 0 ? fn_desc<D, K>(sidx, G.gv) : 0;
    T gT[D + 1][D];
#pragma unroll
    for (int aa = 0; aa <= D; aa++)
#pragma unroll
      for (int k = 0; k < D; k++) gT[aa][k] = (T)G.g[aa][k];
    Acc<T> acc[NACC];
#pragma unroll
    for (int m = 0; m < NACC; m++) acc[m].init();

    for (int q = 0; q < form.ngroups; q++) {
      const StGroupDesc& Gq = form.g[q];
      const int ps = clamp_order(Gq.order), dt = Gq.domain;
      const int sd = dt == XG_IF ? D - 1 : D;
      const int nqc = c_rules.cnt[sd][ps], offc = c_rules.off[sd][ps];
      const int nqs = c_rules.cnt[D][ps], offs = c_rules.off[D][ps];
      const int pt = clamp_order(form.order_time);
      const int nqt = c_rules.cnt[1][pt], offt = c_rules.off[1][pt];
      const bool fixed = Gq.tref >= 0.0;
      const bool on = G.elem >= 0 && (!Gq.defined_on || tbit64(Gq.defined_on, G.elem));
      const int nco = !on ? 0 : (fixed ? 1 : (G.ncut - 1) * nqt);
      // combos: (time interval, time point) -> level set, classification, #points
      for (int c = a; fth && c < nco; c += N) {
        StCombo& Cb = combo[le][c];
        if (fixed) {
          Cb.t = Gq.tref;
          Cb.wt = 1.0;
          lset_trace<D>(kl, G.lst, Gq.tref, Cb.l);
        } else {
          const int iv = c / nqt, iq = c % nqt;
          const double t0 = G.cut[iv], t1 = G.cut[iv + 1];
          Cb.t = t0 + c_rules.x[offt + iq][0] * (t1 - t0);
          Cb.wt = c_rules.w[offt + iq] * (t1 - t0);
          lset_at<D>(kl, G.lst, Cb.t, Cb.l);
        }
        Cb.cls = check_if_straight_cut(Cb.l, D + 1);
        Cb.npts = Cb.cls == XG_IF ? n_subs<D>(Cb.l, dt) * nqc : (Cb.cls == dt ? nqs : 0);
      }
      __syncthreads();
      if (a == 0) {
        int o = 0;
        for (int c = 0; c < nco; c++) {
          coff[le][c] = o;
          o += combo[le][c].npts;
        }
        coff[le][nco] = o;
        ncombo_s[le] = nco;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        int mx = 0;
        for (int k = 0; k < EPB; k++) mx = max(mx, coff[k][ncombo_s[k]]);
        maxpts_s = mx;
      }
      __syncthreads();
      const int maxpts = maxpts_s, npl = coff[le][ncombo_s[le]];
      const T cM = (T)G.coef[q][XG_TERM_MASS], cL = (T)G.coef[q][XG_TERM_LAPLACE];
      const T cC = (T)G.coef[q][XG_TERM_CONV], cT = (T)G.coef[q][6];
      const int used = Gq.used;
      for (int q0 = 0; q0 < maxpts; q0 += CH) {
        for (int qq = a; fth && qq < CH; qq += N) {
          const int qi = q0 + qq;
          double lam[4] = {0.25, 0.25, 0.25, 0.25}, w = 0.0, tau = 0.0;
          if (qi < npl) {
            int c = 0;
            while (coff[le][c + 1] <= qi) c++;
            const StCombo& Cb = combo[le][c];
            const int k = qi - coff[le][c];
            tau = Cb.t;
            double xi[3];
            if (Cb.cls == XG_IF) {
              Sub subs[3];
              const int ns = decompose<D>(Cb.l, dt, subs);
              if (ns < 0) {
                set_err(err, -ns);
              } else {
                const int s = k / nqc, b = k % nqc;
                plain_point(subs[s], sd + 1, c_rules.x[offc + b], xi);
                w = c_rules.w[offc + b] * simplex_volume(subs[s].p, sd + 1);
                if (dt == XG_IF) {
                  Geo<D> gg;  // interface factor from the stored inverse Jacobian
#pragma unroll
                  for (int r = 0; r < D; r++)
#pragma unroll
                    for (int cc = 0; cc < D; cc++) gg.Finv[r][cc] = G.g[r][cc];
                  w = w * if_factor<D>(gg, Cb.l);
                }
              }
            } else {
              xi[0] = c_rules.x[offs + k][0];
              xi[1] = c_rules.x[offs + k][1];
              xi[2] = c_rules.x[offs + k][2];
              w = c_rules.w[offs + k];
            }
            w = w * Cb.wt * G.meas;
            double s3 = 0;
            for (int r = 0; r < D; r++) {
              lam[r] = xi[r];
              s3 += xi[r];
            }
            lam[D] = 1.0 - s3;
          }
          for (int r = 0; r <= D; r++) pts[le][qq][r] = lam[r];
          pts[le][qq][D + 1] = tau;
          pts[le][qq][D + 2] = w;
          double bt[3] = {Gq.b[0], Gq.b[1], Gq.b[2]};
          if ((used & (1 << XG_TERM_CONV)) && Gq.omega != 0.0) {
            const double tp = Gq.t0 + Gq.dt * tau;
            const double cs = cos(Gq.omega * tp), sn = sin(Gq.omega * tp);
            for (int r = 0; r < 3; r++) bt[r] += Gq.bc[r] * cs + Gq.bs[r] * sn;
          }
          for (int r = 0; r < 3; r++) pts[le][qq][D + 3 + r] = bt[r];
        }
        __syncthreads();
#pragma unroll
        for (int qq = 0; qq < (fth ? CH : 0); qq++) {
          T lam[D + 1];
#pragma unroll
          for (int r = 0; r <= D; r++) lam[r] = (T)pts[le][qq][r];
          T phi, grad[D];
          eval_fn<D, T>(desc, lam, gT, phi, grad);
          T psi[3], dpsi[3];
          time_basis<T>(KT, (T)pts[le][qq][D + 1], psi, dpsi);
          const T ps_ = psi[tidx], dps = dpsi[tidx];
          const T w = (T)pts[le][qq][D + 2];
          const T Phi = ps_ * phi;
          tr[le][qq][a][0] = Phi;
          T bg = 0;
#pragma unroll
          for (int k = 0; k < D; k++) {
            const T gk = ps_ * grad[k];
            tr[le][qq][a][1 + k] = gk;
            bg += (T)pts[le][qq][D + 3 + k] * gk;
          }
          tr[le][qq][a][1 + D] = dps * phi;
          tr[le][qq][a][2 + D] = bg;
          te[le][qq][a][0] = (used & (1 << XG_TERM_MASS)) ? w * cM * Phi : (T)0;
          te[le][qq][a][1] = (used & (1 << XG_TERM_LAPLACE)) ? w * cL : (T)0;
          te[le][qq][a][2] = (used & (1 << XG_TERM_CONV)) ? w * cC * Phi : (T)0;
          te[le][qq][a][3] = (used & (1 << 6)) ? w * cT * Phi : (T)0;
        }
        __syncthreads();
        const int nch = min(CH, maxpts - q0);
#pragma unroll
        for (int m = 0; m < NACC; m++) {
          const int t = threadIdx.x + m * NT;
          if (t < EPB * N * N) {
            const int el = t / (N * N), k = t % (N * N), pp = k / N, qv = k % N;
            T v = 0;
            for (int qq = 0; qq < nch; qq++) {
              const T* A = te[el][qq][pp];
              const T* B = tr[el][qq][qv];
              const T* Bp = tr[el][qq][pp];
              T lap = 0;
#pragma unroll
              for (int kk = 1; kk <= D; kk++) lap += Bp[kk] * B[kk];
              v += A[0] * B[0] + A[1] * lap + A[2] * B[2 + D] + A[3] * B[1 + D];
            }
            acc[m].add(v);
          }
        }
        __syncthreads();
      }
    }
#pragma unroll
    for (int m = 0; m < NACC; m++) {
      const int t = threadIdx.x + m * NT;
      if (t < EPB * N * N) {
        const int el = t / (N * N), k = t % (N * N);
        if (geo[el].elem >= 0) {
          const T v = acc[m].get();
          if (!isfinite(v)) set_err(err, XG_ERR_NONFINITE);
          elmat[(int64_t)geo[el].slot * N * N + k] = v;
        }
      }
    }
  }
}

// P1 in space: the moment form.  With the spatial functions the barycentrics
// lambda_j, every term's spatial integral at a time point is a combination
// of the measure mu, the first moments mu_j = int lambda_j and the second
// moments mu_jk = int lambda_j lambda_k of the part at that time point:
//   mass       c psi_i psi_i' mu_jj'
//   Laplace    c psi_i psi_i' mu (grad lambda_j . grad lambda_j')
//   convection c psi_i psi_i' mu_j (b(t) . grad lambda_j')
//   d/dtau     c psi_i dpsi_i' mu_jj'
// (test (i, j), trial (i', j')).  One thread per prism: the time cuts, per
// (time interval, time point) the level set, the part's rule points (the
// straight cut of Decompose or the standard rule, as the quadrature-point
// kernel above) summed into the moments, then the entries; FP64 throughout.
template <int D, int KT, typename T>
__global__ void __launch_bounds__(128) k_st_elmat_p1(int ne, int nv, const int32_t* __restrict__ elv,
                                                     const double* __restrict__ xyz,
                                                     const double* __restrict__ lset_st, StFormDesc form,
                                                     const int32_t* __restrict__ list,
                                                     const int* __restrict__ count_ptr,
                                                     const int* __restrict__ slot_base, T* __restrict__ elmat,
                                                     int* err) {
  constexpr int NS = D + 1, NTB = KT + 1, N = NS * NTB, NM = NS * (NS + 1) / 2;
  const int count = *count_ptr;
  const int sbase = slot_base ? *slot_base : 0;
  const int kl = form.kt_l;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < count; idx += gridDim.x * blockDim.x) {
    const int e = list[idx];
    double xv[D + 1][3], lst[3 * 4];
    for (int v = 0; v <= D; v++) {
      const int vid = elv[(int64_t)v * ne + e];
      for (int i = 0; i <= kl; i++) lst[i * (D + 1) + v] = lset_st[(int64_t)i * nv + vid];
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
    }
    Geo<D> g;
    make_geo<D>(xv, g);
    const double meas = fabs(g.det);
    double gl[D + 1][D];  // physical gradients of the barycentrics
    for (int k = 0; k < D; k++) {
      double sg = 0.0;
      for (int a = 0; a < D; a++) {
        gl[a][k] = g.Finv[a][k];
        sg += g.Finv[a][k];
      }
      gl[D][k] = -sg;
    }
    double cut[2 * 4 + 2];
    const int ncut = time_cuts<D>(kl, lst, cut);
    double GG[NM];  // grad lambda_j . grad lambda_k, j <= k
    {
      int k2 = 0;
      for (int j = 0; j < NS; j++)
        for (int jj = j; jj < NS; jj++) {
          double sg = 0.0;
          for (int k = 0; k < D; k++) sg += gl[j][k] * gl[jj][k];
          GG[k2++] = sg;
        }
    }
    double A[N * N];
    for (int k = 0; k < N * N; k++) A[k] = 0.0;
    double h = -1.0;
    for (int q = 0; q < form.ngroups; q++) {
      const StGroupDesc& Gq = form.g[q];
      if (Gq.defined_on && !tbit64(Gq.defined_on, e)) continue;
      double cf[7];
      for (int k = 0; k < 7; k++) {
        const int hp = Gq.hpow[k];
        if (hp != 0 && h < 0) h = mesh_h<D>(meas);
        cf[k] = hp == 0 ? Gq.c[k] : Gq.c[k] * int_pow(h, hp);
      }
      const bool uM = (Gq.used >> XG_TERM_MASS) & 1, uL = (Gq.used >> XG_TERM_LAPLACE) & 1;
      const bool uC = (Gq.used >> XG_TERM_CONV) & 1, uT = (Gq.used >> 6) & 1;
      const int ps = clamp_order(Gq.order), dt = Gq.domain;
      const int sd = dt == XG_IF ? D - 1 : D;
      const int nqc = c_rules.cnt[sd][ps], offc = c_rules.off[sd][ps];
      const int nqs = c_rules.cnt[D][ps], offs = c_rules.off[D][ps];
      const int pt = clamp_order(form.order_time);
      const int nqt = c_rules.cnt[1][pt], offt = c_rules.off[1][pt];
      const bool fixed = Gq.tref >= 0.0;
      const int nco = fixed ? 1 : (ncut - 1) * nqt;
      for (int c = 0; c < nco; c++) {
        double t, wt, l[4];
        if (fixed) {
          t = Gq.tref;
          wt = 1.0;
          lset_trace<D>(kl, lst, Gq.tref, l);
        } else {
          const int iv = c / nqt, iq = c % nqt;
          const double t0 = cut[iv], t1 = cut[iv + 1];
          t = t0 + c_rules.x[offt + iq][0] * (t1 - t0);
          wt = c_rules.w[offt + iq] * (t1 - t0);
          lset_at<D>(kl, lst, t, l);
        }
        const int cls = check_if_straight_cut(l, D + 1);
        if (cls != XG_IF && cls != dt) continue;
        // the part's moments at this time point (reference measure)
        double mu = 0.0, m1[NS], m2[NM];
        for (int j = 0; j < NS; j++) m1[j] = 0.0;
        for (int j = 0; j < NM; j++) m2[j] = 0.0;
        auto point = [&](const double* xi, double w) {
          double lam[NS], sl = 0.0;
          for (int r = 0; r < D; r++) {
            lam[r] = xi[r];
            sl += xi[r];
          }
          lam[D] = 1.0 - sl;
          mu += w;
          int k = 0;
          for (int j = 0; j < NS; j++) {
            const double wl = w * lam[j];
            m1[j] += wl;
            for (int jj = j; jj < NS; jj++) m2[k++] += wl * lam[jj];
          }
        };
        if (cls == XG_IF) {
          Sub subs[3];
          const int ns = decompose<D>(l, dt, subs);
          if (ns < 0) {
            set_err(err, -ns);
            continue;
          }
          const double fac = dt == XG_IF ? if_factor<D>(g, l) : 1.0;
          for (int s2 = 0; s2 < ns; s2++) {
            const double vol = simplex_volume(subs[s2].p, sd + 1) * fac;
            for (int b = 0; b < nqc; b++) {
              double xi[3];
              plain_point(subs[s2], sd + 1, c_rules.x[offc + b], xi);
              point(xi, c_rules.w[offc + b] * vol);
            }
          }
        } else {
          for (int b = 0; b < nqs; b++) point(c_rules.x[offs + b], c_rules.w[offs + b]);
        }
        // time basis at t, the convection field b(t)
        double psi[3], dpsi[3];
        time_basis<double>(KT, t, psi, dpsi);
        double bt[3] = {Gq.b[0], Gq.b[1], Gq.b[2]};
        if (uC && Gq.omega != 0.0) {
          const double tp = Gq.t0 + Gq.dt * t;
          const double cs = cos(Gq.omega * tp), sn = sin(Gq.omega * tp);
          for (int r = 0; r < 3; r++) bt[r] += Gq.bc[r] * cs + Gq.bs[r] * sn;
        }
        double bg[NS];  // b(t) . grad lambda_j
        for (int j = 0; j < NS; j++) {
          double sb = 0.0;
          for (int k = 0; k < D; k++) sb += bt[k] * gl[j][k];
          bg[j] = sb;
        }
        const double W = wt * meas;
        // the time factors W psi_i psi_i' and W psi_i dpsi_i'
        double PP[NTB][NTB], PD[NTB][NTB];
        for (int i = 0; i < NTB; i++)
          for (int ii = 0; ii < NTB; ii++) {
            PP[i][ii] = W * psi[i] * psi[ii];
            PD[i][ii] = W * psi[i] * dpsi[ii];
          }
        const double cM = uM ? cf[XG_TERM_MASS] : 0.0, cL = uL ? cf[XG_TERM_LAPLACE] * mu : 0.0;
        const double cC = uC ? cf[XG_TERM_CONV] : 0.0, cT = uT ? cf[6] : 0.0;
        for (int j = 0; j < NS; j++)
          for (int jj = 0; jj < NS; jj++) {
            const int lo = j < jj ? j : jj, hi = j < jj ? jj : j;
            const int kk = lo * NS - lo * (lo - 1) / 2 + (hi - lo);
            const double sM = cM * m2[kk] + cL * GG[kk] + cC * m1[j] * bg[jj];
            const double sT = cT * m2[kk];
            for (int i = 0; i < NTB; i++)
              for (int ii = 0; ii < NTB; ii++)
                A[(i * NS + j) * N + ii * NS + jj] += PP[i][ii] * sM + PD[i][ii] * sT;
          }
      }
    }
    T* out = elmat + (int64_t)(sbase + idx) * N * N;
    for (int k = 0; k < N * N; k++) {
      if (!finite_bits(A[k])) set_err(err, XG_ERR_NONFINITE);
      out[k] = (T)A[k];
    }
  }
}

template <int D, int K, int KT, typename T>
static int launch_one(const StLaunch& a, cudaStream_t s) {
  if (K == 1) {
    const int grid = 152 * 16;
    k_st_elmat_p1<D, KT, T><<<grid, 128, 0, s>>>(a.ne, a.nv, a.elv, a.xyz, a.lset_st, a.desc, a.list, a.count,
                                                 a.slot_base, (T*)a.elmat, a.err);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_st_elmat_p1");
  }
  using C = StCfg<D, K, KT>;
  auto kern = k_st_elmat<D, K, KT, T>;
  static int grid[2] = {0, 0};
  int& g = grid[sizeof(T) == 8];
  if (!g) {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, C::NT, 0);
    g = nsm * (per < 1 ? 1 : per);
  }
  kern<<<g, C::NT, 0, s>>>(a.ne, a.nv, a.elv, a.xyz, a.lset_st, a.desc, a.list, a.count, a.slot_base, (T*)a.elmat,
                           a.err);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_st_elmat");
}

template <typename T>
static int launch_t(const StLaunch& a, cudaStream_t s) {
  if (a.D == 2) {
    if (a.K == 1) return a.KT == 1 ? launch_one<2, 1, 1, T>(a, s) : launch_one<2, 1, 2, T>(a, s);
    return a.KT == 1 ? launch_one<2, 2, 1, T>(a, s) : launch_one<2, 2, 2, T>(a, s);
  }
  if (a.K == 1) return a.KT == 1 ? launch_one<3, 1, 1, T>(a, s) : launch_one<3, 1, 2, T>(a, s);
  return a.KT == 1 ? launch_one<3, 2, 1, T>(a, s) : launch_one<3, 2, 2, T>(a, s);
}

int launch_st_elmat(const StLaunch& a, cudaStream_t s) {
  if (a.K < 1 || a.K > 2 || a.KT < 1 || a.KT > 2) {
    set_last_error("space-time forms: space order 1..2 and time order 1..2");
    return XG_ERR_UNSUPPORTED;
  }
  return a.precision == XG_PREC_FP64 ? launch_t<double>(a, s) : launch_t<float>(a, s);
}

}  // namespace xg

// Volume terms of bilinear forms with a coefficient field: the integrand of a
// menu kind (mass, Laplace, the Nitsche normal terms, convection, the
// normal-normal stiffness (n . grad u)(n . grad v) of TraceFEM) times
// c h^p x^e gf(x), gf a GridFunction of an H1 space on the form's mesh.  The
// reference evaluates its CoefficientFunction at the points of the cut rule
// and contracts (xfem/symboliccutbfi.cpp:76-313, the evaluation at
// :168-194); the rule is StraightCutIntegrationRule
// (cutint/straightcutrule.cpp:582-677: the standard rule on uncut elements of
// the term's domain, the sub-simplices of Decompose on cut ones, the
// interface factor for IF; domain XG_WHOLE, dx(definedonelements=...): the
// element's own rule), with the rule code of xg_cut.cuh.  Thread per
// active element, FP64 sums added to the element's rows after the volume
// kernels wrote them (one thread owns an element's rows: no atomics, a fixed
// order).
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "xg_basis.cuh"
#include "xg_cut.cuh"
#include "xg_internal.h"
#include "xg_isomesh.cuh"

namespace xg {

static __device__ RuleTable g_cf_rules;

int upload_rules_cform() {
  XG_CUDA(cudaMemcpyToSymbol(g_cf_rules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

__device__ __forceinline__ bool cf_bit64(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }
__device__ __forceinline__ bool cf_bit32(const uint32_t* b, int64_t i) { return (b[i >> 5] >> (i & 31)) & 1u; }

__device__ __forceinline__ double cf_ipow(double x, int e) {
  double r = 1.0;
  for (int k = 0; k < e; k++) r *= x;
  return r;
}

// does term T contribute on element e of domain type dom (XG_WHOLE: the
// whole element, cut or not)
__device__ __forceinline__ bool term_on(const CoefTermDev& T, int64_t e, int dom) {
  if (T.defined_on && !cf_bit64(T.defined_on, e)) return false;
  return dom == XG_IF || dom == T.domain || T.domain == XG_WHOLE;
}

// descriptor of local function i of an H1 element of runtime order k
template <int D>
__device__ __forceinline__ int desc_rt(int k, int i, const int* gv) {
  return k == 1 ? fn_desc<D, 1>(i, gv) : (k == 2 ? fn_desc<D, 2>(i, gv) : fn_desc<D, 3>(i, gv));
}

// elements with a coefficient term join the active elements (in the uncut
// list unless they are listed as cut already); a warp owns one bit word
__global__ void k_coef_active(int ne, const uint8_t* __restrict__ dom, CoefDesc d, uint32_t* __restrict__ act_un,
                              const uint32_t* __restrict__ act_cut, int64_t nw32) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool add = false;
  if (e < ne && !cf_bit32(act_cut, e)) {
    const int de = dom[e];
    for (int t = 0; t < d.n && !add; t++) add = term_on(d.t[t], e, de);
  }
  const unsigned m = __ballot_sync(0xffffffffu, add);
  if ((threadIdx.x & 31) == 0 && m && (e >> 5) < nw32) act_un[e >> 5] |= m;
}

template <int D, int K, typename T>
__global__ void __launch_bounds__(128) k_coef_elmat(CoefFormLaunch L) {
  constexpr int N = ndof_el(D, K);
  const int n_un = L.counts[0], n = n_un + L.counts[1];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int e = i < n_un ? L.l_un[i] : L.l_cut[i - n_un];
    double xv[4][3], l[4];
    int gv[4] = {0, 0, 0, 0};
    for (int v = 0; v <= D; v++) {
      gv[v] = L.elv[(int64_t)v * L.ne + e];
      l[v] = L.lset[gv[v]];
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? L.xyz[(int64_t)c * L.nv + gv[v]] : 0.0;
    }
    const int cdom = check_if_straight_cut(l, D + 1);
    bool any = false;
    for (int t = 0; t < L.d.n; t++) any |= term_on(L.d.t[t], e, cdom);
    if (!any) continue;
    Geo<D> g;
    make_geo<D>(xv, g);
    const double meas = fabs(g.det), h = mesh_h<D>(meas);
    // physical gradients of the barycentrics, the level set's unit normal
    double gl[D + 1][D], nrm[D];
    double nn = 0.0;
    for (int k = 0; k < D; k++) {
      double s = 0.0, sl = 0.0;
      for (int a = 0; a < D; a++) {
        gl[a][k] = g.Finv[a][k];
        s += g.Finv[a][k];
        sl += g.Finv[a][k] * (l[a] - l[D]);
      }
      gl[D][k] = -s;
      nrm[k] = sl;
      nn += sl * sl;
    }
    {
      const double inv = 1.0 / sqrt(nn);
      for (int k = 0; k < D; k++) nrm[k] *= inv;
    }
    int desc[N];
    for (int a = 0; a < N; a++) desc[a] = fn_desc<D, K>(a, gv);
    double A[N * N];
    for (int k = 0; k < N * N; k++) A[k] = 0.0;
    for (int t = 0; t < L.d.n; t++) {
      const CoefTermDev& Tm = L.d.t[t];
      if (!term_on(Tm, e, cdom)) continue;
      const double c = Tm.hpow == 0 ? Tm.coef : Tm.coef * int_pow(h, Tm.hpow);
      // the coefficient field on this element
      const int kg = Tm.gf_order, ng = kg > 0 ? ndof_el(D, kg) : 0;
      double cg[20];
      int dg[20];
      for (int a = 0; a < ng; a++) {
        cg[a] = Tm.gf[Tm.gf_dofs[(int64_t)a * L.ne + e]];
        dg[a] = desc_rt<D>(kg, a, gv);
      }
      // the deformation in the reference frame: theta_j = J^-1 gdef(edge j)
      const bool deformed = Tm.gdef != nullptr;
      double theta[6][3];
      if (deformed) {
        constexpr int NE = D == 2 ? 3 : 6;
        for (int j = 0; j < NE; j++) {
          const int ed = L.el_edges[(int64_t)j * L.ne + e];
          for (int r = 0; r < 3; r++) {
            double sr = 0.0;
            if (r < D)
              for (int k = 0; k < D; k++) sr += g.Finv[r][k] * Tm.gdef[(int64_t)ed * 3 + k];
            theta[j][r] = sr;
          }
        }
      }
      // the integrand at reference point xi with weight W (physical measure
      // included), physical barycentric gradients gp, unit normal np,
      // physical point xp and the coefficient cp
      auto point = [&](const double* xi, double W, const double (*gp)[D], const double* np, const double* xp,
                       double cp) {
        double lam[D + 1], sl = 0.0;
        for (int k = 0; k < D; k++) {
          lam[k] = xi[k];
          sl += xi[k];
        }
        lam[D] = 1.0 - sl;
        double f = 1.0;
        if (ng > 0) {
          f = 0.0;
          for (int a = 0; a < ng; a++) f += cg[a] * eval_fn_value<D, double>(dg[a], lam);
        }
        if (Tm.e[0] | Tm.e[1] | Tm.e[2])
          f *= cf_ipow(xp[0], Tm.e[0]) * cf_ipow(xp[1], Tm.e[1]) * (D == 3 ? cf_ipow(xp[2], Tm.e[2]) : 1.0);
        double phi[N], gr[N][D], dn[N];
        for (int a = 0; a < N; a++) {
          eval_fn<D, double>(desc[a], lam, gp, phi[a], gr[a]);
          double sd = 0.0;
          for (int k = 0; k < D; k++) sd += (Tm.kind == XG_TERM_CONV ? Tm.b[k] : np[k]) * gr[a][k];
          dn[a] = sd;
        }
        const double Wt = W * cp * f;
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
              case XG_TERM_U_NGRADV: v = phi[b] * dn[a]; break;
              case XG_TERM_NGRADU_NGRADV: v = dn[b] * dn[a]; break;
              default: v = dn[b] * phi[a]; break;  // XG_TERM_NGRADU_V, XG_TERM_CONV
            }
            A[a * N + b] += Wt * v;
          }
      };
      const double ifac = Tm.domain == XG_IF && cdom == XG_IF && !deformed ? if_factor<D>(g, l) : 1.0;
      // rule point xi of the reference element with reference weight wr
      auto ref_point = [&](const double* xi, double wr) {
        if (!deformed) {
          double xp[3] = {0.0, 0.0, 0.0};
          for (int r = 0; r < D; r++) {
            double sr = g.x0[r];
            for (int k = 0; k < D; k++) sr += g.F[r][k] * xi[k];
            xp[r] = sr;
          }
          point(xi, wr * meas * ifac, gl, nrm, xp, c);
          return;
        }
        double y[3], Am[3][3], F[3][3], Fi[3][3], detF;
        iso::deform_at<D>(theta, xi, y, Am);
        for (int r = 0; r < 3; r++)
          for (int k = 0; k < 3; k++) {
            double sr = 0.0;
            for (int q = 0; q < 3; q++) sr += (r < D && q < D ? g.F[r][q] : (r == q ? 1.0 : 0.0)) * Am[q][k];
            F[r][k] = sr;
          }
        if (!iso::invert<D>(F, Fi, &detF)) {
          set_err(L.err, XG_ERR_NONFINITE);
          return;
        }
        const double adet = fabs(detF);
        // physical gradients: Fi^T times the reference gradients
        double gp[D + 1][D], np[D];
        double nn2 = 0.0;
        for (int k = 0; k < D; k++) {
          double sa = 0.0, sn = 0.0;
          for (int a = 0; a < D; a++) {
            gp[a][k] = Fi[a][k];
            sa += Fi[a][k];
            sn += Fi[a][k] * (l[a] - l[D]);
          }
          gp[D][k] = -sa;
          np[k] = sn;
          nn2 += sn * sn;
        }
        const double inv = 1.0 / sqrt(nn2);
        for (int k = 0; k < D; k++) np[k] *= inv;
        double w = wr * adet;
        if (Tm.domain == XG_IF) {
          // |F^-T n_ref|, n_ref the unit reference gradient of the level set
          double gr2 = 0.0;
          for (int k = 0; k < D; k++) gr2 += (l[k] - l[D]) * (l[k] - l[D]);
          w *= sqrt(nn2 / gr2);
        }
        double xp[3] = {0.0, 0.0, 0.0};
        for (int r = 0; r < D; r++) {
          double sr = g.x0[r];
          for (int k = 0; k < D; k++) sr += g.F[r][k] * y[k];
          xp[r] = sr;
        }
        const double cp = Tm.hpow == 0 ? Tm.coef : Tm.coef * int_pow(mesh_h<D>(adet), Tm.hpow);
        point(xi, w, gp, np, xp, cp);
      };
      const int p = clamp_order(Tm.order);
      if (cdom != XG_IF || Tm.domain == XG_WHOLE) {
        const int off = g_cf_rules.off[D][p], cnt = g_cf_rules.cnt[D][p];
        for (int q = 0; q < cnt; q++) ref_point(g_cf_rules.x[off + q], g_cf_rules.w[off + q]);
        continue;
      }
      Sub subs[3];
      const int ns = decompose<D>(l, Tm.domain, subs);
      if (ns < 0) {
        set_err(L.err, -ns);
        continue;
      }
      const int sd = Tm.domain == XG_IF ? D - 1 : D;
      const int off = g_cf_rules.off[sd][p], cnt = g_cf_rules.cnt[sd][p];
      for (int s = 0; s < ns; s++) {
        const double trafofac = simplex_volume(subs[s].p, sd + 1);
        for (int q = 0; q < cnt; q++) {
          double pt[3];
          plain_point(subs[s], sd + 1, g_cf_rules.x[off + q], pt);
          ref_point(pt, g_cf_rules.w[off + q] * trafofac);
        }
      }
    }
    for (int a = 0; a < N; a++) {
      T* row = (T*)L.elmat + (int64_t)L.rowslot[(int64_t)e * N + a] * N;
      for (int b = 0; b < N; b++) {
        const double v = (double)row[b] + A[a * N + b];
        if (!finite_bits(v)) set_err(L.err, XG_ERR_NONFINITE);
        row[b] = (T)v;
      }
    }
  }
}

template <int D, int K, typename T>
int launch_t(const CoefFormLaunch& L, cudaStream_t s) {
  k_coef_elmat<D, K, T><<<152 * 8, 128, 0, s>>>(L);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_coef_elmat");
}

template <typename T>
int launch_k(const CoefFormLaunch& L, cudaStream_t s) {
  if (L.dim == 2) {
    if (L.order == 1) return launch_t<2, 1, T>(L, s);
    if (L.order == 2) return launch_t<2, 2, T>(L, s);
    return launch_t<2, 3, T>(L, s);
  }
  if (L.order == 1) return launch_t<3, 1, T>(L, s);
  if (L.order == 2) return launch_t<3, 2, T>(L, s);
  return launch_t<3, 3, T>(L, s);
}

// MapPatchIntegrationPoint (symboliccutbfi.cpp:1747-1846) on the deformed
// maps: the point xi_from of element `from` sent into element `to` (low-order
// guess from the vertex positions, which the deformation keeps, then Newton
// with the deformed Jacobian, at most 15 steps to 1e-12 sqrt(det)); returns
// |det (J A)| of `from` at the point
template <int D>
__device__ double map_patch_def(const Geo<D>& gf, const double (*thf)[3], const Geo<D>& gt, const double (*tht)[3],
                                const double* xi_from, double* xi_to) {
  double y[3], Am[3][3], F[3][3], Fi[3][3], vec[3] = {0.0, 0.0, 0.0}, det_from;
  iso::deform_at<D>(thf, xi_from, y, Am);
  for (int r = 0; r < 3; r++)
    for (int k = 0; k < 3; k++) {
      double sr = 0.0;
      if (r < D && k < D)
        for (int q = 0; q < D; q++) sr += gf.F[r][q] * Am[q][k];
      F[r][k] = r < D && k < D ? sr : (r == k ? 1.0 : 0.0);
    }
  for (int r = 0; r < D; r++) {
    double sr = gf.x0[r];
    for (int k = 0; k < D; k++) sr += gf.F[r][k] * y[k];
    vec[r] = sr;
  }
  iso::invert<D>(F, Fi, &det_from);
  const double h = sqrt(det_from);  // NaN for a negative determinant: one step, as in the affine statement
  double x00[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < D; i++) {
    double sr = 0.0;
    for (int k = 0; k < D; k++) sr += gt.Finv[i][k] * (vec[k] - gt.x0[k]);
    x00[i] = sr;
  }
  double x0[3] = {x00[0], x00[1], x00[2]};
  int its = 0;
  double diffn = 0.0;
  while (its == 0 || (diffn > 1e-12 * h && its < 15)) {
    double yt[3], At[3][3], Ft[3][3], Fti[3][3], dt;
    iso::deform_at<D>(tht, x0, yt, At);
    double diff[3] = {0.0, 0.0, 0.0};
    for (int r = 0; r < D; r++) {
      double sr = gt.x0[r];
      for (int k = 0; k < D; k++) sr += gt.F[r][k] * yt[k];
      diff[r] = vec[r] - sr;
    }
    for (int r = 0; r < 3; r++)
      for (int k = 0; k < 3; k++) {
        double sr = 0.0;
        if (r < D && k < D)
          for (int q = 0; q < D; q++) sr += gt.F[r][q] * At[q][k];
        Ft[r][k] = r < D && k < D ? sr : (r == k ? 1.0 : 0.0);
      }
    iso::invert<D>(Ft, Fti, &dt);
    diffn = 0.0;
    for (int i = 0; i < D; i++) diffn += diff[i] * diff[i];
    diffn = sqrt(diffn);
    for (int i = 0; i < D; i++) {
      double sr = 0.0;
      for (int k = 0; k < D; k++) sr += Fti[i][k] * diff[k];
      x0[i] += sr;
    }
    its++;
  }
  double dist = 0.0;
  for (int i = 0; i < D; i++) dist += (x0[i] - x00[i]) * (x0[i] - x00[i]);
  dist = sqrt(dist);
  const bool fail = its >= 15 || diffn > 1e-12 * h || dist > 10.0;
  for (int i = 0; i < 3; i++) xi_to[i] = fail ? x00[i] : x0[i];
  return fabs(det_from);
}

// facet-patch terms on the deformed mesh, thread per active facet: both
// elements' rules of the term's order, every point mapped into the other
// element, c (u1 - u2)(v1 - v2) with the point's physical weight, written as
// the facet slot's full rows (in place of the affine patch kernels)
template <int D, int K, typename T>
__global__ void __launch_bounds__(64) k_patch_def(PatchDefLaunch L) {
  constexpr int N = ndof_el(D, K), N2 = 2 * N, NE = D == 2 ? 3 : 6;
  const int count = L.counts[2];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count && i < L.cap_fa; i += gridDim.x * blockDim.x) {
    const int f = L.l_fa[i];
    const int e[2] = {L.fel[f], L.fel[L.nf + f]};
    Geo<D> g[2];
    int gv[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    double th[2][6][3];
    for (int sd = 0; sd < 2; sd++) {
      double xv[4][3];
      for (int v = 0; v <= D; v++) {
        gv[sd][v] = L.elv[(int64_t)v * L.ne + e[sd]];
        for (int c = 0; c < 3; c++) xv[v][c] = c < D ? L.xyz[(int64_t)c * L.nv + gv[sd][v]] : 0.0;
      }
      make_geo<D>(xv, g[sd]);
      for (int j = 0; j < 6; j++)
        for (int r = 0; r < 3; r++) {
          double sr = 0.0;
          if (j < NE && r < D) {
            const int ed = L.el_edges[(int64_t)j * L.ne + e[sd]];
            for (int k = 0; k < D; k++) sr += g[sd].Finv[r][k] * L.gdef[(int64_t)ed * 3 + k];
          }
          th[sd][j][r] = sr;
        }
    }
    int desc[2][N];
    for (int a = 0; a < N; a++) {
      desc[0][a] = fn_desc<D, K>(a, gv[0]);
      desc[1][a] = fn_desc<D, K>(a, gv[1]);
    }
    double A[N2 * N2];
    for (int k = 0; k < N2 * N2; k++) A[k] = 0.0;
    const double h1 = mesh_h<D>(fabs(g[0].det));
    for (int pp = 0; pp < L.npatch; pp++) {
      const PatchDesc& P = L.p[pp];
      if (P.defined_on && !cf_bit64(P.defined_on, f)) continue;
      const double c = P.hpow == 0 ? P.c : P.c * int_pow(h1, P.hpow);
      const int o = clamp_order(P.order), off = g_cf_rules.off[D][o], cnt = g_cf_rules.cnt[D][o];
      for (int l = 0; l < 2 * cnt; l++) {
        const int sd = l < cnt ? 0 : 1, q = l < cnt ? l : l - cnt;
        const double* xi = g_cf_rules.x[off + q];
        double xo[3];
        const double W = g_cf_rules.w[off + q] * c * map_patch_def<D>(g[sd], th[sd], g[1 - sd], th[1 - sd], xi, xo);
        const double* x1 = sd == 0 ? xi : xo;
        const double* x2 = sd == 0 ? xo : xi;
        double lam1[D + 1], lam2[D + 1], s1 = 0.0, s2 = 0.0;
        for (int k = 0; k < D; k++) {
          lam1[k] = x1[k];
          lam2[k] = x2[k];
          s1 += x1[k];
          s2 += x2[k];
        }
        lam1[D] = 1.0 - s1;
        lam2[D] = 1.0 - s2;
        double sh[N2];
        for (int a = 0; a < N; a++) {
          sh[a] = eval_fn_value<D, double>(desc[0][a], lam1);
          sh[N + a] = -eval_fn_value<D, double>(desc[1][a], lam2);
        }
        for (int a = 0; a < N2; a++)
          for (int b = 0; b < N2; b++) A[a * N2 + b] += W * sh[a] * sh[b];
      }
    }
    T* out = (T*)L.famat + (int64_t)i * N2 * N2;
    for (int k = 0; k < N2 * N2; k++) {
      if (!finite_bits(A[k])) set_err(L.err, XG_ERR_NONFINITE);
      out[k] = (T)A[k];
    }
  }
}

template <int D, int K, typename T>
int launch_pd(const PatchDefLaunch& L, cudaStream_t s) {
  k_patch_def<D, K, T><<<152 * 8, 64, 0, s>>>(L);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_patch_def");
}

template <typename T>
int launch_pdk(const PatchDefLaunch& L, cudaStream_t s) {
  if (L.dim == 2) {
    if (L.order == 1) return launch_pd<2, 1, T>(L, s);
    if (L.order == 2) return launch_pd<2, 2, T>(L, s);
    return launch_pd<2, 3, T>(L, s);
  }
  if (L.order == 1) return launch_pd<3, 1, T>(L, s);
  if (L.order == 2) return launch_pd<3, 2, T>(L, s);
  return launch_pd<3, 3, T>(L, s);
}

}  // namespace

int patch_def_launch(const PatchDefLaunch& L, cudaStream_t s) {
  if (L.dim < 2 || L.dim > 3 || L.order < 1 || L.order > 3) return XG_ERR_UNSUPPORTED;
  return L.fp64 ? launch_pdk<double>(L, s) : launch_pdk<float>(L, s);
}

int coef_active_launch(const CoefFormLaunch& L, cudaStream_t s) {
  if (L.d.n <= 0 || L.ne <= 0) return XG_OK;
  k_coef_active<<<(unsigned)((L.nw32 * 32 + 255) / 256), 256, 0, s>>>(L.ne, L.dom, L.d, L.act_un, L.act_cut, L.nw32);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_coef_active");
}

int coef_elmat_launch(const CoefFormLaunch& L, cudaStream_t s) {
  if (L.d.n <= 0) return XG_OK;
  if (L.dim < 2 || L.dim > 3 || L.order < 1 || L.order > 3) return XG_ERR_UNSUPPORTED;
  return L.fp64 ? launch_k<double>(L, s) : launch_k<float>(L, s);
}

}  // namespace xg

// ---- Integrate of polynomials in GridFunctions --------------------------------------
// The reference's Integrate with a CoefficientFunction of GridFunctions
// (cutint/cutintegral.cpp:126-212; the CoefficientFunction evaluated at the
// points of StraightCutIntegrationRule, cutint/straightcutrule.cpp:582-677),
// for sums of products c x^e f_a f_b, each factor a field's value or one of
// its partial derivatives (the H1 error (grad gfu - grad gfex)^2).  Thread per element (grid-stride, a
// fixed assignment), the block sums by a fixed tree and the blocks summed in
// order: deterministic.
namespace xg {
namespace {

constexpr int kMaxFields = 4, kMaxFMonos = 16, kFiThreads = 256, kFiBlocks = 152 * 4;

struct FieldsDesc {
  int nf, nm;
  int order[kMaxFields];
  int grad[kMaxFields];             // some product takes a derivative of the field
  const int32_t* dofs[kMaxFields];  // [nd_i][ne]
  const double* v[kMaxFields];
  double c[kMaxFMonos];
  int e[kMaxFMonos][3];
  int f0[kMaxFMonos], f1[kMaxFMonos];
  int d0[kMaxFMonos], d1[kMaxFMonos];  // -1: the value, else the derivative along x_d
  const double* gdef;                  // mesh deformation [nedges][3] or NULL
  const int32_t* el_edges;             // [nedges per element][ne]
};

template <int D>
__global__ void __launch_bounds__(kFiThreads)
    k_integrate_fields(int ne, int nv, const int32_t* __restrict__ elv, const double* __restrict__ xyz,
                       const double* __restrict__ lset, int dt, int order, FieldsDesc F,
                       const uint64_t* __restrict__ defined_on, double* __restrict__ block_sums, int* err) {
  __shared__ double red[kFiThreads];
  double acc = 0.0;
  const int p = clamp_order(order);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    if (defined_on && !cf_bit64(defined_on, e)) continue;
    double l[4], xv[4][3];
    int gv[4] = {0, 0, 0, 0};
    for (int v = 0; v <= D; v++) {
      gv[v] = elv[(int64_t)v * ne + e];
      l[v] = lset[gv[v]];
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + gv[v]] : 0.0;
    }
    const int cdom = check_if_straight_cut(l, D + 1);
    if (cdom != XG_IF && cdom != dt) continue;
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
    const double ifac = dt == XG_IF && cdom == XG_IF && !F.gdef ? if_factor<D>(g, l) : 1.0;
    // the deformation in the reference frame: theta_j = J^-1 gdef(edge j)
    double theta[6][3];
    if (F.gdef) {
      constexpr int NE = D == 2 ? 3 : 6;
      for (int j = 0; j < 6; j++)
        for (int r = 0; r < 3; r++) {
          double sr = 0.0;
          if (j < NE && r < D) {
            const int ed = F.el_edges[(int64_t)j * ne + e];
            for (int k = 0; k < D; k++) sr += g.Finv[r][k] * F.gdef[(int64_t)ed * 3 + k];
          }
          theta[j][r] = sr;
        }
    }
    // the rule point xi of the reference element with reference weight wr
    auto point = [&](const double* xi, double wr) {
      double lam[D + 1], sl = 0.0, xp[3] = {0.0, 0.0, 0.0}, y[3] = {xi[0], xi[1], D == 3 ? xi[2] : 0.0};
      for (int k = 0; k < D; k++) {
        lam[k] = xi[k];
        sl += xi[k];
      }
      lam[D] = 1.0 - sl;
      double w = wr * meas * ifac, gd[D + 1][D];
      const double(*gp)[D] = gl;
      if (F.gdef) {
        // x = x0 + J (xi + Theta(xi)), F = J (I + grad Theta): weight |det F|
        // (IF: times |F^-T n_ref|), gradients through F^-T
        double Am[3][3], Fm[3][3], Fi[3][3], detF;
        iso::deform_at<D>(theta, xi, y, Am);
        for (int r = 0; r < 3; r++)
          for (int k = 0; k < 3; k++) {
            double sr = 0.0;
            for (int q = 0; q < 3; q++) sr += (r < D && q < D ? g.F[r][q] : (r == q ? 1.0 : 0.0)) * Am[q][k];
            Fm[r][k] = sr;
          }
        if (!iso::invert<D>(Fm, Fi, &detF)) {
          set_err(err, XG_ERR_NONFINITE);
          return;
        }
        double nn2 = 0.0, gr2 = 0.0;
        for (int k = 0; k < D; k++) {
          double sa = 0.0, sn = 0.0;
          for (int a = 0; a < D; a++) {
            gd[a][k] = Fi[a][k];
            sa += Fi[a][k];
            sn += Fi[a][k] * (l[a] - l[D]);
          }
          gd[D][k] = -sa;
          nn2 += sn * sn;
          gr2 += (l[k] - l[D]) * (l[k] - l[D]);
        }
        w = wr * fabs(detF);
        if (dt == XG_IF) w *= sqrt(nn2 / gr2);
        gp = gd;
      }
      for (int r = 0; r < D; r++) {
        double sr = g.x0[r];
        for (int k = 0; k < D; k++) sr += g.F[r][k] * y[k];
        xp[r] = sr;
      }
      // factor table: [field][0] the value, [field][1 + d] the derivative along x_d
      double fv[kMaxFields][4];
      for (int i = 0; i < F.nf; i++) {
        const int k = F.order[i], nd = ndof_el(D, k);
        double s = 0.0, sg[D];
        for (int d = 0; d < D; d++) sg[d] = 0.0;
        for (int a = 0; a < nd; a++) {
          const double ca = F.v[i][F.dofs[i][(int64_t)a * ne + e]];
          if (F.grad[i]) {
            double ph, gr[D];
            eval_fn<D, double>(desc_rt<D>(k, a, gv), lam, gp, ph, gr);
            s += ca * ph;
            for (int d = 0; d < D; d++) sg[d] += ca * gr[d];
          } else {
            s += ca * eval_fn_value<D, double>(desc_rt<D>(k, a, gv), lam);
          }
        }
        fv[i][0] = s;
        fv[i][1] = fv[i][2] = fv[i][3] = 0.0;
        for (int d = 0; d < D; d++) fv[i][1 + d] = sg[d];
      }
      double val = 0.0;
      for (int m = 0; m < F.nm; m++) {
        double t = F.c[m] * cf_ipow(xp[0], F.e[m][0]) * cf_ipow(xp[1], F.e[m][1]) *
                   (D == 3 ? cf_ipow(xp[2], F.e[m][2]) : 1.0);
        if (F.f0[m] >= 0) t *= fv[F.f0[m]][1 + F.d0[m]];
        if (F.f1[m] >= 0) t *= fv[F.f1[m]][1 + F.d1[m]];
        val += t;
      }
      acc += w * val;
    };
    if (cdom != XG_IF) {
      const int off = g_cf_rules.off[D][p], cnt = g_cf_rules.cnt[D][p];
      for (int q = 0; q < cnt; q++) point(g_cf_rules.x[off + q], g_cf_rules.w[off + q]);
      continue;
    }
    Sub subs[3];
    const int ns = decompose<D>(l, dt, subs);
    if (ns < 0) {
      set_err(err, -ns);
      continue;
    }
    const int sd = dt == XG_IF ? D - 1 : D;
    const int off = g_cf_rules.off[sd][p], cnt = g_cf_rules.cnt[sd][p];
    for (int s = 0; s < ns; s++) {
      const double trafofac = simplex_volume(subs[s].p, sd + 1);
      for (int q = 0; q < cnt; q++) {
        double pt[3];
        plain_point(subs[s], sd + 1, g_cf_rules.x[off + q], pt);
        point(pt, g_cf_rules.w[off + q] * trafofac);
      }
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kFiThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
}

__global__ void k_fi_sum(const double* __restrict__ v, int n, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += v[i];
    out[0] = s;
  }
}

}  // namespace
}  // namespace xg

using namespace xg;

extern "C" int xg_integrate_fields(xg_mesh* m, const double* d_lset, int dt, int order, int32_t nfields,
                                   xg_space* const* spaces, const double* const* d_fields, int32_t nmonos,
                                   const xg_fmono* monos, const uint64_t* d_defined_on, const double* d_deform,
                                   double* d_result, void* stream) {
  if (!m || !d_lset || !d_result || dt < 0 || dt > 2 || order < 0 || order > kMaxOrder || nfields < 0 ||
      nmonos < 0 || (nfields > 0 && (!spaces || !d_fields)) || (nmonos > 0 && !monos))
    return XG_ERR_ARG;
  if (nfields > kMaxFields || nmonos > kMaxFMonos) {
    set_last_error("xg_integrate_fields: at most " + std::to_string(kMaxFields) + " fields and " +
                   std::to_string(kMaxFMonos) + " products");
    return XG_ERR_UNSUPPORTED;
  }
  if (m->tensor) {
    set_last_error("xg_integrate_fields: simplex meshes only");
    return XG_ERR_UNSUPPORTED;
  }
  FieldsDesc F{};
  F.nf = nfields;
  F.nm = nmonos;
  for (int i = 0; i < nfields; i++) {
    const xg_space* sp = spaces[i];
    if (!sp || !d_fields[i] || sp->mesh != m || sp->kt >= 0 || sp->order < 1 || sp->order > 3) {
      set_last_error("xg_integrate_fields: field " + std::to_string(i) +
                     " needs a spatial space of order 1..3 on the mesh and its coefficient vector");
      return XG_ERR_ARG;
    }
    F.order[i] = sp->order;
    F.dofs[i] = sp->d_el_dofs;
    F.v[i] = d_fields[i];
  }
  for (int k = 0; k < nmonos; k++) {
    const xg_fmono& q = monos[k];
    if (q.e[0] < 0 || q.e[1] < 0 || q.e[2] < 0 || q.f0 < -1 || q.f0 >= nfields || q.f1 < -1 || q.f1 >= nfields ||
        q.d0 < -1 || q.d0 >= m->dim || q.d1 < -1 || q.d1 >= m->dim || (q.f0 < 0 && q.d0 >= 0) ||
        (q.f1 < 0 && q.d1 >= 0))
      return XG_ERR_ARG;
    F.c[k] = q.coef;
    for (int r = 0; r < 3; r++) F.e[k][r] = q.e[r];
    F.f0[k] = q.f0;
    F.f1[k] = q.f1;
    F.d0[k] = q.d0;
    F.d1[k] = q.d1;
    if (q.d0 >= 0) F.grad[q.f0] = 1;
    if (q.d1 >= 0) F.grad[q.f1] = 1;
  }
  F.gdef = d_deform;
  F.el_edges = m->d_el_edges;
  if (int st = ensure_device_rules()) return st;
  const size_t need = kFiBlocks * sizeof(double);
  if (m->scratch_bytes < need) {
    cudaFree(m->d_scratch);
    m->d_scratch = nullptr;
    m->scratch_bytes = 0;
    XG_CUDA(cudaMalloc(&m->d_scratch, need));
    m->scratch_bytes = need;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* bs = (double*)m->d_scratch;
  if (m->dim == 2)
    k_integrate_fields<2><<<kFiBlocks, kFiThreads, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, d_lset, dt, order, F,
                                                           d_defined_on, bs, m->d_err);
  else
    k_integrate_fields<3><<<kFiBlocks, kFiThreads, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, d_lset, dt, order, F,
                                                           d_defined_on, bs, m->d_err);
  k_fi_sum<<<1, 32, 0, s>>>(bs, kFiBlocks, d_result);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_integrate_fields");
}

// Subdivision cut rules on the GPU (the rule code is xg_subdiv.cuh):
//   xg_integrate_subdiv     Integrate(f * dCut(lset_h, dt, subdivlvl=L)) for a
//                           level set of order 1..3 given as H1 coefficients
//                           (the reference's CutIntegrationRule path for
//                           level sets that are not P1, cutint/xintegration.cpp:
//                           102-116, 1626-1754)
//   xg_subdiv_moments_tet   per element the NEG moments (monomials of degree
//                           <= 4 in reference coordinates) of a P2 level set
//                           given by its values at the vertices and edge
//                           midpoints of the reference tetrahedron
// A group of NC^2 threads (NC = 8 children in 3D, 4 in 2D) runs one element:
// the lattice checks of the root and of its children are split over the
// group's threads (sign flags in shared memory), then every thread walks the
// subtree of one grandchild (or the thread of a first-level leaf fills it), so
// a cut element's tree is spread over 64 threads instead of walked by one.
// Per-thread sums are reduced in a fixed tree, per block and over the blocks
// in order, so repeated calls give the same bits.
#include <cuda_runtime.h>

#include <cstdint>

#include "xg_internal.h"
#include "xg_subdiv.cuh"

namespace xg {

static __device__ RuleTable g_sd_rules;  // the rule code reads its table by pointer

int upload_rules_subdiv() {
  XG_CUDA(cudaMemcpyToSymbol(g_sd_rules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

constexpr int kSdThreads = 128;
constexpr int kSdBlocks = 152 * 8;

__device__ __forceinline__ bool sd_bit(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

__device__ __forceinline__ double sd_ipow(double x, int e) {
  double r = 1.0;
  for (int k = 0; k < e; k++) r *= x;
  return r;
}

template <int D>
struct Grp {
  static constexpr int NC = D == 3 ? 8 : 4;  // children of a simplex
  static constexpr int TPE = NC * NC;        // threads per element
  static constexpr int EPB = kSdThreads / TPE;
};

// sign flags (bit 0: a lattice point >= 0, bit 1: one < 0) of the lattice of
// simplex v at level L, the share of thread t of nt
template <int D, int K>
__device__ int lattice_flags(const sd::Elem<D, K>& el, const double (*v)[3], int L, int t, int nt) {
  const int np = 1 << L, side = np + 1, total = D == 2 ? side * side : side * side * side;
  const double dx = 1.0 / np;
  int f = 0;
  for (int q = t; q < total && f != 3; q += nt) {
    int I[3] = {q % side, (q / side) % side, D == 3 ? q / (side * side) : 0};
    if (I[0] + I[1] + I[2] > np) continue;
    double xi[3];
    sd::lattice_point<D>(v, I, dx, xi);
    f |= sd::lset_at(el, xi) >= 0.0 ? 1 : 2;
  }
  return f;
}

// thread t of an element's group: its share of the element's rule.  flags:
// the element's NC + 1 shared words; every thread of the block calls this
// (the block synchronises four times), those without an element pass live = false.
// The tree is the serial one of sd::element_rule: the root checked at level
// L, its children (if it is cut and L >= 1) at L - 1, each cut child's
// children walked by sd::node_rule from level L - 2.
template <int D, int K, class E>
__device__ int group_rule(const RuleTable* Rp, const sd::Elem<D, K>& el, bool live, int dt, int order, int L, int t,
                          int* flags, E& emit) {
  constexpr int NC = Grp<D>::NC, TPE = Grp<D>::TPE;
  const int S = L < 2 ? L : 2;  // tree levels split over the group
  double root[4][3];
  sd::ref_simplex(D, root);
  __syncthreads();  // the group's flags of the previous element are read
  if (t <= NC) flags[t] = 0;
  __syncthreads();
  if (live && S >= 1) {
    const int f = lattice_flags(el, root, L, t, TPE);
    if (f) atomicOr(&flags[0], f);
  }
  __syncthreads();
  const bool root_cut = flags[0] == 3;
  if (live && S >= 2 && root_cut) {
    double cv[4][3];
    sd::child<D>(root, t / NC, cv);
    const int f = lattice_flags(el, cv, L - 1, t % NC, NC);
    if (f) atomicOr(&flags[1 + t / NC], f);
  }
  __syncthreads();
  if (!live) return 0;
  if (S == 0) return t == 0 ? sd::node_rule(Rp, el, root, L, dt, order, emit) : 0;
  if (!root_cut) {
    // an uncut root (flags 1: POS, 2: NEG) is filled as a whole
    if (t == 0 && (flags[0] == 1 ? XG_POS : XG_NEG) == dt) sd::fill(Rp, el, root, (const double*)nullptr, dt, order, emit);
    return 0;
  }
  double cv[4][3];
  if (S == 1) {
    if (t >= NC) return 0;
    sd::child<D>(root, t, cv);
    return sd::node_rule(Rp, el, cv, L - 1, dt, order, emit);
  }
  const int c1 = t / NC, c2 = t % NC, fc = flags[1 + c1];
  sd::child<D>(root, c1, cv);
  if (fc != 3) {
    if (c2 == 0 && (fc == 1 ? XG_POS : XG_NEG) == dt) sd::fill(Rp, el, cv, (const double*)nullptr, dt, order, emit);
    return 0;
  }
  double gv[4][3];
  sd::child<D>(cv, c2, gv);
  return sd::node_rule(Rp, el, gv, L - 2, dt, order, emit);
}

template <int D, int K>
__global__ void __launch_bounds__(kSdThreads) k_subdiv_integrate(int ne, int nv, const int32_t* __restrict__ elv,
                                                                  const double* __restrict__ xyz,
                                                                  const int32_t* __restrict__ el_dofs,
                                                                  const double* __restrict__ coefs, int dt, int order,
                                                                  int levels, int ex, int ey, int ez,
                                                                  const uint64_t* __restrict__ defined_on,
                                                                  double* __restrict__ block_sums, int* err) {
  constexpr int N = ndof_el(D, K), TPE = Grp<D>::TPE, EPB = Grp<D>::EPB;
  __shared__ double red[kSdThreads];
  __shared__ int flags[EPB][Grp<D>::NC + 1];
  const int le = threadIdx.x / TPE, t = threadIdx.x % TPE;
  double acc = 0.0;
  for (int64_t base = (int64_t)blockIdx.x * EPB; base < ne; base += (int64_t)gridDim.x * EPB) {
    const int64_t e = base + le;
    bool live = e < ne && (!defined_on || sd_bit(defined_on, e));
    sd::Elem<D, K> el;
    if (live) {
      int gv[4] = {0, 0, 0, 0};
      double xv[4][3];
      for (int v = 0; v <= D; v++) {
        gv[v] = elv[(int64_t)v * ne + e];
        for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + gv[v]] : 0.0;
      }
      for (int r = 0; r < 3; r++) {
        el.x0[r] = xv[D][r];
        for (int c = 0; c < 3; c++) el.F[r][c] = c < D ? xv[c][r] - xv[D][r] : 0.0;
      }
      for (int i = 0; i < N; i++) {
        el.coef[i] = coefs[el_dofs[(int64_t)i * ne + e]];
        el.desc[i] = fn_desc<D, K>(i, gv);
      }
    }
    auto emit = [&](const double* x, double w) {
      acc += w * sd_ipow(x[0], ex) * sd_ipow(x[1], ey) * (D == 3 ? sd_ipow(x[2], ez) : 1.0);
    };
    const int st = group_rule<D, K>(&g_sd_rules, el, live, dt, order, levels, t, flags[le], emit);
    if (st) set_err(err, st);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kSdThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
}

__global__ void k_sd_sum(const double* v, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += v[i];
    out[0] = s;
  }
}

// the 35 NEG moments x^a y^b z^c (a + b + c <= 4, by degree, then a, then b
// descending) of each reference tetrahedron, 64 threads per element (the
// group's sums reduced by warp shuffles, then the two warps in order)
__global__ void __launch_bounds__(kSdThreads) k_subdiv_moments(int64_t n, const double* __restrict__ vals10,
                                                               int levels, double* __restrict__ out35,
                                                               const int32_t* __restrict__ list,
                                                               const int32_t* __restrict__ count, int* err) {
  constexpr int TPE = Grp<3>::TPE, EPB = Grp<3>::EPB, WPE = TPE / 32;
  __shared__ int flags[EPB][Grp<3>::NC + 1];
  __shared__ double red[EPB * WPE][35];
  const int E[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  const int le = threadIdx.x / TPE, t = threadIdx.x % TPE, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t items = list ? (int64_t)*count : n;
  for (int64_t base = (int64_t)blockIdx.x * EPB; base < items; base += (int64_t)gridDim.x * EPB) {
    const int64_t it = base + le;
    int64_t e = -1;
    if (it < items) {
      e = list ? (int64_t)list[it] : it;
      if (e < 0 || e >= n) {
        if (t == 0) set_err(err, XG_ERR_ARG);
        e = -1;
      }
    }
    const bool live = e >= 0;
    sd::Elem<3, 2> el;
    if (live) {
      const int gv[4] = {0, 1, 2, 3};
      for (int r = 0; r < 3; r++) {
        el.x0[r] = 0.0;
        for (int c = 0; c < 3; c++) el.F[r][c] = r == c ? 1.0 : 0.0;
      }
      const double* p = vals10 + e * 10;
      // P2 nodal values -> the H1 coefficients: vertex values, 4 p(mid) - 2 (p_a + p_b)
      for (int i = 0; i < 4; i++) el.coef[i] = p[i];
      for (int j = 0; j < 6; j++) el.coef[4 + j] = 4.0 * p[4 + j] - 2.0 * (p[E[j][0]] + p[E[j][1]]);
      for (int i = 0; i < 10; i++) el.desc[i] = fn_desc<3, 2>(i, gv);
    }
    double m[35];
    for (int k = 0; k < 35; k++) m[k] = 0.0;
    auto emit = [&](const double* x, double wq) {
      const double px[5] = {1, x[0], x[0] * x[0], x[0] * x[0] * x[0], x[0] * x[0] * x[0] * x[0]};
      const double py[5] = {1, x[1], x[1] * x[1], x[1] * x[1] * x[1], x[1] * x[1] * x[1] * x[1]};
      const double pz[5] = {1, x[2], x[2] * x[2], x[2] * x[2] * x[2], x[2] * x[2] * x[2] * x[2]};
      int k = 0;
      for (int tt = 0; tt <= 4; tt++)
        for (int a = tt; a >= 0; a--)
          for (int b = tt - a; b >= 0; b--) m[k++] += wq * px[a] * py[b] * pz[tt - a - b];
    };
    const int st = group_rule<3, 2>(&g_sd_rules, el, live, XG_NEG, 4, levels, t, flags[le], emit);
    if (st) set_err(err, st);
    for (int k = 0; k < 35; k++) {
      double v = m[k];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[w][k] = v;
    }
    __syncthreads();
    if (live && t < 35) {
      double v = red[le * WPE][t];
      for (int q = 1; q < WPE; q++) v += red[le * WPE + q][t];
      out35[e * 35 + t] = v;
    }
    __syncthreads();
  }
}

template <int D, int K>
void launch_int(xg_space* sp, const double* coefs, int dt, int order, int levels, int ex, int ey, int ez,
                const uint64_t* defined_on, double* bs, cudaStream_t s) {
  xg_mesh* m = sp->mesh;
  k_subdiv_integrate<D, K><<<kSdBlocks, kSdThreads, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, sp->d_el_dofs, coefs,
                                                           dt, order, levels, ex, ey, ez, defined_on, bs, m->d_err);
}

}  // namespace

int subdiv_moments_launch(const double* d_vals10, int64_t n, int levels, double* d_out35, const int32_t* d_list,
                          const int32_t* d_count, int* d_err, cudaStream_t s) {
  const int64_t blocks = (n + Grp<3>::EPB - 1) / Grp<3>::EPB;
  k_subdiv_moments<<<(unsigned)(blocks < kSdBlocks * 4 ? (blocks > 0 ? blocks : 1) : kSdBlocks * 4), kSdThreads, 0, s>>>(
      n, d_vals10, levels, d_out35, d_list, d_count, d_err);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_subdiv_moments_tet");
}

}  // namespace xg

using namespace xg;

extern "C" {

int xg_integrate_subdiv(xg_space* sp, const double* d_lset_coefs, int dt, int order, int subdivlvl, int ex, int ey,
                        int ez, const uint64_t* d_defined_on, double* d_result, void* stream) {
  if (!sp || !d_lset_coefs || !d_result || dt < 0 || dt > 2 || order < 0 || order > kMaxOrder || ex < 0 ||
      ey < 0 || ez < 0 || subdivlvl < 0 || subdivlvl > sd::kMaxLevels) {
    set_last_error("xg_integrate_subdiv: bad arguments (subdivlvl 0..6, order 0..8)");
    return XG_ERR_ARG;
  }
  if (sp->kt >= 0 || sp->mesh->tensor || sp->ndof != sp->ndof_s || sp->mesh->dim < 2) {
    set_last_error("xg_integrate_subdiv: the level set lives in an H1 space on a simplex mesh");
    return XG_ERR_UNSUPPORTED;
  }
  int st = ensure_device_rules();
  if (st) return st;
  xg_mesh* m = sp->mesh;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t need = kSdBlocks * sizeof(double);
  if (m->scratch_bytes < need) {
    cudaFree(m->d_scratch);
    m->d_scratch = nullptr;
    m->scratch_bytes = 0;
    XG_CUDA(cudaMalloc(&m->d_scratch, need));
    m->scratch_bytes = need;
  }
  double* bs = (double*)m->d_scratch;
  const int D = m->dim, K = sp->order;
  if (D == 2) {
    if (K == 1) launch_int<2, 1>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
    else if (K == 2) launch_int<2, 2>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
    else launch_int<2, 3>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
  } else {
    if (K == 1) launch_int<3, 1>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
    else if (K == 2) launch_int<3, 2>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
    else launch_int<3, 3>(sp, d_lset_coefs, dt, order, subdivlvl, ex, ey, ez, d_defined_on, bs, s);
  }
  k_sd_sum<<<1, 32, 0, s>>>(bs, kSdBlocks, d_result);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_subdiv_integrate");
}

int xg_subdiv_moments_tet(const double* d_vals10, int64_t n, int subdivlvl, double* d_out35, int* d_err,
                          void* stream) {
  if ((n > 0 && (!d_vals10 || !d_out35)) || n < 0 || subdivlvl < 0 || subdivlvl > sd::kMaxLevels) {
    set_last_error("xg_subdiv_moments_tet: bad arguments (subdivlvl 0..6)");
    return XG_ERR_ARG;
  }
  if (n == 0) return XG_OK;
  int st = ensure_device_rules();
  if (st) return st;
  return subdiv_moments_launch(d_vals10, n, subdivlvl, d_out35, nullptr, nullptr, d_err, (cudaStream_t)stream);
}

}  // extern "C"

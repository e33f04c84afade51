// Integrate on quadrilateral and hexahedral meshes (cutint/cutintegral.cpp:126-212).
//
// A level set cuts few elements (about 1 % of a 128^3 hexahedral mesh), and a
// cut element's rule (xg_quadcut.cuh) costs tens of times an uncut element's
// tensor rule.  With one thread per element, a quarter of the warps would run
// at the cost of their one cut element with the other lanes idle, and the
// narrow FP64 pipe of GB300 charges a warp instruction the same whatever the
// number of active lanes.  So the work is split:
//   pass 1 (thread per element)      uncut elements: the tensor rule of the
//                                    unit box, with the multilinear element
//                                    map in monomial form (only det J is
//                                    needed); cut elements go to a list;
//   pass 2 (thread per cut element)  the cut rule of xg_quadcut.cuh, dense;
//   pass 3                           the per-element values summed in a fixed
//                                    order (deterministic whatever the list order).
// Compiled with FMA contraction: the integrals are compared with a tolerance;
// the rule export (xg_quad.cu) keeps the operation order of the CPU statement.
#include <cuda_runtime.h>

#include "xg_internal.h"
#include "xg_quadcut.cuh"

namespace xg {

static __device__ RuleTable g_irules;

int upload_rules_quad_int() {
  XG_CUDA(cudaMemcpyToSymbol(g_irules, &host_rules(), sizeof(RuleTable)));
  return XG_OK;
}

namespace {

constexpr int kQThreads = 128;
constexpr int kQBlocks = 152 * 8;

// x(xi) = sum_m a[m] prod_{d in m} xi_d over the monomials m (bit d: xi_d) of
// the multilinear interpolation of the corners
template <int D>
struct MapC {
  double a[1 << D][D];
};

template <int D>
__device__ __forceinline__ void map_coefs(const double (*xv)[3], MapC<D>& M) {
  constexpr int NV = 1 << D;
#pragma unroll
  for (int m = 0; m < NV; m++)
#pragma unroll
    for (int i = 0; i < D; i++) M.a[m][i] = 0.0;
#pragma unroll
  for (int v = 0; v < NV; v++) {
    // corner bits of vertex v: (0,0,0),(1,0,0),(1,1,0),(0,1,0), then z = 1
    const int cb = ((v == 1 || v == 2 || v == 5 || v == 6) ? 1 : 0) | (((v & 3) >= 2) ? 2 : 0) | (v >= 4 ? 4 : 0);
#pragma unroll
    for (int m = 0; m < NV; m++) {
      if (cb & ~m) continue;
      const bool neg = __popc(m & ~cb) & 1;
#pragma unroll
      for (int i = 0; i < D; i++) M.a[m][i] += neg ? -xv[v][i] : xv[v][i];
    }
  }
}

// point x(xi) and J = dx/dxi
template <int D>
__device__ __forceinline__ void map_eval(const MapC<D>& M, const double* xi, double* x, double J[3][3]) {
  constexpr int NV = 1 << D;
#pragma unroll
  for (int i = 0; i < D; i++) {
    x[i] = 0.0;
#pragma unroll
    for (int k = 0; k < D; k++) J[i][k] = 0.0;
  }
#pragma unroll
  for (int m = 0; m < NV; m++) {
    double mon = 1.0;
#pragma unroll
    for (int d = 0; d < D; d++)
      if (m & (1 << d)) mon *= xi[d];
#pragma unroll
    for (int i = 0; i < D; i++) x[i] += M.a[m][i] * mon;
#pragma unroll
    for (int k = 0; k < D; k++) {
      if (!(m & (1 << k))) continue;
      double dm = 1.0;
#pragma unroll
      for (int d = 0; d < D; d++)
        if (d != k && (m & (1 << d))) dm *= xi[d];
#pragma unroll
      for (int i = 0; i < D; i++) J[i][k] += M.a[m][i] * dm;
    }
  }
}

template <int D>
__device__ __forceinline__ double det_of(const double J[3][3]) {
  if (D == 2) return J[0][0] * J[1][1] - J[0][1] * J[1][0];
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) + J[0][1] * (J[1][2] * J[2][0] - J[1][0] * J[2][2]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

// |J^-T n| |det J| with n the normalised level-set gradient g: the cofactor
// matrix C = det J J^-T gives |C n| directly (no division by det J)
template <int D>
__device__ __forceinline__ double if_measure(const double J[3][3], const double* g) {
  const double inv = 1.0 / sqrt(g[0] * g[0] + g[1] * g[1] + (D == 3 ? g[2] * g[2] : 0.0));
  double c[3];
  if (D == 2) {
    // C = [[J11, -J10], [-J01, J00]]
    c[0] = J[1][1] * g[0] - J[1][0] * g[1];
    c[1] = -J[0][1] * g[0] + J[0][0] * g[1];
    c[2] = 0.0;
  } else {
    double C[3][3];
    C[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    C[0][1] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    C[0][2] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    C[1][0] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    C[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    C[1][2] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    C[2][0] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    C[2][1] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    C[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    for (int i = 0; i < 3; i++) c[i] = C[i][0] * g[0] + C[i][1] * g[1] + C[i][2] * g[2];
  }
  return sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) * inv;
}

__device__ __forceinline__ double ipow(double x, int e) {
  double r = 1.0;
  for (int i = 0; i < e; i++) r *= x;
  return r;
}

__device__ __forceinline__ bool tbit(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

template <int D>
__device__ __forceinline__ void gather(int ne, const int32_t* __restrict__ elv, const double* __restrict__ xyz, int nv,
                                       const double* __restrict__ lset, int e, double* l, double (*xv)[3]) {
  constexpr int NV = 1 << D;
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const int vid = elv[(int64_t)v * ne + e];
    l[v] = lset[vid];
#pragma unroll
    for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
  }
}

struct Mono {
  int ex, ey, ez;
};

template <int D>
__device__ __forceinline__ double fval(const double* x, const Mono& f) {
  return ipow(x[0], f.ex) * ipow(x[1], f.ey) * (D == 3 ? ipow(x[2], f.ez) : 1.0);
}

}  // namespace

// pass 1: uncut elements (tensor rule of the unit box); cut elements listed
template <int D>
__global__ void __launch_bounds__(kQThreads) k_qint_uncut(int ne, const int32_t* __restrict__ elv,
                                                         const double* __restrict__ xyz, int nv,
                                                         const double* __restrict__ lset, int dt, int order, Mono f,
                                                         const uint64_t* __restrict__ defined_on,
                                                         double* __restrict__ ev, int32_t* __restrict__ cutlist) {
  constexpr int NV = 1 << D;
  const RuleTable& R = g_irules;
  const int o = clamp_order(order), off = R.off[1][o], n1 = R.cnt[1][o];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double val = 0.0;
    bool cut = false;
    if (!defined_on || tbit(defined_on, e)) {
      double l[NV], xv[NV][3];
      gather<D>(ne, elv, xyz, nv, lset, (int)e, l, xv);
      const int dom = qc::qcheck(l, NV, 0.0);
      cut = dom == XG_IF;
      if (!cut && dom == dt) {
        MapC<D> M;
        map_coefs<D>(xv, M);
        const int n3 = D == 3 ? n1 : 1;
        for (int a = 0; a < n1; a++)
          for (int b = 0; b < n1; b++)
            for (int c = 0; c < n3; c++) {
              const double xi[3] = {R.x[off + a][0], R.x[off + b][0], D == 3 ? R.x[off + c][0] : 0.0};
              const double w = D == 3 ? R.w[off + a] * R.w[off + b] * R.w[off + c] : R.w[off + a] * R.w[off + b];
              double x[3], J[3][3];
              map_eval<D>(M, xi, x, J);
              val += w * fabs(det_of<D>(J)) * fval<D>(x, f);
            }
      }
    }
    ev[e] = val;
    // warp-aggregated append of the cut elements (order irrelevant: values go to ev[e])
    const unsigned mask = __activemask();
    const unsigned ball = __ballot_sync(mask, cut);
    if (ball) {
      const int lane = threadIdx.x & 31, leader = __ffs(ball) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(cutlist, __popc(ball));
      base = __shfl_sync(mask, base, leader);
      if (cut) cutlist[1 + base + __popc(ball & ((1u << lane) - 1))] = (int32_t)e;
    }
  }
}

// pass 2: the cut rule of each listed element
template <int D>
__global__ void __launch_bounds__(kQThreads) k_qint_cut(int ne, const int32_t* __restrict__ elv,
                                                       const double* __restrict__ xyz, int nv,
                                                       const double* __restrict__ lset, int dt, int order, int pol,
                                                       Mono f, const int32_t* __restrict__ cutlist,
                                                       double* __restrict__ ev, int* err) {
  constexpr int NV = 1 << D;
  const int ncut = cutlist[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncut; i += gridDim.x * blockDim.x) {
    const int e = cutlist[1 + i];
    double l[NV], xv[NV][3];
    gather<D>(ne, elv, xyz, nv, lset, e, l, xv);
    MapC<D> M;
    map_coefs<D>(xv, M);
    const qc::QL L = D == 2 ? qc::ql_quad(l) : qc::ql_hex(l);
    double acc = 0.0;
    auto emit = [&](const double* p, double w) {
      double x[3], J[3][3];
      map_eval<D>(M, p, x, J);
      double meas;
      if (dt == XG_IF) {
        double g[3];
        qc::ql_grad(L, p, g);
        meas = if_measure<D>(J, g);
      } else {
        meas = fabs(det_of<D>(J));
      }
      acc += w * meas * fval<D>(x, f);
    };
    const int st = qc::tp_cut_rule<D>(&g_irules, l, dt, order, pol, emit);
    if (st > 0) set_err(err, st);
    ev[e] = acc;
  }
}

// pass 3: fixed-order sums (a fixed element range per block, a fixed tree)
__global__ void __launch_bounds__(kQThreads) k_qint_blocks(const double* __restrict__ ev, int64_t n,
                                                          double* __restrict__ bs) {
  __shared__ double red[kQThreads];
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = blockIdx.x * per, b1 = b0 + per < n ? b0 + per : n;
  double acc = 0.0;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) acc += ev[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kQThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) bs[blockIdx.x] = red[0];
}

__global__ void k_qint_final(const double* bs, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += bs[i];
    out[0] = s;
  }
}

static int launch_check_qi(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return XG_OK;
}

// scratch: ev[ne] doubles, block sums [kQBlocks], cut list [ne + 1] ints
int quad_integrate(xg_mesh* m, const double* d_lset, int dt, int order, int pol, int ex, int ey, int ez,
                   const uint64_t* d_defined_on, double* d_result, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const size_t need = sizeof(double) * ((size_t)m->ne + kQBlocks) + sizeof(int32_t) * ((size_t)m->ne + 1);
  if (m->scratch_bytes < need) {
    cudaFree(m->d_scratch);
    m->d_scratch = nullptr;
    m->scratch_bytes = 0;
    XG_CUDA(cudaMalloc(&m->d_scratch, need));
    m->scratch_bytes = need;
  }
  double* ev = (double*)m->d_scratch;
  double* bs = ev + m->ne;
  int32_t* list = (int32_t*)(bs + kQBlocks);
  XG_CUDA(cudaMemsetAsync(list, 0, sizeof(int32_t), s));
  const Mono f{ex, ey, ez};
  if (m->dim == 2) {
    k_qint_uncut<2><<<kQBlocks, kQThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, dt, order, f,
                                                   d_defined_on, ev, list);
    k_qint_cut<2><<<kQBlocks, kQThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, dt, order, pol, f, list,
                                                 ev, m->d_err);
  } else {
    k_qint_uncut<3><<<kQBlocks, kQThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, dt, order, f,
                                                   d_defined_on, ev, list);
    k_qint_cut<3><<<kQBlocks, kQThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, dt, order, pol, f, list,
                                                 ev, m->d_err);
  }
  k_qint_blocks<<<kQBlocks, kQThreads, 0, s>>>(ev, m->ne, bs);
  k_qint_final<<<1, 32, 0, s>>>(bs, kQBlocks, d_result);
  return launch_check_qi("k_qint");
}

}  // namespace xg

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
// Both build the trees of all elements level by level (one thread per node
// and level, then one thread per leaf), so the warps of each kernel run the
// same kind of work; the leaves' values (the integral, or the moments per
// element) are summed in a fixed order, so repeated calls give the same
// bits.  A thread walking one element's tree depth first (sd::element_rule,
// the host check's path) ran its FP64 instructions 5.5 of 32 lanes full.
#include <cuda_runtime.h>

#include <cstdint>
#include <utility>
#include <vector>

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

__global__ void k_sd_sum(const double* v, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += v[i];
    out[0] = s;
  }
}

// ---- breadth-first moments ---------------------------------------------------------
// The tree of every element level by level: a node is (item, path) with the
// path's 3-bit digits the child indices from the root, so a thread rebuilds
// its simplex with the same child() arithmetic as the depth-first walk.
// Per level one thread per node classifies it (the checks of sd::node_rule:
// expand, plain leaf, cut leaf or nothing), scans give the children's and
// leaves' positions in node order, and the leaves are filled densely (one
// thread per leaf: the warps of a fill kernel run the same rule), then each
// element's moments are summed over its leaves, level by level, in order.

enum { SD_NONE = 0, SD_EXPAND = 1, SD_PLAIN = 2, SD_CUT = 3 };

struct SdNode {
  int32_t item;
  uint32_t path;
};

__device__ __forceinline__ void sd_elem(const double* __restrict__ vals10, int64_t e, sd::Elem<3, 2>& el) {
  const int E[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  const int gv[4] = {0, 1, 2, 3};
  for (int r = 0; r < 3; r++) {
    el.x0[r] = 0.0;
    for (int c = 0; c < 3; c++) el.F[r][c] = r == c ? 1.0 : 0.0;
  }
  const double* p = vals10 + e * 10;
  for (int i = 0; i < 4; i++) el.coef[i] = p[i];
  for (int j = 0; j < 6; j++) el.coef[4 + j] = 4.0 * p[4 + j] - 2.0 * (p[E[j][0]] + p[E[j][1]]);
  for (int i = 0; i < 10; i++) el.desc[i] = fn_desc<3, 2>(i, gv);
}

__device__ __forceinline__ void sd_simplex(uint32_t path, int depth, double (*v)[3]) {
  sd::ref_simplex(3, v);
  for (int d = 0; d < depth; d++) {
    double w[4][3];
    sd::child<3>(v, (int)((path >> (3 * d)) & 7u), w);
    for (int i = 0; i < 4; i++)
      for (int r = 0; r < 3; r++) v[i][r] = w[i][r];
  }
}

// the element of item i (a list entry or the item itself)
__device__ __forceinline__ int64_t sd_item_elem(const int32_t* list, int64_t base, int32_t item) {
  return list ? (int64_t)list[base + item] : base + item;
}

// m[k] += w x^a y^b z^c in the moments' order, with the products w x^a y^b
// formed once per (a, b)
__device__ __forceinline__ void sd_moments_point(const double* x, double w, double* m) {
  double wx[5], py[5], pz[5];
  wx[0] = w;
  py[0] = 1.0;
  pz[0] = 1.0;
#pragma unroll
  for (int i = 1; i < 5; i++) {
    wx[i] = wx[i - 1] * x[0];
    py[i] = py[i - 1] * x[1];
    pz[i] = pz[i - 1] * x[2];
  }
  int k = 0;
#pragma unroll
  for (int t = 0; t <= 4; t++)
#pragma unroll
    for (int a = t; a >= 0; a--) {
      const double wxy0 = wx[a];
#pragma unroll
      for (int b = t - a; b >= 0; b--) m[k++] += (wxy0 * py[b]) * pz[t - a - b];
    }
}

// the P2 level set of an element as a quadratic in x, y, z: q[0] + q[1] x +
// q[2] y + q[3] z + q[4] x^2 + q[5] y^2 + q[6] z^2 + q[7] xy + q[8] xz + q[9] yz
// (lambda_i = x_i for i < 3, lambda_3 = 1 - x - y - z; vertex functions
// lambda_i, edge functions lambda_a lambda_b)
__device__ __forceinline__ void sd_quadratic(const sd::Elem<3, 2>& el, double* q) {
  const double L[4][4] = {{0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}, {1, -1, -1, -1}};  // const, x, y, z
  const int E[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  for (int k = 0; k < 10; k++) q[k] = 0.0;
  for (int v = 0; v < 4; v++)
    for (int k = 0; k < 4; k++) q[k] += el.coef[v] * L[v][k];
  for (int j = 0; j < 6; j++) {
    const double* A = L[E[j][0]];
    const double* B = L[E[j][1]];
    const double c = el.coef[4 + j];
    q[0] += c * A[0] * B[0];
    q[1] += c * (A[0] * B[1] + A[1] * B[0]);
    q[2] += c * (A[0] * B[2] + A[2] * B[0]);
    q[3] += c * (A[0] * B[3] + A[3] * B[0]);
    q[4] += c * A[1] * B[1];
    q[5] += c * A[2] * B[2];
    q[6] += c * A[3] * B[3];
    q[7] += c * (A[1] * B[2] + A[2] * B[1]);
    q[8] += c * (A[1] * B[3] + A[3] * B[1]);
    q[9] += c * (A[2] * B[3] + A[3] * B[2]);
  }
}
__device__ __forceinline__ double sd_qval(const double* q, const double* x) {
  return q[0] + x[0] * (q[1] + q[4] * x[0] + q[7] * x[1] + q[8] * x[2]) + x[1] * (q[2] + q[5] * x[1] + q[9] * x[2]) +
         x[2] * (q[3] + q[6] * x[2]);
}
// CheckIfCut on the lattice of simplex v at level L (sd::lattice_domain with
// the quadratic form)
__device__ __forceinline__ int sd_qlattice(const double* q, const double (*v)[3], int L) {
  const int np = 1 << L;
  const double dx = 1.0 / np;
  bool pos = false, neg = false;
  for (int i2 = 0; i2 <= np; i2++)
    for (int i1 = 0; i1 + i2 <= np; i1++)
      for (int i0 = 0; i0 + i1 + i2 <= np; i0++) {
        const int I[3] = {i0, i1, i2};
        double xi[3];
        sd::lattice_point<3>(v, I, dx, xi);
        if (sd_qval(q, xi) >= 0.0) pos = true;
        else neg = true;
        if (pos && neg) return XG_IF;
      }
  return pos ? XG_POS : XG_NEG;
}

__global__ void __launch_bounds__(128) k_sd_classify(const SdNode* __restrict__ nodes, int64_t nn,
                                                     const double* __restrict__ vals10, const int32_t* __restrict__ list,
                                                     int64_t base, int depth, int lev, uint8_t* __restrict__ cls,
                                                     int32_t* __restrict__ cnt3) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x) {
    const SdNode nd = nodes[i];
    sd::Elem<3, 2> el;
    sd_elem(vals10, sd_item_elem(list, base, nd.item), el);
    double v[4][3], q[10];
    sd_simplex(nd.path, depth, v);
    sd_quadratic(el, q);
    const int dself = sd_qlattice(q, v, lev);
    int c;
    if (dself != XG_IF) {
      c = dself == XG_NEG ? SD_PLAIN : SD_NONE;
    } else if (lev == 0) {
      double l[4];
      for (int k = 0; k < 4; k++) l[k] = sd_qval(q, v[k]);
      const int dv = sd::vertex_domain(l, 4);
      c = dv == XG_IF ? SD_CUT : (dv == XG_NEG ? SD_PLAIN : SD_NONE);
    } else {
      c = SD_EXPAND;
    }
    cls[i] = (uint8_t)c;
    cnt3[i] = c == SD_EXPAND ? 8 : 0;
    cnt3[nn + i] = c == SD_PLAIN ? 1 : 0;
    cnt3[2 * nn + i] = c == SD_CUT ? 1 : 0;
  }
}

// exclusive scan of int32 counts (per-block scans, one block over the block
// sums, offsets added); totals to tot
constexpr int kSdScan = 1024;
__global__ void __launch_bounds__(kSdScan) k_sd_scan_local(const int32_t* __restrict__ in, int64_t n,
                                                           int32_t* __restrict__ out, int32_t* __restrict__ bsum) {
  __shared__ int32_t sh[kSdScan];
  const int64_t i = blockIdx.x * (int64_t)kSdScan + threadIdx.x;
  const int32_t x = i < n ? in[i] : 0;
  sh[threadIdx.x] = x;
  __syncthreads();
  for (int o = 1; o < kSdScan; o <<= 1) {
    const int32_t y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += y;
    __syncthreads();
  }
  if (i < n) out[i] = sh[threadIdx.x] - x;
  if (threadIdx.x == kSdScan - 1) bsum[blockIdx.x] = sh[threadIdx.x];
}
// one block: exclusive scan of the block sums, 1024 at a time with a carry
__global__ void __launch_bounds__(kSdScan) k_sd_scan_top(int32_t* bsum, int nb, int32_t* tot) {
  __shared__ int32_t sh[kSdScan];
  int32_t carry = 0;
  for (int b0 = 0; b0 < nb; b0 += kSdScan) {
    const int i = b0 + threadIdx.x;
    const int32_t x = i < nb ? bsum[i] : 0;
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int o = 1; o < kSdScan; o <<= 1) {
      const int32_t y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += y;
      __syncthreads();
    }
    if (i < nb) bsum[i] = carry + sh[threadIdx.x] - x;
    const int32_t blk = sh[kSdScan - 1];
    __syncthreads();
    carry += blk;
  }
  if (threadIdx.x == 0) *tot = carry;
}
__global__ void k_sd_scan_add(int32_t* out, int64_t n, const int32_t* bsum) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] += bsum[i / kSdScan];
}

__global__ void __launch_bounds__(128) k_sd_emit(const SdNode* __restrict__ nodes, int64_t nn,
                                                 const uint8_t* __restrict__ cls, const int32_t* __restrict__ pos3,
                                                 int depth, int nch, SdNode* __restrict__ next,
                                                 SdNode* __restrict__ plain, SdNode* __restrict__ cut,
                                                 int32_t* __restrict__ plain_depth) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x) {
    const SdNode nd = nodes[i];
    const int c = cls[i];
    if (c == SD_EXPAND) {
      const int64_t o = pos3[i];
      for (int k = 0; k < nch; k++) next[o + k] = SdNode{nd.item, nd.path | ((uint32_t)k << (3 * depth))};
    } else if (c == SD_PLAIN) {
      plain[pos3[nn + i]] = nd;
      plain_depth[pos3[nn + i]] = depth;
    } else if (c == SD_CUT) {
      cut[pos3[2 * nn + i]] = nd;
    }
  }
}

// one thread per leaf: its 35 moments (plain rule, or the straight cut of the
// vertex values on a level-0 simplex)
__global__ void __launch_bounds__(128) k_sd_fill(const SdNode* __restrict__ leaves, const int32_t* __restrict__ depths,
                                                 int64_t nl, int cut_depth, const double* __restrict__ vals10,
                                                 const int32_t* __restrict__ list, int64_t base,
                                                 double* __restrict__ mom, int* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl; i += (int64_t)gridDim.x * blockDim.x) {
    const SdNode nd = leaves[i];
    sd::Elem<3, 2> el;
    sd_elem(vals10, sd_item_elem(list, base, nd.item), el);
    double v[4][3];
    sd_simplex(nd.path, depths ? depths[i] : cut_depth, v);
    double m[35];
    for (int k = 0; k < 35; k++) m[k] = 0.0;
    auto emit = [&](const double* x, double w) { sd_moments_point(x, w, m); };
    if (depths) {
      sd::fill(&g_sd_rules, el, v, (const double*)nullptr, XG_NEG, 4, emit);
    } else {
      double l[4], q[10];
      sd_quadratic(el, q);
      for (int k = 0; k < 4; k++) l[k] = sd_qval(q, v[k]);
      const int st = sd::fill(&g_sd_rules, el, v, l, XG_NEG, 4, emit);
      if (st) set_err(err, st);
    }
    for (int k = 0; k < 35; k++) mom[i * 35 + k] = m[k];
  }
}

// per (item, moment): the sums over the item's leaves, plain leaves level by
// level, then the cut leaves, each range in order (leaves sorted by item
// within a level)
struct SdSegs {
  int n;
  int64_t off[sd::kMaxLevels + 2];
};
__device__ __forceinline__ int64_t sd_lower(const SdNode* a, int64_t lo, int64_t hi, int32_t item) {
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (a[mid].item < item) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
__global__ void __launch_bounds__(128) k_sd_reduce(int64_t items, const SdNode* __restrict__ plain,
                                                   const double* __restrict__ mp, SdSegs ps,
                                                   const SdNode* __restrict__ cut, const double* __restrict__ mc,
                                                   int64_t ncut, const int32_t* __restrict__ list, int64_t base,
                                                   double* __restrict__ out35) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < items * 35;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t it = (int32_t)(t / 35);
    const int k = (int)(t % 35);
    double acc = 0.0;
    for (int s2 = 0; s2 < ps.n; s2++) {
      const int64_t lo = sd_lower(plain, ps.off[s2], ps.off[s2 + 1], it);
      const int64_t hi = sd_lower(plain, lo, ps.off[s2 + 1], it + 1);
      for (int64_t j = lo; j < hi; j++) acc += mp[j * 35 + k];
    }
    const int64_t lo = sd_lower(cut, 0, ncut, it), hi = sd_lower(cut, lo, ncut, it + 1);
    for (int64_t j = lo; j < hi; j++) acc += mc[j * 35 + k];
    out35[sd_item_elem(list, base, it) * 35 + k] = acc;
  }
}

int sd_scan(const int32_t* in, int64_t n, int32_t* out, int32_t* bsum, int32_t* tot, cudaStream_t s) {
  const int nb = (int)((n + kSdScan - 1) / kSdScan);
  k_sd_scan_local<<<nb, kSdScan, 0, s>>>(in, n, out, bsum);
  k_sd_scan_top<<<1, kSdScan, 0, s>>>(bsum, nb, tot);
  k_sd_scan_add<<<nb, kSdScan, 0, s>>>(out, n, bsum);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_sd_scan");
}

unsigned sd_grid(int64_t n) {
  const int64_t b = (n + 127) / 128;
  return (unsigned)(b < 152 * 64 ? (b > 0 ? b : 1) : 152 * 64);
}

// device scratch of one call, stream-ordered (released when the call's work is done)
struct SdBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  SdBuf() = default;
  SdBuf(const SdBuf&) = delete;
  SdBuf& operator=(const SdBuf&) = delete;
  SdBuf(SdBuf&& o) noexcept : p(o.p), s(o.s) { o.p = nullptr; }
  SdBuf& operator=(SdBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      s = o.s;
      o.p = nullptr;
    }
    return *this;
  }
  int get(size_t bytes, cudaStream_t st) {
    release();
    s = st;
    const cudaError_t e = cudaMallocAsync(&p, bytes ? bytes : 8, st);
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_fail(e, "cudaMallocAsync");
    }
    return XG_OK;
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
  }
  ~SdBuf() { release(); }
};

// the moments of items [base, base + items) of the list (or of the elements)
int sd_bfs_chunk(const double* d_vals10, const int32_t* d_list, int64_t base, int64_t items, int levels,
                 double* d_out35, int* d_err, cudaStream_t s) {
  // roots
  SdBuf b_cur;
  if (int st = b_cur.get(sizeof(SdNode) * items, s)) return st;
  {
    std::vector<SdNode> h(items);
    for (int64_t i = 0; i < items; i++) h[i] = SdNode{(int32_t)i, 0u};
    XG_CUDA(cudaMemcpyAsync(b_cur.p, h.data(), sizeof(SdNode) * items, cudaMemcpyHostToDevice, s));
    XG_CUDA(cudaStreamSynchronize(s));  // h leaves scope
  }
  std::vector<SdBuf> plain_b, pdepth_b, cutb;
  std::vector<int64_t> nplain;
  int64_t ncut = 0;
  SdBuf cut_final;
  SdNode* cur = (SdNode*)b_cur.p;
  SdBuf next_b;
  int64_t nn = items;
  SdBuf cur_owner;
  for (int depth = 0; depth <= levels && nn > 0; depth++) {
    const int lev = levels - depth;
    SdBuf w;
    const int nb = (int)((3 * nn + kSdScan - 1) / kSdScan);
    if (int st = w.get(nn + 8 * 6 * nn + 4 * (size_t)nb + 64, s)) return st;
    uint8_t* cls = (uint8_t*)w.p;
    int32_t* cnt3 = (int32_t*)(((uintptr_t)w.p + nn + 15) & ~(uintptr_t)15);
    int32_t* pos3 = cnt3 + 3 * nn;
    int32_t* tots = pos3 + 3 * nn;
    int32_t* bsum = tots + 4;
    k_sd_classify<<<sd_grid(nn), 128, 0, s>>>(cur, nn, d_vals10, d_list, base, depth, lev, cls, cnt3);
    for (int q = 0; q < 3; q++)
      if (int st = sd_scan(cnt3 + q * nn, nn, pos3 + q * nn, bsum, tots + q, s)) return st;
    int32_t h_t[3];
    XG_CUDA(cudaMemcpyAsync(h_t, tots, sizeof(h_t), cudaMemcpyDeviceToHost, s));
    XG_CUDA(cudaStreamSynchronize(s));
    SdBuf nb_next, nb_plain, nb_pd, nb_cut;
    if (int st = nb_next.get(sizeof(SdNode) * (size_t)h_t[0], s)) return st;
    if (int st = nb_plain.get(sizeof(SdNode) * (size_t)h_t[1], s)) return st;
    if (int st = nb_pd.get(sizeof(int32_t) * (size_t)h_t[1], s)) return st;
    if (int st = nb_cut.get(sizeof(SdNode) * (size_t)h_t[2], s)) return st;
    k_sd_emit<<<sd_grid(nn), 128, 0, s>>>(cur, nn, cls, pos3, depth, 8, (SdNode*)nb_next.p, (SdNode*)nb_plain.p,
                                          (SdNode*)nb_cut.p, (int32_t*)nb_pd.p);
    XG_CUDA(cudaGetLastError());
    nplain.push_back(h_t[1]);
    plain_b.push_back(std::move(nb_plain));
    pdepth_b.push_back(std::move(nb_pd));
    if (h_t[2] > 0) {
      ncut = h_t[2];  // cut leaves appear only at level 0 (the last depth)
      cut_final = std::move(nb_cut);
    }
    cur_owner = std::move(next_b);
    next_b = std::move(nb_next);
    cur = (SdNode*)next_b.p;
    nn = h_t[0];
  }
  // plain leaves of all levels in one array (level-major), cut leaves
  int64_t np = 0;
  for (int64_t x : nplain) np += x;
  SdBuf allp, alld, mp, mc;
  if (int st = allp.get(sizeof(SdNode) * np, s)) return st;
  if (int st = alld.get(sizeof(int32_t) * np, s)) return st;
  if (int st = mp.get(sizeof(double) * 35 * np, s)) return st;
  if (int st = mc.get(sizeof(double) * 35 * ncut, s)) return st;
  SdSegs segs = {};
  segs.n = (int)nplain.size();
  int64_t o = 0;
  for (size_t q = 0; q < nplain.size(); q++) {
    segs.off[q] = o;
    if (nplain[q]) {
      XG_CUDA(cudaMemcpyAsync((SdNode*)allp.p + o, plain_b[q].p, sizeof(SdNode) * nplain[q], cudaMemcpyDeviceToDevice, s));
      XG_CUDA(cudaMemcpyAsync((int32_t*)alld.p + o, pdepth_b[q].p, sizeof(int32_t) * nplain[q],
                              cudaMemcpyDeviceToDevice, s));
    }
    o += nplain[q];
  }
  segs.off[nplain.size()] = o;
  if (np > 0)
    k_sd_fill<<<sd_grid(np), 128, 0, s>>>((const SdNode*)allp.p, (const int32_t*)alld.p, np, 0, d_vals10, d_list, base,
                                          (double*)mp.p, d_err);
  if (ncut > 0)
    k_sd_fill<<<sd_grid(ncut), 128, 0, s>>>((const SdNode*)cut_final.p, nullptr, ncut, levels, d_vals10, d_list, base,
                                            (double*)mc.p, d_err);
  k_sd_reduce<<<sd_grid(items * 35), 128, 0, s>>>(items, (const SdNode*)allp.p, (const double*)mp.p, segs,
                                                  (const SdNode*)cut_final.p, (const double*)mc.p, ncut, d_list, base,
                                                  d_out35);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_sd_bfs");
}

// ---- breadth-first Integrate --------------------------------------------------------
// The same level-by-level tree for the elements of a mesh and a level set of
// order K given by its H1 coefficients: nodes (element, path), per level a
// classification (the roots outside the element set drop out), the leaves
// filled one thread each with the integrand x^e, and the leaf values summed
// in a fixed order (block ranges, then the blocks, then the chunks).

struct SdMesh {
  int ne, nv;
  const int32_t* elv;
  const double* xyz;
  const int32_t* el_dofs;  // [nd][ne]
  const double* coefs;
  const uint64_t* defined_on;
};

template <int D, int K>
__device__ __forceinline__ void sdi_elem(const SdMesh& M, int64_t e, sd::Elem<D, K>& el) {
  int gv[4] = {0, 0, 0, 0};
  double xv[4][3];
  for (int v = 0; v <= D; v++) {
    gv[v] = M.elv[(int64_t)v * M.ne + e];
    for (int c = 0; c < 3; c++) xv[v][c] = c < D ? M.xyz[(int64_t)c * M.nv + gv[v]] : 0.0;
  }
  for (int r = 0; r < 3; r++) {
    el.x0[r] = xv[D][r];
    for (int c = 0; c < 3; c++) el.F[r][c] = c < D ? xv[c][r] - xv[D][r] : 0.0;
  }
  for (int i = 0; i < sd::Elem<D, K>::N; i++) {
    el.coef[i] = M.coefs[M.el_dofs[(int64_t)i * M.ne + e]];
    el.desc[i] = fn_desc<D, K>(i, gv);
  }
}

template <int D>
__device__ __forceinline__ void sdi_simplex(uint32_t path, int depth, double (*v)[3]) {
  sd::ref_simplex(D, v);
  for (int d = 0; d < depth; d++) {
    double w[4][3];
    sd::child<D>(v, (int)((path >> (3 * d)) & 7u), w);
    for (int i = 0; i < 4; i++)
      for (int r = 0; r < 3; r++) v[i][r] = w[i][r];
  }
}

template <int D, int K>
__global__ void __launch_bounds__(128) k_sdi_classify(const SdNode* __restrict__ nodes, int64_t nn, SdMesh M,
                                                      int64_t base, int depth, int lev, int dt,
                                                      uint8_t* __restrict__ cls, int32_t* __restrict__ cnt3) {
  constexpr int NC = D == 2 ? 4 : 8;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x) {
    const SdNode nd = nodes[i];
    const int64_t e = base + nd.item;
    int c = SD_NONE;
    if (depth > 0 || !M.defined_on || sd_bit(M.defined_on, e)) {
      sd::Elem<D, K> el;
      sdi_elem<D, K>(M, e, el);
      double v[4][3];
      sdi_simplex<D>(nd.path, depth, v);
      const int dself = sd::lattice_domain(el, v, lev);
      if (dself != XG_IF) {
        c = dself == dt ? SD_PLAIN : SD_NONE;
      } else if (lev == 0) {
        double l[4];
        for (int k = 0; k <= D; k++) l[k] = sd::lset_at(el, v[k]);
        const int dv = sd::vertex_domain(l, D + 1);
        c = dv == XG_IF ? SD_CUT : (dv == dt ? SD_PLAIN : SD_NONE);
      } else {
        c = SD_EXPAND;
      }
    }
    cls[i] = (uint8_t)c;
    cnt3[i] = c == SD_EXPAND ? NC : 0;
    cnt3[nn + i] = c == SD_PLAIN ? 1 : 0;
    cnt3[2 * nn + i] = c == SD_CUT ? 1 : 0;
  }
}

// one thread per leaf: the integral of x^e over its part
template <int D, int K>
__global__ void __launch_bounds__(128) k_sdi_fill(const SdNode* __restrict__ leaves,
                                                  const int32_t* __restrict__ depths, int64_t nl, int cut_depth,
                                                  SdMesh M, int64_t base, int dt, int order, int ex, int ey, int ez,
                                                  double* __restrict__ val, int* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl; i += (int64_t)gridDim.x * blockDim.x) {
    const SdNode nd = leaves[i];
    sd::Elem<D, K> el;
    sdi_elem<D, K>(M, base + nd.item, el);
    double v[4][3];
    sdi_simplex<D>(nd.path, depths ? depths[i] : cut_depth, v);
    double acc = 0.0;
    auto emit = [&](const double* x, double w) {
      acc += w * sd_ipow(x[0], ex) * sd_ipow(x[1], ey) * (D == 3 ? sd_ipow(x[2], ez) : 1.0);
    };
    if (depths) {
      sd::fill(&g_sd_rules, el, v, (const double*)nullptr, dt, order, emit);
    } else {
      double l[4];
      for (int k = 0; k <= D; k++) l[k] = sd::lset_at(el, v[k]);
      const int st = sd::fill(&g_sd_rules, el, v, l, dt, order, emit);
      if (st) set_err(err, st);
    }
    val[i] = acc;
  }
}

// fixed-order sum of n values: block b sums its range [b * per, (b + 1) * per)
// in a tree, then one thread adds the blocks' sums in order into out
__global__ void __launch_bounds__(kSdThreads) k_sdi_blocks(const double* __restrict__ v, int64_t n,
                                                          double* __restrict__ bs) {
  __shared__ double red[kSdThreads];
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = blockIdx.x * per, b1 = b0 + per < n ? b0 + per : n;
  double acc = 0.0;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) acc += v[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int st = kSdThreads / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) bs[blockIdx.x] = red[0];
}

template <int D, int K>
int sdi_chunk(const SdMesh& M, int64_t base, int64_t items, int levels, int dt, int order, int ex, int ey, int ez,
              double* d_partial, int* d_err, cudaStream_t s) {
  constexpr int NC = D == 2 ? 4 : 8;
  SdBuf b_cur;
  if (int st = b_cur.get(sizeof(SdNode) * items, s)) return st;
  {
    std::vector<SdNode> h(items);
    for (int64_t i = 0; i < items; i++) h[i] = SdNode{(int32_t)i, 0u};
    XG_CUDA(cudaMemcpyAsync(b_cur.p, h.data(), sizeof(SdNode) * items, cudaMemcpyHostToDevice, s));
    XG_CUDA(cudaStreamSynchronize(s));
  }
  std::vector<SdBuf> plain_b, pdepth_b;
  std::vector<int64_t> nplain;
  int64_t ncut = 0;
  SdBuf cut_final, next_b, cur_owner;
  SdNode* cur = (SdNode*)b_cur.p;
  int64_t nn = items;
  for (int depth = 0; depth <= levels && nn > 0; depth++) {
    const int lev = levels - depth;
    SdBuf w;
    const int nb = (int)((3 * nn + kSdScan - 1) / kSdScan);
    if (int st = w.get(nn + 8 * 6 * nn + 4 * (size_t)nb + 64, s)) return st;
    uint8_t* cls = (uint8_t*)w.p;
    int32_t* cnt3 = (int32_t*)(((uintptr_t)w.p + nn + 15) & ~(uintptr_t)15);
    int32_t* pos3 = cnt3 + 3 * nn;
    int32_t* tots = pos3 + 3 * nn;
    int32_t* bsum = tots + 4;
    k_sdi_classify<D, K><<<sd_grid(nn), 128, 0, s>>>(cur, nn, M, base, depth, lev, dt, cls, cnt3);
    for (int q = 0; q < 3; q++)
      if (int st = sd_scan(cnt3 + q * nn, nn, pos3 + q * nn, bsum, tots + q, s)) return st;
    int32_t h_t[3];
    XG_CUDA(cudaMemcpyAsync(h_t, tots, sizeof(h_t), cudaMemcpyDeviceToHost, s));
    XG_CUDA(cudaStreamSynchronize(s));
    SdBuf nb_next, nb_plain, nb_pd, nb_cut;
    if (int st = nb_next.get(sizeof(SdNode) * (size_t)h_t[0], s)) return st;
    if (int st = nb_plain.get(sizeof(SdNode) * (size_t)h_t[1], s)) return st;
    if (int st = nb_pd.get(sizeof(int32_t) * (size_t)h_t[1], s)) return st;
    if (int st = nb_cut.get(sizeof(SdNode) * (size_t)h_t[2], s)) return st;
    k_sd_emit<<<sd_grid(nn), 128, 0, s>>>(cur, nn, cls, pos3, depth, NC, (SdNode*)nb_next.p, (SdNode*)nb_plain.p,
                                          (SdNode*)nb_cut.p, (int32_t*)nb_pd.p);
    XG_CUDA(cudaGetLastError());
    nplain.push_back(h_t[1]);
    plain_b.push_back(std::move(nb_plain));
    pdepth_b.push_back(std::move(nb_pd));
    if (h_t[2] > 0) {
      ncut = h_t[2];  // cut leaves appear only at level 0 (the last depth)
      cut_final = std::move(nb_cut);
    }
    cur_owner = std::move(next_b);
    next_b = std::move(nb_next);
    cur = (SdNode*)next_b.p;
    nn = h_t[0];
  }
  // values of the plain leaves (level-major) and the cut leaves, then their sum
  int64_t np = 0;
  for (int64_t x : nplain) np += x;
  SdBuf vals, bs;
  if (int st = vals.get(sizeof(double) * (np + ncut), s)) return st;
  if (int st = bs.get(sizeof(double) * kSdBlocks, s)) return st;
  double* val = (double*)vals.p;
  int64_t o = 0;
  for (size_t q = 0; q < nplain.size(); q++) {
    if (nplain[q])
      k_sdi_fill<D, K><<<sd_grid(nplain[q]), 128, 0, s>>>((const SdNode*)plain_b[q].p, (const int32_t*)pdepth_b[q].p,
                                                          nplain[q], 0, M, base, dt, order, ex, ey, ez, val + o, d_err);
    o += nplain[q];
  }
  if (ncut > 0)
    k_sdi_fill<D, K><<<sd_grid(ncut), 128, 0, s>>>((const SdNode*)cut_final.p, nullptr, ncut, levels, M, base, dt,
                                                    order, ex, ey, ez, val + o, d_err);
  const int64_t nv = np + ncut;
  const int nbk = (int)(nv < kSdBlocks * (int64_t)kSdThreads ? (nv + kSdThreads - 1) / kSdThreads : kSdBlocks);
  if (nv > 0) {
    k_sdi_blocks<<<nbk, kSdThreads, 0, s>>>(val, nv, (double*)bs.p);
    k_sd_sum<<<1, 32, 0, s>>>((const double*)bs.p, nbk, d_partial);
  } else {
    XG_CUDA(cudaMemsetAsync(d_partial, 0, sizeof(double), s));
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_sdi");
}

template <int D, int K>
int sdi_run(const SdMesh& M, int levels, int dt, int order, int ex, int ey, int ez, double* d_result, int* d_err,
            cudaStream_t s) {
  const int64_t chunk = (int64_t)1 << 15, ne = M.ne;
  const int64_t nch = (ne + chunk - 1) / chunk;
  SdBuf parts;
  if (int st = parts.get(sizeof(double) * (nch > 0 ? nch : 1), s)) return st;
  for (int64_t c = 0; c < nch; c++) {
    const int64_t b = c * chunk, m = ne - b < chunk ? ne - b : chunk;
    if (int st = sdi_chunk<D, K>(M, b, m, levels, dt, order, ex, ey, ez, (double*)parts.p + c, d_err, s)) return st;
  }
  if (nch > 0) k_sd_sum<<<1, 32, 0, s>>>((const double*)parts.p, (int)nch, d_result);
  else XG_CUDA(cudaMemsetAsync(d_result, 0, sizeof(double), s));
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_sd_sum");
}

}  // namespace

int subdiv_moments_launch(const double* d_vals10, int64_t n, int levels, double* d_out35, const int32_t* d_list,
                          const int32_t* d_count, int* d_err, cudaStream_t s) {
  int64_t items = n;
  if (d_list) {
    int32_t c = 0;
    XG_CUDA(cudaMemcpyAsync(&c, d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    XG_CUDA(cudaStreamSynchronize(s));
    items = c < 0 ? 0 : (c > n ? n : c);
  }
  // chunks of items keep the leaf arrays bounded (about 130 leaves per cut
  // element at level 3, 35 moments each)
  const int64_t chunk = (int64_t)1 << 15;
  for (int64_t b = 0; b < items; b += chunk) {
    const int64_t m = items - b < chunk ? items - b : chunk;
    if (int st = sd_bfs_chunk(d_vals10, d_list, b, m, levels, d_out35, d_err, s)) return st;
  }
  return XG_OK;
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
  SdMesh M;
  M.ne = m->ne;
  M.nv = m->nv;
  M.elv = m->d_elv;
  M.xyz = m->d_xyz;
  M.el_dofs = sp->d_el_dofs;
  M.coefs = d_lset_coefs;
  M.defined_on = d_defined_on;
  const int D = m->dim, K = sp->order;
  if (D == 2) {
    if (K == 1) return sdi_run<2, 1>(M, subdivlvl, dt, order, ex, ey, ez, d_result, m->d_err, s);
    if (K == 2) return sdi_run<2, 2>(M, subdivlvl, dt, order, ex, ey, ez, d_result, m->d_err, s);
    return sdi_run<2, 3>(M, subdivlvl, dt, order, ex, ey, ez, d_result, m->d_err, s);
  }
  if (K == 1) return sdi_run<3, 1>(M, subdivlvl, dt, order, ex, ey, ez, d_result, m->d_err, s);
  if (K == 2) return sdi_run<3, 2>(M, subdivlvl, dt, order, ex, ey, ez, d_result, m->d_err, s);
  return sdi_run<3, 3>(M, subdivlvl, dt, order, ex, ey, ez, d_result, m->d_err, s);
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

// Marking, rule export and integration kernels of libxg.
// This translation unit is compiled with -fmad=false: cut points, sub-simplex
// volumes, cut ratios and rule points/weights follow the CPU statement of
// ngsxfem's straightcutrule.cpp operation by operation.
#include <algorithm>
#include <mutex>

#include "xg_cut.cuh"
#include "xg_internal.h"

namespace xg {

static __constant__ RuleTable c_rules;

int upload_rules_asm();  // xg_asm.cu
int upload_rules_st();   // xg_st.cu
int upload_rules_lf();   // xg_lf.cu

int ensure_device_rules() {
  static std::mutex mu;
  static std::vector<int> done;
  int dev = 0;
  XG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if (std::find(done.begin(), done.end(), dev) != done.end()) return XG_OK;
  XG_CUDA(cudaMemcpyToSymbol(c_rules, &host_rules(), sizeof(RuleTable)));
  int st = upload_rules_asm();
  if (!st) st = upload_rules_st();
  if (!st) st = upload_rules_lf();
  if (!st) st = upload_rules_quad();
  if (!st) st = upload_rules_quad_int();
  if (!st) st = upload_rules_mlset();
  if (!st) st = upload_rules_isomesh();
  if (!st) st = upload_rules_skel();
  if (!st) st = upload_rules_subdiv();
  if (!st) st = upload_rules_mlform();
  if (!st) st = upload_rules_bform();
  if (!st) st = upload_rules_cform();
  if (!st) st = upload_rules_qform();
  if (st) return st;
  done.push_back(dev);
  return XG_OK;
}

// ---- InterpolateToP1 perturbation (utils/p1interpol.cpp:104-107) -------------------
__global__ void k_perturb(double* v, int64_t n, double eps) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (fabs(v[i]) < eps) v[i] = eps;
}

// ---- CutInformation::Update, element part (xfem/cutinfo.cpp:83-132) ------------------
// One thread per element, 32 elements per warp; the warp's ballots are the
// 32-bit words of the 8 combined-domain bitsets.
// Pass 1 (thread per element): sign classes by integer tests on the bit
// patterns; uncut elements get their domain, ratio 1 (NEG) or 0 (POS) -- the
// exact value of NEG / (NEG + POS) with one part empty -- and their bits; the
// elements whose signs differ are marked IF in the bitsets and appended to a
// list (warp-aggregated, order irrelevant: every element's result depends on
// its own values only).
template <int D>
__global__ void __launch_bounds__(256) k_cutinfo(int ne, const int32_t* __restrict__ elv,
                                                 const double* __restrict__ lset, uint8_t* __restrict__ dom,
                                                 double* __restrict__ ratio, uint32_t* __restrict__ bits, int64_t nw32,
                                                 int32_t* __restrict__ cutlist) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool valid = e < ne;
  int t = XG_POS;
  if (valid) {
    double l[D + 1];
#pragma unroll
    for (int i = 0; i <= D; i++) l[i] = __ldg(&lset[__ldg(&elv[(int64_t)i * ne + e])]);
    t = check_if_straight_cut(l, D + 1);
    if (t != XG_IF) {
      dom[e] = (uint8_t)t;
      ratio[e] = t == XG_NEG ? 1.0 : 0.0;
    }
  }
  const bool is_cut = valid && t == XG_IF;
  const unsigned mc = __ballot_sync(0xffffffffu, is_cut);
  if (mc) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&cutlist[0], __popc(mc));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (is_cut) cutlist[1 + base + __popc(mc & ((1u << lane) - 1))] = (int32_t)e;
  }
  const unsigned mneg = __ballot_sync(0xffffffffu, valid && t == XG_NEG);
  const unsigned mpos = __ballot_sync(0xffffffffu, valid && t == XG_POS);
  const unsigned many = __ballot_sync(0xffffffffu, valid);
  const int64_t w = e >> 5;
  if (lane == 0 && w < nw32) {
    bits[0 * nw32 + w] = 0u;
    bits[1 * nw32 + w] = mneg;
    bits[2 * nw32 + w] = mpos;
    bits[3 * nw32 + w] = mneg | mpos;
    bits[4 * nw32 + w] = mc;
    bits[5 * nw32 + w] = mneg | mc;
    bits[6 * nw32 + w] = mpos | mc;
    bits[7 * nw32 + w] = many;
  }
}

// Pass 2 (thread per listed element, dense): order-0 cut rules for POS then
// NEG, weights summed in rule order (cutinfo.cpp:92-104); an element whose
// parts are not both non-empty (all level-set values zero) moves from IF to
// its class in the bitsets.
template <int D>
__global__ void __launch_bounds__(128) k_cutinfo_cut(int ne, const int32_t* __restrict__ elv,
                                                     const double* __restrict__ lset, uint8_t* __restrict__ dom,
                                                     double* __restrict__ ratio, uint32_t* __restrict__ bits,
                                                     int64_t nw32, const int32_t* __restrict__ cutlist, int* err) {
  const int n = cutlist[0];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int e = cutlist[1 + k];
    double l[D + 1];
#pragma unroll
    for (int i = 0; i <= D; i++) l[i] = __ldg(&lset[__ldg(&elv[(int64_t)i * ne + e])]);
    double part_vol[2] = {0.0, 0.0};
    P3 cut[4];
    const int nc = calc_if_points<D>(l, cut);  // shared by both passes
#pragma unroll
    for (int pass = 0; pass < 2; pass++) {
      const int np = pass == 0 ? XG_POS : XG_NEG;
      Sub subs[3];
      int ns = nc < 0 ? nc : decompose_cuts<D>(l, np, cut, nc, subs);
      if (ns < 0) {
        set_err(err, -ns);
        ns = 0;
      }
      const double wb = c_rules.w[c_rules.off[D][0]];
      for (int s = 0; s < ns; s++) part_vol[np] += wb * simplex_volume(subs[s].p, D + 1);
    }
    ratio[e] = part_vol[XG_NEG] / (part_vol[XG_NEG] + part_vol[XG_POS]);
    int t;
    if (part_vol[XG_NEG] > 0.0) t = (part_vol[XG_POS] > 0.0) ? XG_IF : XG_NEG;
    else t = XG_POS;
    dom[e] = (uint8_t)t;
    if (t != XG_IF) {
      const int64_t w = e >> 5;
      const uint32_t bit = 1u << (e & 31);
      atomicAnd(&bits[4 * nw32 + w], ~bit);
      atomicAnd(&bits[(t == XG_NEG ? 6 : 5) * nw32 + w], ~bit);
      atomicOr(&bits[(t == XG_NEG ? 1 : 2) * nw32 + w], bit);
      atomicOr(&bits[3 * nw32 + w], bit);
    }
  }
}

template <int D>
int cutinfo_launch(int n, const int32_t* elv, const double* d_lset, uint8_t* d_dom, double* d_ratio, uint64_t* d_bits,
                   int64_t nw64, int32_t* cutlist, int* err, cudaStream_t s) {
  XG_CUDA(cudaMemsetAsync(cutlist, 0, sizeof(int32_t), s));
  k_cutinfo<D><<<(unsigned)((nw64 * 64 + 255) / 256), 256, 0, s>>>(n, elv, d_lset, d_dom, d_ratio,
                                                                   (uint32_t*)d_bits, 2 * nw64, cutlist);
  k_cutinfo_cut<D><<<152 * 4, 128, 0, s>>>(n, elv, d_lset, d_dom, d_ratio, (uint32_t*)d_bits, 2 * nw64, cutlist,
                                           err);
  return XG_OK;
}

// ---- CutInformation::Update, node part (xfem/cutinfo.cpp:134-224) ----------------------
// Nodes (vertices, edges, faces, the element) of IF elements -> cut-neighbouring
// bits; nodes of NEG elements -> NEG (all others stay POS); cells: cut ratio > 0.5 -> NEG.
__global__ void k_cut_nodes(int dim, int ne, const int32_t* __restrict__ elv, const int32_t* __restrict__ el_edges,
                            const int32_t* __restrict__ el_faces, const uint8_t* __restrict__ dom,
                            const double* __restrict__ ratio, unsigned long long* nb_v, unsigned long long* nb_e,
                            unsigned long long* nb_f, unsigned long long* nb_el, uint8_t* dv, uint8_t* de, uint8_t* df,
                            uint8_t* dc) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int t = dom[e], nvl = dim + 1, nle = dim == 2 ? 3 : 6;
  if (t == XG_IF) {
    for (int i = 0; i < nvl; i++) {
      const int v = elv[(int64_t)i * ne + e];
      atomicOr(&nb_v[v >> 6], 1ull << (v & 63));
    }
    for (int j = 0; j < nle; j++) {
      const int k = el_edges[(int64_t)j * ne + e];
      atomicOr(&nb_e[k >> 6], 1ull << (k & 63));
    }
    if (dim == 3)
      for (int j = 0; j < 4; j++) {
        const int k = el_faces[(int64_t)j * ne + e];
        atomicOr(&nb_f[k >> 6], 1ull << (k & 63));
      }
    atomicOr(&nb_el[e >> 6], 1ull << (e & 63));
  } else if (t == XG_NEG) {
    for (int i = 0; i < nvl; i++) dv[elv[(int64_t)i * ne + e]] = XG_NEG;
    for (int j = 0; j < nle; j++) de[el_edges[(int64_t)j * ne + e]] = XG_NEG;
    if (dim == 3)
      for (int j = 0; j < 4; j++) df[el_faces[(int64_t)j * ne + e]] = XG_NEG;
  }
  dc[e] = ratio[e] > 0.5 ? XG_NEG : XG_POS;
}

// ---- GetElementsWithThresholdContribution (xfem/cutinfo.cpp:263-284) -------------------
__global__ void k_threshold(const double* __restrict__ ratio, int64_t n, int dt, double threshold, uint32_t* out,
                            int64_t nw32) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool set = false;
  if (e < n) {
    const double thr = dt == XG_POS ? 1.0 - threshold : threshold;
    set = dt == XG_NEG ? ratio[e] >= thr : ratio[e] <= thr;
  }
  const unsigned m = __ballot_sync(0xffffffffu, set);
  if ((threadIdx.x & 31) == 0 && (e >> 5) < nw32) out[e >> 5] = m;
}

__device__ __forceinline__ bool tbit(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

// ---- GetFacetsWithNeighborTypes (xfem/cutinfo.cpp:476-538) ----------------------------
__global__ void k_facet_mark(int64_t nf, const int32_t* __restrict__ fel, const uint64_t* __restrict__ a,
                             const uint64_t* __restrict__ b, int bnd_a, int bnd_b, int use_and, uint32_t* out,
                             int64_t nw32) {
  const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool set = false;
  if (f < nf) {
    int l = fel[f], r = fel[nf + f];
    bool al = tbit(a, l), bl = tbit(b, l);
    bool ar = r >= 0 ? tbit(a, r) : (bool)bnd_a;
    bool br = r >= 0 ? tbit(b, r) : (bool)bnd_b;
    set = use_and ? ((al && br) || (ar && bl)) : ((al || br) || (ar || bl));
  }
  const unsigned m = __ballot_sync(0xffffffffu, set);
  if ((threadIdx.x & 31) == 0 && (f >> 5) < nw32) out[f >> 5] = m;
}

// ---- GetElementsWithNeighborFacets (xfem/cutinfo.cpp:540-566) --------------------------
__global__ void k_el_nbr_facets(int64_t nf, const int32_t* __restrict__ fel, const uint64_t* __restrict__ fb,
                                unsigned long long* out) {
  const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (f >= nf || !tbit(fb, f)) return;
  for (int s = 0; s < 2; s++) {
    int e = fel[s * nf + f];
    if (e >= 0) atomicOr(&out[e >> 6], 1ull << (e & 63));
  }
}

// ---- StraightCutIntegrationRule export (cutint/straightcutrule.cpp:582-677) ------------
template <int D>
__global__ void k_cut_rules(int ne, const int32_t* __restrict__ elv, const double* __restrict__ xyz, int nv,
                            const double* __restrict__ lset, const int32_t* __restrict__ elems, int n, int dt,
                            int order, int max_pts, int32_t* counts, double* pts, double* wts, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int e = elems[i];
  if (e < 0 || e >= ne) {  // an element number outside the mesh: no read of it
    set_err(err, XG_ERR_ARG);
    counts[i] = 0;
    return;
  }
  double l[D + 1];
  double xv[D + 1][3];
#pragma unroll
  for (int v = 0; v <= D; v++) {
    int vid = elv[(int64_t)v * ne + e];
    l[v] = lset[vid];
#pragma unroll
    for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
  }
  const int cdom = check_if_straight_cut(l, D + 1);
  const int p = clamp_order(order);
  double* P = pts + (int64_t)i * max_pts * 3;
  double* W = wts + (int64_t)i * max_pts;
  if (cdom != XG_IF) {
    if (cdom != dt) { counts[i] = -1; return; }
    const int off = c_rules.off[D][p], cnt = c_rules.cnt[D][p];
    if (cnt > max_pts) { set_err(err, XG_ERR_CAPACITY); counts[i] = 0; return; }
    for (int q = 0; q < cnt; q++) {
      for (int c = 0; c < 3; c++) P[3 * q + c] = c_rules.x[off + q][c];
      W[q] = c_rules.w[off + q];
    }
    counts[i] = cnt;
    return;
  }
  Sub subs[3];
  const int ns = decompose<D>(l, dt, subs);
  if (ns < 0) { set_err(err, -ns); counts[i] = 0; return; }
  const int sd = dt == XG_IF ? D - 1 : D;  // sub-simplex dimension
  const int off = c_rules.off[sd][p], cnt = c_rules.cnt[sd][p];
  if (ns * cnt > max_pts) { set_err(err, XG_ERR_CAPACITY); counts[i] = 0; return; }
  double fac = 1.0;
  if (dt == XG_IF) {
    Geo<D> g;
    make_geo<D>(xv, g);
    fac = if_factor<D>(g, l);
  }
  int k = 0;
  for (int s = 0; s < ns; s++) {
    const double trafofac = simplex_volume(subs[s].p, sd + 1);
    for (int q = 0; q < cnt; q++, k++) {
      double pt[3];
      plain_point(subs[s], sd + 1, c_rules.x[off + q], pt);
      for (int c = 0; c < 3; c++) P[3 * k + c] = pt[c];
      double w = c_rules.w[off + q] * trafofac;
      if (dt == XG_IF) w = w * fac;
      W[k] = w;
    }
  }
  counts[i] = k;
}

// ---- Integrate (cutint/cutintegral.cpp:126-212) ---------------------------------------
// Fixed assignment of elements to threads and a fixed reduction tree make the
// sum deterministic.
constexpr int kIntThreads = 256;

__device__ __forceinline__ double ipow(double x, int e) {
  double r = 1.0;
  for (int i = 0; i < e; i++) r *= x;
  return r;
}

template <int D>
__global__ void k_integrate(int ne, const int32_t* __restrict__ elv, const double* __restrict__ xyz, int nv,
                            const double* __restrict__ lset, int dt, int order, int ex, int ey, int ez,
                            const uint64_t* __restrict__ defined_on, double* block_sums, int* err) {
  __shared__ double red[kIntThreads];
  double acc = 0.0;
  const int p = clamp_order(order);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    if (defined_on && !tbit(defined_on, e)) continue;
    double l[D + 1];
    double xv[D + 1][3];
#pragma unroll
    for (int v = 0; v <= D; v++) {
      int vid = elv[(int64_t)v * ne + e];
      l[v] = lset[vid];
#pragma unroll
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
    }
    Geo<D> g;
    make_geo<D>(xv, g);
    const double meas = fabs(g.det);
    const int cdom = check_if_straight_cut(l, D + 1);
    auto point_value = [&](const double* xi, double w) {
      double x[3] = {0, 0, 0};
#pragma unroll
      for (int i = 0; i < D; i++) {
        double s = g.x0[i];
#pragma unroll
        for (int k = 0; k < D; k++) s += g.F[i][k] * xi[k];
        x[i] = s;
      }
      double fv = ipow(x[0], ex) * ipow(x[1], ey) * (D == 3 ? ipow(x[2], ez) : 1.0);
      acc += w * meas * fv;
    };
    if (cdom != XG_IF) {
      if (cdom != dt) continue;
      const int off = c_rules.off[D][p], cnt = c_rules.cnt[D][p];
      for (int q = 0; q < cnt; q++) point_value(c_rules.x[off + q], c_rules.w[off + q]);
      continue;
    }
    Sub subs[3];
    const int ns = decompose<D>(l, dt, subs);
    if (ns < 0) { set_err(err, -ns); continue; }
    const int sd = dt == XG_IF ? D - 1 : D;
    const int off = c_rules.off[sd][p], cnt = c_rules.cnt[sd][p];
    const double fac = dt == XG_IF ? if_factor<D>(g, l) : 1.0;
    for (int s = 0; s < ns; s++) {
      const double trafofac = simplex_volume(subs[s].p, sd + 1);
      for (int q = 0; q < cnt; q++) {
        double pt[3];
        plain_point(subs[s], sd + 1, c_rules.x[off + q], pt);
        double w = c_rules.w[off + q] * trafofac;
        if (dt == XG_IF) w = w * fac;
        point_value(pt, w);
      }
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kIntThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
}

__global__ void k_sum_fixed(const double* v, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += v[i];
    out[0] = s;
  }
}

// ---- allocation-free Integrate -----------------------------------------------------
// Some callers cannot allocate device memory at the time they integrate: code
// running while a stream is being captured into a CUDA graph (cudaMalloc is
// not allowed there), real-time loops that forbid allocator calls, and hosts
// whose device memory is owned by another allocator.  xg_integrate_noalloc
// serves them: its per-block partial sums live in this file-scope array
// instead of workspace allocated on first use.  Every GPU that loads the
// library holds the array (128 KiB) until the process exits.
constexpr int kNoAllocMaxBlocks = 16384;                      // partial sums held
constexpr int kNoAllocElemsPerBlock = kIntThreads * 16;      // elements per block
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks];

// Device address of g_noalloc_partials on the current device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up once
// per device (with that device current) and cached.
static int noalloc_partials(double** out) {
  static std::mutex mu;
  static std::vector<std::pair<int, double*>> cache;
  int dev = 0;
  XG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  for (auto& c : cache)
    if (c.first == dev) {
      *out = c.second;
      return XG_OK;
    }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
  if (e != cudaSuccess) return cuda_fail(e, "xg_integrate_noalloc: cudaGetSymbolAddress");
  cache.push_back({dev, (double*)p});
  *out = (double*)p;
  return XG_OK;
}


// ---- space-time CutInfo (xfem/cutinfo.cpp:83-132 with time_order = 0) ---------------
// SpaceTimeCutIntegrationRule with space and time orders 0: per time interval
// one time point, per (sub-)simplex one point.
// Space-time CutInfo (cutinfo.cpp:61-132 with the space-time rule of
// spacetimecutrule.cpp:106-244, order 0).  Pass 1 (thread per element): an
// element whose space-time nodal values all have one strict sign and whose
// level set is P0/P1 in time keeps that sign over the whole slab: its domain,
// ratio (1 or 0, the exact NEG / (NEG + POS)) and bits are written here; the
// other elements go to a list (warp-aggregated, order irrelevant) and are left
// out of the class bitsets, which pass 2 completes.
template <int D>
__global__ void __launch_bounds__(128) k_cutinfo_st(int ne, int nv, const int32_t* __restrict__ elv,
                                                    const double* __restrict__ lset_st, int kt,
                                                    uint8_t* __restrict__ dom, double* __restrict__ ratio,
                                                    uint32_t* __restrict__ bits, int64_t nw32,
                                                    int32_t* __restrict__ cutlist) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool valid = e < ne;
  int t = -1;
  if (valid && kt <= 1) {
    bool hp = false, hn = false, hz = false;
    for (int v = 0; v <= D; v++) {
      const int vid = elv[(int64_t)v * ne + e];
      for (int i = 0; i <= kt; i++) {
        const double x = lset_st[(int64_t)i * nv + vid];
        const bool p = d_pos(x), n = d_neg(x);
        hp |= p;
        hn |= n;
        hz |= !p && !n;
      }
    }
    if (!hz && hp != hn) t = hn ? XG_NEG : XG_POS;
  }
  if (t >= 0) {
    dom[e] = (uint8_t)t;
    ratio[e] = t == XG_NEG ? 1.0 : 0.0;
  }
  const bool listed = valid && t < 0;
  const unsigned ml = __ballot_sync(0xffffffffu, listed);
  if (ml) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&cutlist[0], __popc(ml));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (listed) cutlist[1 + base + __popc(ml & ((1u << lane) - 1))] = (int32_t)e;
  }
  const unsigned mneg = __ballot_sync(0xffffffffu, valid && t == XG_NEG);
  const unsigned mpos = __ballot_sync(0xffffffffu, valid && t == XG_POS);
  const unsigned many = __ballot_sync(0xffffffffu, valid);
  const int64_t w = e >> 5;
  if (lane == 0 && w < nw32) {
    bits[0 * nw32 + w] = 0u;
    bits[1 * nw32 + w] = mneg;
    bits[2 * nw32 + w] = mpos;
    bits[3 * nw32 + w] = mneg | mpos;
    bits[4 * nw32 + w] = 0u;
    bits[5 * nw32 + w] = mneg;
    bits[6 * nw32 + w] = mpos;
    bits[7 * nw32 + w] = many;
  }
}

// Pass 2 (thread per listed element, dense): time cut points, order-0 space-time
// rules for POS then NEG, ratio and domain; the class bits are added atomically.
template <int D>
__global__ void __launch_bounds__(128) k_cutinfo_st_cut(int ne, int nv, const int32_t* __restrict__ elv,
                                                        const double* __restrict__ lset_st, int kt,
                                                        uint8_t* __restrict__ dom, double* __restrict__ ratio,
                                                        uint32_t* __restrict__ bits, int64_t nw32,
                                                        const int32_t* __restrict__ cutlist, int* err) {
  const int nlist = cutlist[0];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nlist; k += gridDim.x * blockDim.x) {
    const int e = cutlist[1 + k];
    double lst[3 * (D + 1)];
    for (int v = 0; v <= D; v++) {
      const int vid = elv[(int64_t)v * ne + e];
      for (int i = 0; i <= kt; i++) lst[i * (D + 1) + v] = lset_st[(int64_t)i * nv + vid];
    }
    double cut[2 * (D + 1) + 2];
    const int nc = time_cuts<D>(kt, lst, cut);
    const double w0 = c_rules.w[c_rules.off[D][0]];
    const double wt = c_rules.w[c_rules.off[1][0]];
    const double xt = c_rules.x[c_rules.off[1][0]][0];
    double part_vol[2] = {0.0, 0.0};
#pragma unroll
    for (int pass = 0; pass < 2; pass++) {
      const int np = pass == 0 ? XG_POS : XG_NEG;
      for (int i = 0; i + 1 < nc; i++) {
        const double t0 = cut[i], t1 = cut[i + 1];
        const double tt = t0 + xt * (t1 - t0);
        double l[D + 1];
        lset_at<D>(kt, lst, tt, l);
        const int cls = check_if_straight_cut(l, D + 1);
        if (cls == XG_IF) {
          Sub subs[3];
          int ns = decompose<D>(l, np, subs);
          if (ns < 0) {
            set_err(err, -ns);
            ns = 0;
          }
          for (int q = 0; q < ns; q++) part_vol[np] += w0 * simplex_volume(subs[q].p, D + 1) * wt * (t1 - t0);
        } else if (cls == np) {
          part_vol[np] += w0 * wt * (t1 - t0);
        }
      }
    }
    ratio[e] = part_vol[XG_NEG] / (part_vol[XG_NEG] + part_vol[XG_POS]);
    int t;
    if (part_vol[XG_NEG] > 0.0) t = (part_vol[XG_POS] > 0.0) ? XG_IF : XG_NEG;
    else t = XG_POS;
    dom[e] = (uint8_t)t;
    const int64_t w = e >> 5;
    const uint32_t bit = 1u << (e & 31);
    if (t == XG_NEG) {
      atomicOr(&bits[1 * nw32 + w], bit);
      atomicOr(&bits[3 * nw32 + w], bit);
      atomicOr(&bits[5 * nw32 + w], bit);
    } else if (t == XG_POS) {
      atomicOr(&bits[2 * nw32 + w], bit);
      atomicOr(&bits[3 * nw32 + w], bit);
      atomicOr(&bits[6 * nw32 + w], bit);
    } else {
      atomicOr(&bits[4 * nw32 + w], bit);
      atomicOr(&bits[5 * nw32 + w], bit);
      atomicOr(&bits[6 * nw32 + w], bit);
    }
  }
}

// ---- SpaceTimeCutIntegrationRule export (cutint/spacetimecutrule.cpp:106-244) -------
template <int D>
__global__ void k_st_cut_rules(int ne, const int32_t* __restrict__ elv, const double* __restrict__ xyz, int nv,
                               const double* __restrict__ lset_st, int kt, const int32_t* __restrict__ elems, int n,
                               int dt, int order_space, int order_time, int max_pts, int32_t* counts, double* pts,
                               double* wts, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int e = elems[i];
  if (e < 0 || e >= ne) {  // an element number outside the mesh: no read of it
    set_err(err, XG_ERR_ARG);
    counts[i] = 0;
    return;
  }
  double lst[3 * (D + 1)];
  double xv[D + 1][3];
  for (int v = 0; v <= D; v++) {
    const int vid = elv[(int64_t)v * ne + e];
    for (int kk = 0; kk <= kt; kk++) lst[kk * (D + 1) + v] = lset_st[(int64_t)kk * nv + vid];
#pragma unroll
    for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
  }
  Geo<D> g;
  make_geo<D>(xv, g);
  double cut[2 * (D + 1) + 2];
  const int nc = time_cuts<D>(kt, lst, cut);
  const int ps = clamp_order(order_space < 0 ? 5 : order_space), pt = clamp_order(order_time);
  const int offt = c_rules.off[1][pt], cntt = c_rules.cnt[1][pt];
  const int offs = c_rules.off[D][ps], cnts = c_rules.cnt[D][ps];
  const int sd = dt == XG_IF ? D - 1 : D;
  const int offc = c_rules.off[sd][ps], cntc = c_rules.cnt[sd][ps];
  const int maxsize = 5 * cnts * (nc - 1) * cntt;
  double* P = pts + (int64_t)i * max_pts * 4;
  double* W = wts + (int64_t)i * max_pts;
  int k = 0;
  for (int it = 0; it + 1 < nc; it++) {
    const double t0 = cut[it], t1 = cut[it + 1];
    for (int q = 0; q < cntt; q++) {
      const double tt = t0 + c_rules.x[offt + q][0] * (t1 - t0);
      const double wtq = c_rules.w[offt + q];
      double l[D + 1];
      lset_at<D>(kt, lst, tt, l);
      const int cls = check_if_straight_cut(l, D + 1);
      if (cls == XG_IF) {
        Sub subs[3];
        const int ns = decompose<D>(l, dt, subs);
        if (ns < 0) { set_err(err, -ns); counts[i] = 0; return; }
        if (k + ns * cntc > max_pts) { set_err(err, XG_ERR_CAPACITY); counts[i] = 0; return; }
        const double fac = dt == XG_IF ? if_factor<D>(g, l) : 1.0;
        for (int s = 0; s < ns; s++) {
          const double trafofac = simplex_volume(subs[s].p, sd + 1);
          for (int b = 0; b < cntc; b++, k++) {
            double pt3[3];
            plain_point(subs[s], sd + 1, c_rules.x[offc + b], pt3);
            P[4 * k + 0] = pt3[0]; P[4 * k + 1] = pt3[1]; P[4 * k + 2] = pt3[2]; P[4 * k + 3] = tt;
            double w = c_rules.w[offc + b] * trafofac;
            if (dt == XG_IF) w = w * fac;
            W[k] = w * wtq * (t1 - t0);
          }
        }
      } else if (cls == dt) {
        if (k + cnts > max_pts) { set_err(err, XG_ERR_CAPACITY); counts[i] = 0; return; }
        for (int b = 0; b < cnts; b++, k++) {
          P[4 * k + 0] = c_rules.x[offs + b][0]; P[4 * k + 1] = c_rules.x[offs + b][1];
          P[4 * k + 2] = c_rules.x[offs + b][2]; P[4 * k + 3] = tt;
          W[k] = c_rules.w[offs + b] * wtq * (t1 - t0);
        }
      }
    }
  }
  if (k > maxsize) set_err(err, XG_ERR_CAPACITY);
  counts[i] = k == 0 ? -1 : k;
}

}  // namespace xg

using namespace xg;

static int launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return XG_OK;
}

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// entry points that need simplices (facet topology, the simplex cut kernels)
static int need_simplices(const xg_mesh* m, const char* what) {
  if (!m->tensor) return XG_OK;
  set_last_error(std::string(what) +
                 ": quadrilateral / hexahedral meshes support xg_cut_rules, xg_integrate and xg_cutinfo_update only");
  return XG_ERR_UNSUPPORTED;
}

extern "C" {

int xg_interpolate_p1_perturb(double* d_vals, int64_t n, double eps, void* stream) {
  if (!d_vals || n < 0) return XG_ERR_ARG;
  if (n == 0) return XG_OK;
  unsigned g = nblk(n, 256);
  if (g > 152 * 32) g = 152 * 32;
  k_perturb<<<g, 256, 0, (cudaStream_t)stream>>>(d_vals, n, eps);
  return launch_check("k_perturb");
}

int xg_cutinfo_update(xg_mesh* m, const double* d_lset, uint8_t* d_dom, double* d_ratio, uint64_t* d_bits,
                      void* stream) {
  if (!m) return XG_ERR_ARG;
  if (m->tensor) {
    if (!d_lset || !d_dom || !d_ratio || !d_bits) return XG_ERR_ARG;
    return xg::quad_cutinfo(m, d_lset, d_dom, d_ratio, d_bits, stream);
  }
  return xg::cutinfo_update_ws(m, d_lset, d_dom, d_ratio, d_bits, m->d_cutlist, stream);
}
}  // extern "C"

namespace xg {
int cutinfo_update_ws(xg_mesh* m, const double* d_lset, uint8_t* d_dom, double* d_ratio, uint64_t* d_bits,
                      int32_t* cutlist, void* stream) {
  if (!m || !d_lset || !d_dom || !d_ratio || !d_bits || !cutlist) return XG_ERR_ARG;
  // the grid covers whole 64-bit words so every 32-bit half is written
  const int64_t nw64 = (m->ne + 63) / 64;
  cudaStream_t s = (cudaStream_t)stream;
  int st = m->dim == 2 ? cutinfo_launch<2>(m->ne, m->d_elv, d_lset, d_dom, d_ratio, d_bits, nw64, cutlist,
                                           m->d_err, s)
                       : cutinfo_launch<3>(m->ne, m->d_elv, d_lset, d_dom, d_ratio, d_bits, nw64, cutlist,
                                           m->d_err, s);
  return st ? st : launch_check("k_cutinfo");
}
}  // namespace xg

extern "C" {

int xg_cutinfo_update_bnd(xg_mesh* m, const double* d_lset, uint8_t* d_dom, double* d_ratio, uint64_t* d_bits,
                          void* stream) {
  if (!m || !d_lset || !d_dom || !d_ratio || !d_bits) return XG_ERR_ARG;
  if (int st_t = need_simplices(m, "xg_cutinfo_update_bnd")) return st_t;
  if (m->nbnd == 0) return XG_OK;
  const int64_t nw64 = (m->nbnd + 63) / 64;
  cudaStream_t s = (cudaStream_t)stream;
  // the (D-1)-simplices of the boundary with their vertices in ascending order
  int st = m->dim == 2 ? cutinfo_launch<1>((int)m->nbnd, m->d_bnd_v, d_lset, d_dom, d_ratio, d_bits, nw64,
                                           m->d_cutlist, m->d_err, s)
                       : cutinfo_launch<2>((int)m->nbnd, m->d_bnd_v, d_lset, d_dom, d_ratio, d_bits, nw64,
                                           m->d_cutlist, m->d_err, s);
  return st ? st : launch_check("k_cutinfo (BND)");
}

int xg_cutinfo_nodes(xg_mesh* m, const uint8_t* d_dom, const double* d_ratio, uint64_t* d_nb_v, uint64_t* d_nb_e,
                     uint64_t* d_nb_f, uint64_t* d_nb_el, uint8_t* d_dom_v, uint8_t* d_dom_e, uint8_t* d_dom_f,
                     uint8_t* d_dom_cell, void* stream) {
  if (!m || !d_dom || !d_ratio || !d_nb_v || !d_nb_e || !d_nb_el || !d_dom_v || !d_dom_e || !d_dom_cell ||
      (m->dim == 3 && (!d_nb_f || !d_dom_f)))
    return XG_ERR_ARG;
  if (int st_t = need_simplices(m, "xg_cutinfo_nodes")) return st_t;
  cudaStream_t s = (cudaStream_t)stream;
  XG_CUDA(cudaMemsetAsync(d_nb_v, 0, sizeof(uint64_t) * ((m->nv + 63) / 64), s));
  XG_CUDA(cudaMemsetAsync(d_nb_e, 0, sizeof(uint64_t) * ((m->nedges + 63) / 64), s));
  XG_CUDA(cudaMemsetAsync(d_nb_el, 0, sizeof(uint64_t) * ((m->ne + 63) / 64), s));
  XG_CUDA(cudaMemsetAsync(d_dom_v, XG_POS, (size_t)m->nv, s));
  XG_CUDA(cudaMemsetAsync(d_dom_e, XG_POS, (size_t)m->nedges, s));
  if (m->dim == 3) {
    XG_CUDA(cudaMemsetAsync(d_nb_f, 0, sizeof(uint64_t) * ((m->nfaces + 63) / 64), s));
    XG_CUDA(cudaMemsetAsync(d_dom_f, XG_POS, (size_t)m->nfaces, s));
  }
  k_cut_nodes<<<nblk(m->ne, 256), 256, 0, s>>>(m->dim, m->ne, m->d_elv, m->d_el_edges, m->d_el_faces, d_dom, d_ratio,
                                               (unsigned long long*)d_nb_v, (unsigned long long*)d_nb_e,
                                               (unsigned long long*)d_nb_f, (unsigned long long*)d_nb_el, d_dom_v,
                                               d_dom_e, d_dom_f, d_dom_cell);
  return launch_check("k_cut_nodes");
}

int xg_elements_with_threshold(const double* d_ratio, int64_t n, int dt, double threshold, uint64_t* d_out,
                               void* stream) {
  if (!d_ratio || !d_out || n < 0 || (dt != XG_NEG && dt != XG_POS)) return XG_ERR_ARG;
  if (n == 0) return XG_OK;
  const int64_t nw64 = (n + 63) / 64;
  k_threshold<<<nblk(nw64 * 64, 256), 256, 0, (cudaStream_t)stream>>>(d_ratio, n, dt, threshold, (uint32_t*)d_out,
                                                                      2 * nw64);
  return launch_check("k_threshold");
}

int xg_mesh_check(xg_mesh* m) {
  if (!m) return XG_ERR_ARG;
  int h = 0;
  XG_CUDA(cudaMemcpy(&h, m->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  XG_CUDA(cudaMemset(m->d_err, 0, sizeof(int)));
  if (h) set_last_error(std::string("device error: ") + xg_status_string(h));
  return h;
}

int xg_facets_with_neighbor_types(xg_mesh* m, const uint64_t* d_a, const uint64_t* d_b, int bnd_a, int bnd_b,
                                  int use_and, uint64_t* d_out, void* stream) {
  if (!m || !d_a || !d_b || !d_out) return XG_ERR_ARG;
  if (int st_t = need_simplices(m, "xg_facets_with_neighbor_types")) return st_t;
  const int64_t nw64 = (m->nfacets + 63) / 64;
  k_facet_mark<<<nblk(nw64 * 64, 256), 256, 0, (cudaStream_t)stream>>>(m->nfacets, m->d_facet_els, d_a, d_b, bnd_a,
                                                                       bnd_b, use_and, (uint32_t*)d_out, 2 * nw64);
  return launch_check("k_facet_mark");
}

int xg_elements_with_neighbor_facets(xg_mesh* m, const uint64_t* d_facets, uint64_t* d_out, void* stream) {
  if (!m || !d_facets || !d_out) return XG_ERR_ARG;
  if (int st_t = need_simplices(m, "xg_elements_with_neighbor_facets")) return st_t;
  cudaStream_t s = (cudaStream_t)stream;
  XG_CUDA(cudaMemsetAsync(d_out, 0, sizeof(uint64_t) * ((m->ne + 63) / 64), s));
  k_el_nbr_facets<<<nblk(m->nfacets, 256), 256, 0, s>>>(m->nfacets, m->d_facet_els, d_facets,
                                                         (unsigned long long*)d_out);
  return launch_check("k_el_nbr_facets");
}

int xg_cut_rules_ex(xg_mesh* m, const double* d_lset, const int32_t* d_elems, int32_t n, int dt, int order,
                    int quad_dir_policy, int32_t max_pts, int32_t* d_counts, double* d_pts, double* d_wts,
                    void* stream) {
  if (!m || !d_lset || !d_elems || n < 0 || dt < 0 || dt > 2 || order < 0 || order > kMaxOrder || max_pts <= 0 ||
      !d_counts || !d_pts || !d_wts || quad_dir_policy < 0 || quad_dir_policy > 2)
    return XG_ERR_ARG;
  if (n == 0) return XG_OK;
  if (m->tensor)
    return quad_cut_rules(m, d_lset, d_elems, n, dt, order, quad_dir_policy, max_pts, d_counts, d_pts, d_wts, stream);
  cudaStream_t s = (cudaStream_t)stream;
  if (m->dim == 2)
    k_cut_rules<2><<<nblk(n, 128), 128, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, d_elems, n, dt, order,
                                                max_pts, d_counts, d_pts, d_wts, m->d_err);
  else
    k_cut_rules<3><<<nblk(n, 128), 128, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, d_elems, n, dt, order,
                                                max_pts, d_counts, d_pts, d_wts, m->d_err);
  return launch_check("k_cut_rules");
}

int xg_cut_rules(xg_mesh* m, const double* d_lset, const int32_t* d_elems, int32_t n, int dt, int order,
                 int32_t max_pts, int32_t* d_counts, double* d_pts, double* d_wts, void* stream) {
  return xg_cut_rules_ex(m, d_lset, d_elems, n, dt, order, XG_QUAD_FIND_OPTIMAL, max_pts, d_counts, d_pts, d_wts,
                         stream);
}

int xg_quad_rule_capacity(int dim, int dt, int order) {
  if ((dim != 2 && dim != 3) || dt < 0 || dt > 2 || order < 0 || order > kMaxOrder) return -1;
  return quad_rule_capacity(dim, dt, order);
}

int xg_integrate_ex(xg_mesh* m, const double* d_lset, int dt, int order, int quad_dir_policy, int ex, int ey, int ez,
                    const uint64_t* d_defined_on, double* d_result, void* stream) {
  if (!m || !d_lset || !d_result || dt < 0 || dt > 2 || order < 0 || order > kMaxOrder || ex < 0 || ey < 0 ||
      ez < 0 || quad_dir_policy < 0 || quad_dir_policy > 2)
    return XG_ERR_ARG;
  if (m->tensor)
    return quad_integrate(m, d_lset, dt, order, quad_dir_policy, ex, ey, ez, d_defined_on, d_result, stream);
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = 152 * 4;
  if (m->scratch_bytes < nb * sizeof(double)) {
    cudaFree(m->d_scratch);
    m->d_scratch = nullptr;
    m->scratch_bytes = 0;
    XG_CUDA(cudaMalloc(&m->d_scratch, nb * sizeof(double)));
    m->scratch_bytes = nb * sizeof(double);
  }
  double* bs = (double*)m->d_scratch;
  if (m->dim == 2)
    k_integrate<2><<<nb, kIntThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, dt, order, ex, ey, ez,
                                              d_defined_on, bs, m->d_err);
  else
    k_integrate<3><<<nb, kIntThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, dt, order, ex, ey, ez,
                                              d_defined_on, bs, m->d_err);
  k_sum_fixed<<<1, 32, 0, s>>>(bs, nb, d_result);
  return launch_check("k_integrate");
}

int xg_integrate(xg_mesh* m, const double* d_lset, int dt, int order, int ex, int ey, int ez,
                 const uint64_t* d_defined_on, double* d_result, void* stream) {
  return xg_integrate_ex(m, d_lset, dt, order, XG_QUAD_FIND_OPTIMAL, ex, ey, ez, d_defined_on, d_result, stream);
}

int xg_cutinfo_update_st(xg_mesh* m, const double* d_lset_st, int kt_lset, uint8_t* d_dom, double* d_ratio,
                         uint64_t* d_bits, void* stream) {
  if (!m) return XG_ERR_ARG;
  if (int st_t = need_simplices(m, "xg_cutinfo_update_st")) return st_t;
  return xg::cutinfo_update_st_ws(m, d_lset_st, kt_lset, d_dom, d_ratio, d_bits, m->d_cutlist, stream);
}
}  // extern "C"

namespace xg {
int cutinfo_update_st_ws(xg_mesh* m, const double* d_lset_st, int kt_lset, uint8_t* d_dom, double* d_ratio,
                         uint64_t* d_bits, int32_t* cutlist, void* stream) {
  if (!m || !d_lset_st || !d_dom || !d_ratio || !d_bits || !cutlist || kt_lset < 0 || kt_lset > 2)
    return XG_ERR_ARG;
  const int64_t nw64 = (m->ne + 63) / 64;
  cudaStream_t s = (cudaStream_t)stream;
  XG_CUDA(cudaMemsetAsync(cutlist, 0, sizeof(int32_t), s));
  if (m->dim == 2) {
    k_cutinfo_st<2><<<nblk(nw64 * 64, 128), 128, 0, s>>>(m->ne, m->nv, m->d_elv, d_lset_st, kt_lset, d_dom, d_ratio,
                                                         (uint32_t*)d_bits, 2 * nw64, cutlist);
    k_cutinfo_st_cut<2><<<152 * 8, 128, 0, s>>>(m->ne, m->nv, m->d_elv, d_lset_st, kt_lset, d_dom, d_ratio,
                                                 (uint32_t*)d_bits, 2 * nw64, cutlist, m->d_err);
  } else {
    k_cutinfo_st<3><<<nblk(nw64 * 64, 128), 128, 0, s>>>(m->ne, m->nv, m->d_elv, d_lset_st, kt_lset, d_dom, d_ratio,
                                                         (uint32_t*)d_bits, 2 * nw64, cutlist);
    k_cutinfo_st_cut<3><<<152 * 8, 128, 0, s>>>(m->ne, m->nv, m->d_elv, d_lset_st, kt_lset, d_dom, d_ratio,
                                                 (uint32_t*)d_bits, 2 * nw64, cutlist, m->d_err);
  }
  return launch_check("k_cutinfo_st");
}
}  // namespace xg

extern "C" {

int xg_st_cut_rules(xg_mesh* m, const double* d_lset_st, int kt_lset, const int32_t* d_elems, int32_t n, int dt,
                    int order_space, int order_time, int32_t max_pts, int32_t* d_counts, double* d_pts, double* d_wts,
                    void* stream) {
  if (!m || !d_lset_st || !d_elems || n < 0 || dt < 0 || dt > 2 || kt_lset < 0 || kt_lset > 2 || order_space < -1 ||
      order_space > kMaxOrder || order_time < 0 || order_time > kMaxOrder || max_pts <= 0 || !d_counts || !d_pts ||
      !d_wts)
    return XG_ERR_ARG;
  if (int st_t = need_simplices(m, "xg_st_cut_rules")) return st_t;
  if (n == 0) return XG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (m->dim == 2)
    k_st_cut_rules<2><<<nblk(n, 64), 64, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset_st, kt_lset, d_elems, n, dt,
                                                 order_space, order_time, max_pts, d_counts, d_pts, d_wts, m->d_err);
  else
    k_st_cut_rules<3><<<nblk(n, 64), 64, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset_st, kt_lset, d_elems, n, dt,
                                                 order_space, order_time, max_pts, d_counts, d_pts, d_wts, m->d_err);
  return launch_check("k_st_cut_rules");
}

int xg_integrate_noalloc(xg_mesh* m, const double* d_lset, int dt, int order, int ex, int ey, int ez,
                         const uint64_t* d_defined_on, double* d_result, void* stream) {
  if (!m || !d_lset || !d_result || dt < 0 || dt > 2 || order < 0 || order > kMaxOrder || ex < 0 || ey < 0 || ez < 0)
    return XG_ERR_ARG;
  if (int st_t = need_simplices(m, "xg_integrate_noalloc")) return st_t;
  const int64_t nb64 = (m->ne + kNoAllocElemsPerBlock - 1) / kNoAllocElemsPerBlock;
  if (nb64 > kNoAllocMaxBlocks) {
    set_last_error("xg_integrate_noalloc: the mesh has " + std::to_string(m->ne) + " elements; the static scratch of " +
                   std::to_string(kNoAllocMaxBlocks) + " partial sums covers at most " +
                   std::to_string((int64_t)kNoAllocMaxBlocks * kNoAllocElemsPerBlock) + " elements");
    return XG_ERR_CAPACITY;
  }
  const int nb = nb64 < 1 ? 1 : (int)nb64;
  double* partials = nullptr;
  int st = noalloc_partials(&partials);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (m->dim == 2)
    k_integrate<2><<<nb, kIntThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, dt, order, ex, ey, ez,
                                              d_defined_on, partials, m->d_err);
  else
    k_integrate<3><<<nb, kIntThreads, 0, s>>>(m->ne, m->d_elv, m->d_xyz, m->nv, d_lset, dt, order, ex, ey, ez,
                                              d_defined_on, partials, m->d_err);
  k_sum_fixed<<<1, 32, 0, s>>>(partials, nb, d_result);
  return launch_check("xg_integrate_noalloc");
}

}  // extern "C"

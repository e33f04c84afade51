// Assembly kernels of libxg: work-list compaction, cut element matrices,
// facet-patch (ghost-penalty) matrices and the deterministic row-wise scatter
// into a compressed-row matrix, plus the xg_form object and the CutFEM step.
//
// Reference behaviour:
//   SymbolicCutBilinearFormIntegrator::T_CalcElementMatrixAdd  xfem/symboliccutbfi.cpp:76-486
//   SymbolicFacetPatchBilinearFormIntegrator::T_CalcFacetMatrix xfem/symboliccutbfi.cpp:1982-2377
//   MapPatchIntegrationPoint                                   xfem/symboliccutbfi.cpp:1747-1846
//   RestrictedBilinearForm graph / Restrict()                  utils/restrictedblf.cpp:7-168
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "xg_basis.cuh"
#include "xg_cut.cuh"
#include "xg_internal.h"
#include "xg_rows.h"
#include "xg_moments.cuh"
#include "xg_patch.cuh"

namespace xg {

static __constant__ RuleTable c_rules;
// FP32 copy of the rule points and weights: the mixed kernels place their
// quadrature points in FP32 (the FP64 pipe of GB300 is narrow)
struct RuleTableF {
  float x[kRuleCap][3];
  float w[kRuleCap];
};
static __constant__ RuleTableF c_rules_f;

int upload_mono();

int upload_rules_asm() {
  XG_CUDA(cudaMemcpyToSymbol(c_rules, &host_rules(), sizeof(RuleTable)));
  static RuleTableF rf;
  const RuleTable& R = host_rules();
  for (int q = 0; q < kRuleCap; q++) {
    for (int k = 0; k < 3; k++) rf.x[q][k] = (float)R.x[q][k];
    rf.w[q] = (float)R.w[q];
  }
  XG_CUDA(cudaMemcpyToSymbol(c_rules_f, &rf, sizeof(RuleTableF)));
  return upload_mono();
}

__device__ __forceinline__ bool tbit(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }
__device__ __forceinline__ bool tbit32(const uint32_t* b, int64_t i) { return (b[i >> 5] >> (i & 31)) & 1u; }

// ============================================================================
// Compaction of a bitset into an ascending index list (deterministic):
// block popcounts -> single-block scan -> per-block write.
// ============================================================================
constexpr int kCThreads = 256;
constexpr int kCWarpWords = 16;                            // words per warp
constexpr int kCChunk = (kCThreads / 32) * kCWarpWords;     // 32-bit words per block

__device__ __forceinline__ int block_excl_scan_int(int v, int* total, int* sm /* >= 32 */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int t = lane < nw ? sm[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    sm[lane] = t;  // inclusive warp totals
  }
  __syncthreads();
  int base = wid > 0 ? sm[wid - 1] : 0;
  if (total) *total = sm[nw - 1];
  __syncthreads();
  return base + x - v;
}

__global__ void k_popc_blocks(const uint32_t* __restrict__ bits, int64_t nwords, int* __restrict__ bsum) {
  __shared__ int sm[32];
  const int64_t w = (int64_t)blockIdx.x * kCChunk + threadIdx.x;
  const int c = (threadIdx.x < kCChunk && w < nwords) ? __popc(bits[w]) : 0;
  int total;
  block_excl_scan_int(c, &total, sm);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// single block: in-place exclusive scan of n ints, total -> *total_out (+ *extra if given)
__global__ void k_scan_small(int* __restrict__ v, int n, int* __restrict__ total_out) {
  __shared__ int sm[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += blockDim.x) {
    int i = base + threadIdx.x;
    int x = i < n ? v[i] : 0;
    int tot;
    int ex = block_excl_scan_int(x, &tot, sm);
    if (i < n) v[i] = ex + carry;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total_out = carry;
}

// Warp per kCWarpWords consecutive words: lane l of the warp writes bit l of
// each word, at the word's offset plus the set bits below it (coalesced).
__global__ void k_write_list(const uint32_t* __restrict__ bits, int64_t nwords, const int* __restrict__ boff,
                             int32_t* __restrict__ list, int32_t* __restrict__ slot, const int* __restrict__ slot_base) {
  __shared__ int sm[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int sb = slot_base ? *slot_base : 0;
  const int64_t w0 = (int64_t)blockIdx.x * kCChunk + (int64_t)wid * kCWarpWords;
  const uint32_t mine = (lane < kCWarpWords && w0 + lane < nwords) ? bits[w0 + lane] : 0u;
  // exclusive prefix of the words' counts within the warp, then over the block's warps
  const int cnt = __popc(mine);
  int x = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  const int wtotal = __shfl_sync(0xffffffffu, x, 31);
  const int wexcl = x - cnt;
  if (lane == 0) sm[wid] = wtotal;
  __syncthreads();
  int base = boff[blockIdx.x];
  for (int k = 0; k < wid; k++) base += sm[k];
  const unsigned below = (1u << lane) - 1;
#pragma unroll 4
  for (int k = 0; k < kCWarpWords; k++) {
    const uint32_t word = __shfl_sync(0xffffffffu, mine, k);
    const int off = __shfl_sync(0xffffffffu, wexcl, k);
    if ((word >> lane) & 1u) {
      const int pos = base + off + __popc(word & below);
      const int idx = (int)((w0 + k) * 32 + lane);
      list[pos] = idx;
      if (slot) slot[idx] = pos + sb;
    }
  }
}

// ============================================================================
// Row-pointer scan over int64 counts (n read from the device).
// ============================================================================
constexpr int kSThreads = 256;
constexpr int kSPerThread = 8;
constexpr int kSChunk = kSThreads * kSPerThread;

__device__ __forceinline__ long long block_excl_scan_ll(long long v, long long* total, long long* sm) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[wid] = x;
  __syncthreads();
  if (wid == 0) {
    long long t = lane < nw ? sm[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    sm[lane] = t;
  }
  __syncthreads();
  long long base = wid > 0 ? sm[wid - 1] : 0;
  if (total) *total = sm[nw - 1];
  __syncthreads();
  return base + x - v;
}

__global__ void k_sum64_blocks(const int64_t* __restrict__ v, const int* __restrict__ n_ptr, long long* bsum) {
  __shared__ long long sm[32];
  const int n = *n_ptr;
  int64_t i0 = (int64_t)blockIdx.x * kSChunk + (int64_t)threadIdx.x * kSPerThread;
  long long c = 0;
  for (int k = 0; k < kSPerThread; k++)
    if (i0 + k < n) c += v[i0 + k];
  long long tot;
  block_excl_scan_ll(c, &tot, sm);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void k_scan64_small(long long* v, int nblocks) {
  __shared__ long long sm[32];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nblocks; base += blockDim.x) {
    int i = base + threadIdx.x;
    long long x = i < nblocks ? v[i] : 0;
    long long tot;
    long long ex = block_excl_scan_ll(x, &tot, sm);
    if (i < nblocks) v[i] = ex + carry;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
}

// rowptr[i] = exclusive prefix of cnt, rowptr[n] = total, counts_out[1] = total
__global__ void k_scan64_apply(const int64_t* __restrict__ cnt, const int* __restrict__ n_ptr,
                               const long long* __restrict__ boff, int64_t* __restrict__ rowptr,
                               int64_t* __restrict__ counts_out, int64_t cap_nnz, int* err) {
  __shared__ long long sm[32];
  const int n = *n_ptr;
  int64_t i0 = (int64_t)blockIdx.x * kSChunk + (int64_t)threadIdx.x * kSPerThread;
  long long c[kSPerThread];
  long long s = 0;
  for (int k = 0; k < kSPerThread; k++) {
    c[k] = (i0 + k < n) ? cnt[i0 + k] : 0;
    s += c[k];
  }
  long long tot;
  long long pos = boff[blockIdx.x] + block_excl_scan_ll(s, &tot, sm);
  for (int k = 0; k < kSPerThread; k++) {
    if (i0 + k < n) rowptr[i0 + k] = pos;
    if (i0 + k == n - 1) {
      rowptr[n] = pos + c[k];
      counts_out[0] = n;
      counts_out[1] = pos + c[k];
      if (pos + c[k] > cap_nnz) set_err(err, XG_ERR_CAPACITY);
    }
    pos += c[k];
  }
  if (n == 0 && blockIdx.x == 0 && threadIdx.x == 0) {
    rowptr[0] = 0;
    counts_out[0] = 0;
    counts_out[1] = 0;
  }
}

// ============================================================================
// Active sets
// ============================================================================
// uncut-active: domain of the element equals the domain of a volume group that
// contains it; cut-active: a cut element contained in any volume group.
__global__ void k_active_elements(int ne, const uint8_t* __restrict__ dom, FormDesc form, uint32_t* uncut_bits,
                                  uint32_t* cut_bits, int64_t nw32) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool un = false, cu = false;
  if (e < ne) {
    const int d = dom[e];
    for (int g = 0; g < form.ngroups; g++) {
      const GroupDesc& G = form.g[g];
      bool in = !G.defined_on || tbit(G.defined_on, e);
      if (!in) continue;
      if (d == XG_IF) cu = true;
      else if (G.domain == d) un = true;
    }
  }
  unsigned mu = __ballot_sync(0xffffffffu, un), mc = __ballot_sync(0xffffffffu, cu);
  if ((threadIdx.x & 31) == 0 && (e >> 5) < nw32) {
    uncut_bits[e >> 5] = mu;
    cut_bits[e >> 5] = mc;
  }
}

// space-time forms: an element is active if a volume group contains it; the
// elements uncut in the slab (NEG or POS over the whole slab) and the cut ones
// go to separate lists
__global__ void k_active_st(int ne, const uint8_t* __restrict__ dom, StFormDesc form, uint32_t* uncut_bits,
                            uint32_t* cut_bits, int64_t nw32) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool act = false;
  if (e < ne)
    for (int g = 0; g < form.ngroups; g++)
      if (!form.g[g].defined_on || tbit(form.g[g].defined_on, e)) act = true;
  const bool cut = act && dom[e] == XG_IF;
  const unsigned mu = __ballot_sync(0xffffffffu, act && !cut), mc = __ballot_sync(0xffffffffu, cut);
  if ((threadIdx.x & 31) == 0 && (e >> 5) < nw32) {
    uncut_bits[e >> 5] = mu;
    cut_bits[e >> 5] = mc;
  }
}

__global__ void k_active_facets(int64_t nf, const int32_t* __restrict__ fel, FormDesc form, uint32_t* bits,
                                int64_t nw32) {
  const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool act = false;
  if (f < nf && fel[nf + f] >= 0) {
    for (int p = 0; p < form.npatch; p++)
      if (!form.p[p].defined_on || tbit(form.p[p].defined_on, f)) act = true;
    for (int p = 0; p < form.nskel; p++)
      if (!form.s[p].defined_on || tbit(form.s[p].defined_on, f)) act = true;
  }
  unsigned m = __ballot_sync(0xffffffffu, act);
  if ((threadIdx.x & 31) == 0 && (f >> 5) < nw32) bits[f >> 5] = m;
}

// dofs of active elements and of both elements of active facets
// active dofs: a byte per dof set by every active element and both elements
// of every active facet (idempotent plain stores), then packed into bits by
// warp ballot; the packing pass clears the bytes for the next step
__global__ void k_mark_dofs(int ne, int nd, const int32_t* __restrict__ el_dofs_aos, const int32_t* __restrict__ l_un,
                            const int32_t* __restrict__ l_cut, const int32_t* __restrict__ l_fa,
                            const int* __restrict__ counts, int64_t nf, const int32_t* __restrict__ fel,
                            uint8_t* __restrict__ dof_flag, const int32_t* __restrict__ el_rowslot,
                            uint8_t* __restrict__ act_slot) {
  const int nun = counts[0], ncut = counts[1], nfa = counts[2];
  const int64_t total = (int64_t)(nun + ncut + 2 * nfa) * nd;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t item = t / nd;
    const int j = (int)(t - item * nd);
    int e;
    if (item < nun) e = l_un[item];
    else if (item < nun + ncut) e = l_cut[item - nun];
    else {
      const int64_t q = item - nun - ncut;
      e = fel[(q & 1) * nf + l_fa[q >> 1]];
    }
    dof_flag[el_dofs_aos[(int64_t)e * nd + j]] = 1;
    // spatial scatter: the active element's row slot (xg_rows.h)
    if (act_slot && item < nun + ncut) act_slot[el_rowslot[(int64_t)e * nd + j]] = 1;
  }
}

__global__ void k_pack_dofs(uint8_t* __restrict__ dof_flag, int64_t ndof, uint32_t* __restrict__ bits, int64_t nw32) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool on = i < ndof && dof_flag[i];
  if (on) dof_flag[i] = 0;
  const unsigned m = __ballot_sync(0xffffffffu, on);
  if ((threadIdx.x & 31) == 0 && (i >> 5) < nw32) bits[i >> 5] = m;
}

// ============================================================================
// Element matrices.
//
// FP64 is the narrow pipe of GB300, so the kernels minimise FP64 work:
//  * uncut elements (standard rule on an affine simplex): the rule's sums are
//    pre-contracted on the host into reference tables per term group
//    (mass, gradient pairs, convection), the kernel combines them with
//    G = F^-1 F^-T, |det F| and the coefficients -- the same rule, reassociated;
//  * cut elements: sub-simplex quadrature (StraightCutIntegrationRule) with the
//    contraction over matrix entries, only the upper triangle for symmetric
//    forms;
//  * matrices of symmetric forms are stored as packed upper triangles.
// ============================================================================

// Storage of element and patch matrices.  FP64: full n x n rows (row p
// contiguous), so the scatter reads each matrix row as one segment; kernels
// of symmetric forms compute the upper triangle and store both halves.  FP32
// (mixed): packed upper triangles of symmetric matrices (half the bytes, which
// matters more there than the segment reads).
template <typename T>
__host__ __device__ constexpr bool full_rows() {
  return sizeof(T) == 8;
}
template <typename T>
__host__ __device__ inline int64_t mat_stride(int n, bool sym) {
  return full_rows<T>() || !sym ? (int64_t)n * n : (int64_t)tri_size(n);
}
// entry (p, q) of a matrix of the layout, p <= q when sym
template <typename T>
__device__ __forceinline__ void store_entry(T* __restrict__ m, int n, int p, int q, T v, bool sym) {
  if (full_rows<T>() || !sym) {
    m[p * n + q] = v;
    if (sym && p != q) m[q * n + p] = v;
  } else {
    m[tri_index(p, q, n)] = v;
  }
}
// Output of the element and patch kernels.  Compact (rowslot == nullptr):
// matrix `slot` at m + slot * mat_stride, or at m + slot * n * n with full
// rows in both precisions (`full`: the patch matrices of spatial forms).  Rows
// (element rows of spatial forms, xg_rows.h): row p of matrix `key` at
// m + rowslot[key * n + p] * n, full rows in both precisions.
template <typename T>
__device__ __forceinline__ void store_out(T* __restrict__ m, const int32_t* __restrict__ rowslot, int64_t key,
                                          int64_t slot, int n, int p, int q, T v, bool sym, bool full = false) {
  if (rowslot) {
    const int32_t* rs = rowslot + key * n;
    m[(int64_t)__ldg(&rs[p]) * n + q] = v;
    if (sym && p != q) m[(int64_t)__ldg(&rs[q]) * n + p] = v;
  } else if (full) {  // compact, full rows in both precisions
    T* b = m + slot * (int64_t)n * n;
    b[p * n + q] = v;
    if (sym && p != q) b[q * n + p] = v;
  } else {
    store_entry<T>(m + slot * mat_stride<T>(n, sym), n, p, q, v, sym);
  }
}
template <typename T>
__device__ __forceinline__ T load_entry(const T* __restrict__ m, int n, int p, int q, bool sym) {
  if (full_rows<T>() || !sym) return m[p * n + q];
  return m[p <= q ? tri_index(p, q, n) : tri_index(q, p, n)];
}

// entry k -> (p, q) tables in shared memory
__device__ __forceinline__ void entry_tables(int n, bool sym, unsigned char* ep, unsigned char* eq) {
  const int E = sym ? tri_size(n) : n * n;
  for (int k = threadIdx.x; k < E; k += blockDim.x) {
    int p, q;
    if (sym) {
      p = 0;
      int rem = k;
      while (rem >= n - p) {
        rem -= n - p;
        p++;
      }
      q = p + rem;
    } else {
      p = k / n;
      q = k % n;
    }
    ep[k] = (unsigned char)p;
    eq[k] = (unsigned char)q;
  }
}

// Per-group reference tables of the uncut kernel (device pointers, NULL = kind unused).
struct UncutTabs {
  const double* m[kMaxGroups];  // [E]
  const double* t[kMaxGroups];  // [D(D+1)/2][E] gradient-pair tables, (a<=b) row-major
  const double* c[kMaxGroups];  // [D][E] convection tables (full storage only)
  // FP32 copies for the mixed form's contractions (spatial forms)
  const float* mf[kMaxGroups];
  const float* tf[kMaxGroups];
  const float* cf[kMaxGroups];
  int ok_f;  // the FP32 copies exist
};

// physical-gradient Gram matrix of the barycentric coordinates, G = F^-1 F^-T (a<=b)
// and per group beta = F^-1 b; per element in shared memory
template <int D>
struct UnGeoS {
  double G[D * (D + 1) / 2];
  double beta[kMaxGroups][D];
  double coef[kMaxGroups][5];
  // FP32 copies for the mixed form's contractions
  float Gf[D * (D + 1) / 2];
  float betaf[kMaxGroups][D];
  float coeff[kMaxGroups][5];
  double meas;
  int gv[D + 1];
  int elem, slot, dom;
};

// EPB: elements per block (the autotuner's choice among kUncutEpb)
template <int D, int K, bool SYM, typename T, int EPB_ = 32>
struct UnCfg {
  static constexpr int N = ndof_el(D, K);
  static constexpr int E = SYM ? tri_size(N) : N * N;
  static constexpr int EPB = EPB_;
  static constexpr int NT = 256;
};

// Sign of local function i relative to the canonical orientation of the tables
// (cubic edge functions flip when the edge's global orientation differs).
template <int D, int K>
__device__ __forceinline__ int fn_sign(int i, const int* gv) {
  if (K < 3 || i <= D) return 1;
  int r = i - (D + 1);
  const int nedge = D == 2 ? 3 : 6;
  if (r >= nedge * 2) return 1;
  if ((r & 1) == 0) return 1;
  int a, b;
  local_edge(D, r >> 1, a, b);
  return gv[a] < gv[b] ? 1 : -1;
}

template <int D, int K, bool SYM, typename T, int EPB_>
__global__ void __launch_bounds__(256) k_elmat_uncut(int ne, int nv, const int32_t* __restrict__ elv,
                                                     const double* __restrict__ xyz,
                                                     const uint8_t* __restrict__ dom, FormDesc form, UncutTabs tabs,
                                                     const int32_t* __restrict__ list,
                                                     const int* __restrict__ counts, T* __restrict__ elmat, int* err,
                                                     const int32_t* __restrict__ rowslot) {
  using C = UnCfg<D, K, SYM, T, EPB_>;
  constexpr int N = C::N, E = C::E, EPB = C::EPB, NG = D * (D + 1) / 2;
  __shared__ UnGeoS<D> geo[EPB];
  __shared__ unsigned char ep[E], eq[E];
  entry_tables(N, SYM, ep, eq);
  const int count = counts[0];
  for (int batch = blockIdx.x; batch * EPB < count; batch += gridDim.x) {
    __syncthreads();
    if (threadIdx.x < EPB) {
      UnGeoS<D>& G = geo[threadIdx.x];
      const int idx = batch * EPB + threadIdx.x;
      G.elem = idx < count ? list[idx] : -1;
      G.slot = idx;
      if (G.elem >= 0) {
        const int e = G.elem;
        double xv[D + 1][3];
#pragma unroll
        for (int v = 0; v <= D; v++) {
          const int vid = elv[(int64_t)v * ne + e];
          G.gv[v] = vid;
#pragma unroll
          for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
        }
        Geo<D> g;
        make_geo<D>(xv, g);
        G.meas = fabs(g.det);
        int k = 0;
#pragma unroll
        for (int a = 0; a < D; a++)
#pragma unroll
          for (int b = a; b < D; b++) {
            double s = 0;
#pragma unroll
            for (int c = 0; c < D; c++) s += g.Finv[a][c] * g.Finv[b][c];
            G.G[k++] = s;
          }
        G.dom = dom[e];
        double h = -1.0;
        for (int q = 0; q < form.ngroups; q++) {
          for (int kk = 0; kk < 5; kk++) {
            const int hp = form.g[q].hpow[kk];
            if (hp != 0 && h < 0) h = mesh_h<D>(G.meas);
            // |det F| folded into the coefficients
            G.coef[q][kk] = (hp == 0 ? form.g[q].c[kk] : form.g[q].c[kk] * int_pow(h, hp)) * G.meas;
          }
          if (form.g[q].used & (1 << XG_TERM_CONV))
#pragma unroll
            for (int a = 0; a < D; a++) {
              double s = 0;
#pragma unroll
              for (int c = 0; c < D; c++) s += g.Finv[a][c] * form.g[q].b[c];
              G.beta[q][a] = s;
            }
        }
        if (sizeof(T) == 4) {  // the mixed form contracts in FP32
#pragma unroll
          for (int a = 0; a < D * (D + 1) / 2; a++) G.Gf[a] = (float)G.G[a];
          for (int q = 0; q < form.ngroups; q++) {
#pragma unroll
            for (int kk = 0; kk < 5; kk++) G.coeff[q][kk] = (float)G.coef[q][kk];
            if (form.g[q].used & (1 << XG_TERM_CONV))
#pragma unroll
              for (int a = 0; a < D; a++) G.betaf[q][a] = (float)G.beta[q][a];
          }
        }
      }
    }
    __syncthreads();
    if (sizeof(T) == 4 && tabs.ok_f) {
      // mixed form: FP32 contractions of the FP32 tables, compensated sum over
      // the groups' terms
      for (int t = threadIdx.x; t < EPB * E; t += blockDim.x) {
        const int le = t / E, k = t % E;
        const UnGeoS<D>& G = geo[le];
        if (G.elem < 0) continue;
        Acc<float> v;
        v.init();
        for (int q = 0; q < form.ngroups; q++) {
          const GroupDesc& Gq = form.g[q];
          if (Gq.domain != G.dom || (Gq.defined_on && !tbit(Gq.defined_on, G.elem))) continue;
          if (Gq.used & (1 << XG_TERM_MASS)) v.add(G.coeff[q][0] * __ldg(&tabs.mf[q][k]));
          if (Gq.used & (1 << XG_TERM_LAPLACE)) {
            float s = 0.f;
#pragma unroll
            for (int a = 0; a < NG; a++) s = fmaf(G.Gf[a], __ldg(&tabs.tf[q][a * E + k]), s);
            v.add(G.coeff[q][1] * s);
          }
          if (Gq.used & (1 << XG_TERM_CONV)) {
            float s = 0.f;
#pragma unroll
            for (int a = 0; a < D; a++) s = fmaf(G.betaf[q][a], __ldg(&tabs.cf[q][a * E + k]), s);
            v.add(G.coeff[q][4] * s);
          }
        }
        float r = v.get();
        if (K == 3) r = neg_if(r, fn_sign<D, K>(ep[k], G.gv) != fn_sign<D, K>(eq[k], G.gv));
        if (!isfinite(r)) set_err(err, XG_ERR_NONFINITE);
        store_out<T>(elmat, rowslot, G.elem, G.slot, N, ep[k], eq[k], (T)r, SYM);
      }
      continue;
    }
    for (int t = threadIdx.x; t < EPB * E; t += blockDim.x) {
      const int le = t / E, k = t % E;
      const UnGeoS<D>& G = geo[le];
      if (G.elem < 0) continue;
      double v = 0.0;
      for (int q = 0; q < form.ngroups; q++) {
        const GroupDesc& Gq = form.g[q];
        if (Gq.domain != G.dom || (Gq.defined_on && !tbit(Gq.defined_on, G.elem))) continue;
        if (Gq.used & (1 << XG_TERM_MASS)) v += G.coef[q][0] * __ldg(&tabs.m[q][k]);
        if (Gq.used & (1 << XG_TERM_LAPLACE)) {
          double s = 0;
#pragma unroll
          for (int a = 0; a < NG; a++) s += G.G[a] * __ldg(&tabs.t[q][a * E + k]);
          v += G.coef[q][1] * s;
        }
        if (Gq.used & (1 << XG_TERM_CONV)) {
          double s = 0;
#pragma unroll
          for (int a = 0; a < D; a++) s += G.beta[q][a] * __ldg(&tabs.c[q][a * E + k]);
          v += G.coef[q][4] * s;
        }
      }
      if (K == 3) v = neg_if(v, fn_sign<D, K>(ep[k], G.gv) != fn_sign<D, K>(eq[k], G.gv));
      if (!finite_bits(v)) set_err(err, XG_ERR_NONFINITE);
      store_out<T>(elmat, rowslot, G.elem, G.slot, N, ep[k], eq[k], (T)v, SYM);
    }
  }
}

// ---------------------------------------------------------------------------
// Space-time elements uncut in the slab (NEG or POS at every time of the
// slab): the space-time rule is the time rule times the spatial standard rule
// (cutint/spacetimecutrule.cpp:106-244 with one time interval and a
// sign-definite level set at every time point), so with Phi = psi_a(tau) phi_j
//   mass     sum_t w psi_a psi_b      x  spatial mass table
//   laplace  sum_t w psi_a psi_b      x  sum_ab G_ab x gradient-pair tables
//   conv     sum_r beta_r x convection tables,  beta = F^-1 sum_t w psi_a psi_b b(t)
//   dt       sum_t w psi_a psi_b'     x  spatial mass table
// (fixed-time groups: the single time tref with weight 1) -- the same sums,
// reassociated.  The time sums are built on the host with the form's time rule.
// ---------------------------------------------------------------------------
struct StTimeTabs {
  double tm[kMaxGroups][9];     // sum_t w psi_a psi_b  (a test, b trial time index)
  double td[kMaxGroups][9];     // sum_t w psi_a psi_b'
  double tb[kMaxGroups][9][3];  // sum_t w psi_a psi_b b(t)
};

template <int D, int KT>
struct StUnGeoS {
  double G[D * (D + 1) / 2];
  double beta[kMaxGroups][(KT + 1) * (KT + 1)][D];
  double coef[kMaxGroups][7];
  int elem, slot, dom;
};

template <int D, int K, int KT, typename T>
__global__ void __launch_bounds__(256) k_st_elmat_uncut(int ne, int nv, const int32_t* __restrict__ elv,
                                                         const double* __restrict__ xyz,
                                                         const uint8_t* __restrict__ dom, StFormDesc form,
                                                         UncutTabs tabs, StTimeTabs tt,
                                                         const int32_t* __restrict__ list,
                                                         const int* __restrict__ counts, T* __restrict__ elmat,
                                                         int* err) {
  constexpr int NS = ndof_el(D, K), N = NS * (KT + 1), E = N * N, ES = NS * NS, NTT = (KT + 1) * (KT + 1);
  constexpr int NG = D * (D + 1) / 2, EPB = (D == 3 || KT == 2) ? 16 : 32;
  __shared__ StUnGeoS<D, KT> geo[EPB];
  const int count = counts[0];
  for (int batch = blockIdx.x; batch * EPB < count; batch += gridDim.x) {
    __syncthreads();
    if (threadIdx.x < EPB) {
      StUnGeoS<D, KT>& G = geo[threadIdx.x];
      const int idx = batch * EPB + threadIdx.x;
      G.elem = idx < count ? list[idx] : -1;
      G.slot = idx;
      if (G.elem >= 0) {
        const int e = G.elem;
        double xv[D + 1][3];
#pragma unroll
        for (int v = 0; v <= D; v++) {
          const int vid = elv[(int64_t)v * ne + e];
#pragma unroll
          for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
        }
        Geo<D> g;
        make_geo<D>(xv, g);
        const double meas = fabs(g.det);
        int k = 0;
#pragma unroll
        for (int a = 0; a < D; a++)
#pragma unroll
          for (int b = a; b < D; b++) {
            double s = 0;
#pragma unroll
            for (int c = 0; c < D; c++) s += g.Finv[a][c] * g.Finv[b][c];
            G.G[k++] = s;
          }
        G.dom = dom[e];
        double h = -1.0;
        for (int q = 0; q < form.ngroups; q++) {
          const StGroupDesc& Gq = form.g[q];
          for (int kk = 0; kk < 7; kk++) {
            const int hp = Gq.hpow[kk];
            if (hp != 0 && h < 0) h = mesh_h<D>(meas);
            // |det F| folded into the coefficients
            G.coef[q][kk] = (hp == 0 ? Gq.c[kk] : Gq.c[kk] * int_pow(h, hp)) * meas;
          }
          if (Gq.used & (1 << XG_TERM_CONV))
            for (int ti = 0; ti < NTT; ti++)
#pragma unroll
              for (int a = 0; a < D; a++) {
                double s = 0;
#pragma unroll
                for (int c = 0; c < D; c++) s += g.Finv[a][c] * tt.tb[q][ti][c];
                G.beta[q][ti][a] = s;
              }
        }
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < EPB * E; t += blockDim.x) {
      const int le = t / E, k = t - le * E;
      const StUnGeoS<D, KT>& G = geo[le];
      if (G.elem < 0) continue;
      const int pp = k / N, qv = k - pp * N;
      const int ta = pp / NS, sj = pp - ta * NS, tb = qv / NS, sk = qv - tb * NS;
      const int ks = sj * NS + sk, ti = ta * (KT + 1) + tb;
      double v = 0.0;
      for (int q = 0; q < form.ngroups; q++) {
        const StGroupDesc& Gq = form.g[q];
        if (Gq.domain != G.dom || (Gq.defined_on && !tbit(Gq.defined_on, G.elem))) continue;
        const int used = Gq.used;
        if (used & ((1 << XG_TERM_MASS) | (1 << 6))) {
          double c = 0.0;
          if (used & (1 << XG_TERM_MASS)) c += G.coef[q][XG_TERM_MASS] * tt.tm[q][ti];
          if (used & (1 << 6)) c += G.coef[q][6] * tt.td[q][ti];
          v += c * __ldg(&tabs.m[q][ks]);
        }
        if (used & (1 << XG_TERM_LAPLACE)) {
          double s = 0;
#pragma unroll
          for (int a = 0; a < NG; a++) s += G.G[a] * __ldg(&tabs.t[q][a * ES + ks]);
          v += G.coef[q][XG_TERM_LAPLACE] * tt.tm[q][ti] * s;
        }
        if (used & (1 << XG_TERM_CONV)) {
          double s = 0;
#pragma unroll
          for (int a = 0; a < D; a++) s += G.beta[q][ti][a] * __ldg(&tabs.c[q][a * ES + ks]);
          v += G.coef[q][XG_TERM_CONV] * s;
        }
      }
      if (!finite_bits(v)) set_err(err, XG_ERR_NONFINITE);
      elmat[(int64_t)G.slot * E + k] = (T)v;
    }
  }
}

// ---------------------------------------------------------------------------
// Cut elements: sub-simplex quadrature.  Per chunk of points: point
// generation (FP64), features per function (thread per function), then the
// contraction over matrix entries flattened over the block.
// ---------------------------------------------------------------------------
template <int D, int K, bool SYM, typename T>
struct CutCfg {
  static constexpr int N = ndof_el(D, K);
  static constexpr int E = SYM ? tri_size(N) : N * N;
  static constexpr int EPB = N <= 4 ? 16 : (N <= 10 ? 8 : 4);
  static constexpr int CH = N <= 4 ? 3 : 4;
  static constexpr int NT = N * EPB;
  static constexpr int NACC = (EPB * E + NT - 1) / NT;
  static constexpr int NF = D + 3;  // phi, grad (D), n.grad, b.grad
};

struct CutGeoS {
  double g[4][3];
  double nrm[3];
  double meas;
  double iffac;
  double l[4];
  int gv[4];
  int elem, slot;
  int ns[3];
  double coef[kMaxGroups][5];
};
struct CutSubS {
  Sub sub[3][3];
  double vol[3][3];
};

// Per-element setup of a cut element: geometry, unit normal of the P1 level
// set, coefficients, and the sub-simplices (and their volumes) of the domain
// types the form integrates over.
template <int D>
__device__ void cut_setup(int e, int ne, int nv, const int32_t* __restrict__ elv, const double* __restrict__ xyz,
                          const double* __restrict__ lset, const FormDesc& form, int needs_mask, CutGeoS& G,
                          CutSubS& SS, int* err) {
  G.ns[0] = G.ns[1] = G.ns[2] = 0;
  double xv[D + 1][3];
#pragma unroll
  for (int v = 0; v <= D; v++) {
    const int vid = elv[(int64_t)v * ne + e];
    G.gv[v] = vid;
    G.l[v] = lset[vid];
#pragma unroll
    for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
  }
  Geo<D> g;
  make_geo<D>(xv, g);
  G.meas = fabs(g.det);
  double gs[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; a++)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      G.g[a][k] = k < D ? g.Finv[a][k] : 0.0;
      gs[k] += G.g[a][k];
    }
#pragma unroll
  for (int k = 0; k < 3; k++) G.g[D][k] = -gs[k];
  double gl[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < D; k++) {
    double s = 0;
#pragma unroll
    for (int a = 0; a < D; a++) s += g.Finv[a][k] * (G.l[a] - G.l[D]);
    gl[k] = s;
  }
  const double nn = l2norm3(gl[0], gl[1], gl[2]);
#pragma unroll
  for (int k = 0; k < 3; k++) G.nrm[k] = gl[k] / nn;
  double h = -1.0;
  for (int q = 0; q < form.ngroups; q++)
    for (int k = 0; k < 5; k++) {
      const int hp = form.g[q].hpow[k];
      if (hp != 0 && h < 0) h = mesh_h<D>(G.meas);
      G.coef[q][k] = hp == 0 ? form.g[q].c[k] : form.g[q].c[k] * int_pow(h, hp);
    }
  P3 cut[4];
  const int nc = calc_if_points<D>(G.l, cut);  // shared by the domains
  for (int dt = 0; dt < 3; dt++) {
    if (!((needs_mask >> dt) & 1)) continue;
    int ns = nc < 0 ? nc : decompose_cuts<D>(G.l, dt, cut, nc, SS.sub[dt]);
    if (ns < 0) {
      set_err(err, -ns);
      ns = 0;
    }
    G.ns[dt] = ns;
    const int sd = dt == XG_IF ? D - 1 : D;
    for (int s = 0; s < ns; s++) SS.vol[dt][s] = simplex_volume(SS.sub[dt][s].p, sd + 1);
  }
  G.iffac = ((needs_mask >> XG_IF) & 1) ? if_factor<D>(g, G.l) : 0.0;
}

// thread per cut element (the first cap of the list): cut_setup into global memory
template <int D>
__global__ void k_cut_geo(int ne, int nv, const int32_t* __restrict__ elv, const double* __restrict__ xyz,
                          const double* __restrict__ lset, FormDesc form, const int32_t* __restrict__ list,
                          const int* __restrict__ counts, CutGeoS* __restrict__ cg, CutSubS* __restrict__ cs,
                          int64_t cap, int* err, int needs_mask) {
  const int count = counts[1];
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < count && idx < cap; idx += gridDim.x * blockDim.x) {
    CutGeoS G;
    CutSubS SS;
    G.elem = list[idx];
    G.slot = counts[0] + idx;
    cut_setup<D>(G.elem, ne, nv, elv, xyz, lset, form, needs_mask, G, SS, err);
    cg[idx] = G;
    cs[idx] = SS;
  }
}

// Quadrature-point form of the cut element matrices, for the cut elements
// from `first` on (those beyond the moment workspace; normally none).
template <int D, int K, bool SYM, typename T>
__global__ void __launch_bounds__(CutCfg<D, K, SYM, T>::NT) k_elmat_cut(
    int ne, int nv, const int32_t* __restrict__ elv, const double* __restrict__ xyz, const double* __restrict__ lset,
    FormDesc form, const int32_t* __restrict__ list, const int* __restrict__ counts, T* __restrict__ elmat, int* err,
    int needs_mask, const CutGeoS* __restrict__ cg, const CutSubS* __restrict__ cs, int64_t cap, int first,
    const int32_t* __restrict__ rowslot) {
  using C = CutCfg<D, K, SYM, T>;
  constexpr int N = C::N, E = C::E, EPB = C::EPB, CH = C::CH, NT = C::NT, NACC = C::NACC, NF = C::NF;
  __shared__ CutGeoS geo[EPB];
  __shared__ CutSubS subs[EPB];
  __shared__ T pts[EPB][CH][D + 2];  // barycentric coordinates and w |det F|
  __shared__ T tr[EPB][CH][N][NF];  // trial features: phi, grad, n.grad, b.grad
  __shared__ T te[EPB][CH][N][NF];  // test features scaled by w and the coefficients
  __shared__ unsigned char ep[E], eq[E];
  __shared__ int npts_s[EPB];
  __shared__ int maxpts_s;
  static_assert(sizeof(geo) + sizeof(subs) + sizeof(pts) + sizeof(tr) + sizeof(te) < 48 * 1024,
                "k_elmat_cut shared memory");
  const int count = counts[1];
  if (first >= count) return;
  entry_tables(N, SYM, ep, eq);
  const int slot_base = counts[0];
  const int le = threadIdx.x / N, i = threadIdx.x % N;

  for (int batch = blockIdx.x; first + batch * EPB < count; batch += gridDim.x) {
    __syncthreads();
    if (threadIdx.x < EPB) {
      CutGeoS& G = geo[threadIdx.x];
      const int idx = first + batch * EPB + threadIdx.x;
      if (idx < count && idx < cap) {
        G = cg[idx];
        subs[threadIdx.x] = cs[idx];
      } else {
        G.elem = idx < count ? list[idx] : -1;
        G.slot = slot_base + idx;
        G.ns[0] = G.ns[1] = G.ns[2] = 0;
        if (G.elem >= 0) cut_setup<D>(G.elem, ne, nv, elv, xyz, lset, form, needs_mask, G, subs[threadIdx.x], err);
      }
    }
    __syncthreads();

    const CutGeoS& G = geo[le];
    const int desc = G.elem >= 0 ? fn_desc<D, K>(i, G.gv) : 0;
    T gT[D + 1][D];
#pragma unroll
    for (int a = 0; a <= D; a++)
#pragma unroll
      for (int k = 0; k < D; k++) gT[a][k] = (T)G.g[a][k];
    Acc<T> acc[NACC];
#pragma unroll
    for (int m = 0; m < NACC; m++) acc[m].init();

    for (int q = 0; q < form.ngroups; q++) {
      const GroupDesc& Gq = form.g[q];
      const int p = clamp_order(Gq.order);
      const int dt = Gq.domain;
      const int sd = dt == XG_IF ? D - 1 : D;
      const int nqb = c_rules.cnt[sd][p], offb = c_rules.off[sd][p];
      if (i == 0) {
        int np = 0;
        if (G.elem >= 0 && (!Gq.defined_on || tbit(Gq.defined_on, G.elem))) np = G.ns[dt] * nqb;
        npts_s[le] = np;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        int mx = 0;
        for (int k = 0; k < EPB; k++) mx = max(mx, npts_s[k]);
        maxpts_s = mx;
      }
      __syncthreads();
      const int maxpts = maxpts_s;
      const int np = npts_s[le];
      const T cM = (T)G.coef[q][0], cL = (T)G.coef[q][1], cN1 = (T)G.coef[q][2], cN2 = (T)G.coef[q][3],
              cC = (T)G.coef[q][4];
      const int used = Gq.used;
      T nrmT[3], bT[3];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        nrmT[k] = (T)G.nrm[k];
        bT[k] = (T)Gq.b[k];
      }
      for (int q0 = 0; q0 < maxpts; q0 += CH) {
        if constexpr (sizeof(T) == 4) {
          for (int qq = i; qq < CH; qq += N) {
            const int qi = q0 + qq;
            float w = 0.f, pt[3] = {0.25f, 0.25f, 0.25f};
            if (qi < np) {
              const CutSubS& SS = subs[le];
              const int sidx = qi / nqb, b = qi % nqb;
              const Sub& sub = SS.sub[dt][sidx];
              const float* ip = c_rules_f.x[offb + b];
              float ow = 1.f;
              for (int m = 0; m < sd; ++m) ow -= ip[m];
#pragma unroll
              for (int k = 0; k < 3; k++) pt[k] = ow * (float)sub.p[0].c[k];
              for (int m = 0; m < sd; ++m)
#pragma unroll
                for (int k = 0; k < 3; k++) pt[k] += ip[m] * (float)sub.p[m + 1].c[k];
              w = c_rules_f.w[offb + b] * (float)SS.vol[dt][sidx];
              if (dt == XG_IF) w *= (float)G.iffac;
            }
            float s3 = 0.f;
#pragma unroll
            for (int a = 0; a < D; a++) {
              pts[le][qq][a] = pt[a];
              s3 += pt[a];
            }
            pts[le][qq][D] = 1.f - s3;
            pts[le][qq][D + 1] = w * (float)G.meas;
          }
        } else
        for (int qq = i; qq < CH; qq += N) {
          const int qi = q0 + qq;
          double w = 0.0, pt[3] = {0.25, 0.25, 0.25};
          if (qi < np) {
            const CutSubS& SS = subs[le];
            const int s = qi / nqb, b = qi % nqb;
            plain_point(SS.sub[dt][s], sd + 1, c_rules.x[offb + b], pt);
            w = c_rules.w[offb + b] * SS.vol[dt][s];
            if (dt == XG_IF) w = w * G.iffac;
          }
          double s3 = 0;
#pragma unroll
          for (int a = 0; a < D; a++) {
            pts[le][qq][a] = (T)pt[a];
            s3 += pt[a];
          }
          pts[le][qq][D] = (T)(1.0 - s3);
          pts[le][qq][D + 1] = (T)(w * G.meas);
        }
        __syncthreads();
        // features of function i at the chunk's points (zero weight beyond np);
        // only the parts the group's integrand kinds use
        const bool need_dn = used & ((1 << XG_TERM_NGRADU_V) | (1 << XG_TERM_U_NGRADV));
        const bool need_db = used & (1 << XG_TERM_CONV);
#pragma unroll
        for (int qq = 0; qq < CH; qq++) {
          const T* lam = pts[le][qq];
          T phi, grad[D];
          eval_fn<D, T>(desc, lam, gT, phi, grad);
          T dn = 0, db = 0;
          if (need_dn) {
#pragma unroll
            for (int k = 0; k < D; k++) dn += nrmT[k] * grad[k];
          }
          if (need_db) {
#pragma unroll
            for (int k = 0; k < D; k++) db += bT[k] * grad[k];
          }
          const T w = pts[le][qq][D + 1];
          tr[le][qq][i][0] = phi;
#pragma unroll
          for (int k = 0; k < D; k++) tr[le][qq][i][1 + k] = grad[k];
          tr[le][qq][i][1 + D] = dn;
          tr[le][qq][i][2 + D] = db;
          // test side: v = A phi_q + G.grad_q + E dn_q + F db_q
          T A = 0;
          if (used & (1 << XG_TERM_MASS)) A += cM * phi;
          if (used & (1 << XG_TERM_U_NGRADV)) A += cN2 * dn;
          te[le][qq][i][0] = w * A;
          if (used & (1 << XG_TERM_LAPLACE)) {
            const T wl = w * cL;
#pragma unroll
            for (int k = 0; k < D; k++) te[le][qq][i][1 + k] = wl * grad[k];
          }
          te[le][qq][i][1 + D] = (used & (1 << XG_TERM_NGRADU_V)) ? w * cN1 * phi : (T)0;
          te[le][qq][i][2 + D] = (used & (1 << XG_TERM_CONV)) ? w * cC * phi : (T)0;
        }
        __syncthreads();
        const int nch = min(CH, maxpts - q0);
        const bool uA = used & ((1 << XG_TERM_MASS) | (1 << XG_TERM_U_NGRADV));
        const bool uL = used & (1 << XG_TERM_LAPLACE);
        const bool uE = used & (1 << XG_TERM_NGRADU_V);
        const bool uF = used & (1 << XG_TERM_CONV);
#pragma unroll
        for (int m = 0; m < NACC; m++) {
          const int t = threadIdx.x + m * NT;
          if (t < EPB * E) {
            const int el = t / E, k = t % E, pp = ep[k], qv = eq[k];
            T v = 0;
            for (int qq = 0; qq < nch; qq++) {
              const T* a = te[el][qq][pp];
              const T* b = tr[el][qq][qv];
              if (uA) v += a[0] * b[0];
              if (uL) {
#pragma unroll
                for (int kk = 1; kk <= D; kk++) v += a[kk] * b[kk];
              }
              if (uE) v += a[1 + D] * b[1 + D];
              if (uF) v += a[2 + D] * b[2 + D];
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
      if (t < EPB * E) {
        const int el = t / E, k = t % E;
        if (geo[el].elem >= 0) {
          const T v = acc[m].get();
          if (!isfinite(v)) set_err(err, XG_ERR_NONFINITE);
          store_out<T>(elmat, rowslot, geo[el].elem, geo[el].slot, N, ep[k], eq[k], v, SYM);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Cut elements by barycentric moments.  Every basis function is a polynomial
// in the barycentric coordinates lambda, and so is every integrand of the term
// menu, with element constants in front:
//   mass        phi_p phi_q
//   laplace     grad phi_p . grad phi_q = sum_ab G_ab d_a phi_p d_b phi_q,
//               G_ab = grad lambda_a . grad lambda_b
//   n.grad u v  sum_b nu_b phi_p d_b phi_q,     nu_b = n . grad lambda_b
//   b.grad u v  sum_b beta_b phi_p d_b phi_q,   beta_b = b . grad lambda_b
// (d_a = derivative by lambda_a).  The quadrature sum of the cut rule is
// therefore a fixed integer combination of the rule's moments
//   mu_gamma = sum_x w_x |det F| lambda(x)^gamma
// -- the same sums, reassociated.  k_cut_moments computes the moments of every
// (domain, rule) set of the form; k_cut_entries combines them with integer
// tables built on the host.  Per cut P2 tet this takes about a seventh of the
// FP64 operations of evaluating the functions at every point.
// ---------------------------------------------------------------------------
constexpr int kMomPts = 128, kMomNT = 256;  // points per chunk of a block, threads
// elements per block of the moment kernel (x points per element = kMomPts):
// 8 x 16 for tets, 16 x 8 for triangles (measured)
template <int D>
__host__ __device__ constexpr int mom_epb() {
  return D == 3 ? 8 : 16;
}
constexpr int kEntEPB = 32, kEntNT = 256;


// moment index m -> (index of (e0, e1) in the pair table A, index of (e2, e3)
// (3D) or e2 (2D) in the table B), graded order; [0] 2D (84 used), [1] 3D (210)
static __constant__ uint16_t c_mono[2][210];

struct MomDesc {
  int nsets;
  int dt[kMaxGroups], order[kMaxGroups], deg[kMaxGroups], M[kMaxGroups], off[kMaxGroups];
  int set_of[kMaxGroups];  // moment set of every group
  int MT;                  // moments per element over all sets
  int NA, NB;              // widest power-pair tables
};

struct EntTabs {
  const int32_t* ptr[4];  // [E+1] term offsets per entry: MASS, LAP, PD, DP
  const int32_t* idx[4];  // monomial | aux << 16 (aux: packed (a <= b) for LAP, b for PD/DP)
  const void* coef[4];    // integer coefficients in the kernel's precision
};

// A[pair(e0, e1)] = p0[e0] p1[e1] for e0 + e1 <= DD (pair(e0, e1) = s(s+1)/2 + e1, s = e0 + e1)
template <int DD, typename T>
__device__ __forceinline__ void fill_pairs(const T* p0, const T* p1, T* out) {
#pragma unroll
  for (int s = 0; s <= DD; s++)
#pragma unroll
    for (int e1 = 0; e1 <= s; e1++) out[s * (s + 1) / 2 + e1] = p0[s - e1] * p1[e1];
}

template <int DD, int D, typename T>
__device__ __forceinline__ void point_tables(const T* lam, T w, T* a, T* b) {
  T p0[DD + 1], p1[DD + 1], p2[DD + 1];
  p0[0] = w;
  p1[0] = (T)1;
  p2[0] = (T)1;
#pragma unroll
  for (int e = 1; e <= DD; e++) {
    p0[e] = p0[e - 1] * lam[0];
    p1[e] = p1[e - 1] * lam[1];
    p2[e] = p2[e - 1] * lam[2];
  }
  fill_pairs<DD, T>(p0, p1, a);
  if constexpr (D == 3) {
    T p3[DD + 1];
    p3[0] = (T)1;
#pragma unroll
    for (int e = 1; e <= DD; e++) p3[e] = p3[e - 1] * lam[3];
    fill_pairs<DD, T>(p2, p3, b);
  } else {
#pragma unroll
    for (int e = 0; e <= DD; e++) b[e] = p2[e];
  }
}

template <int D, typename T>
__global__ void __launch_bounds__(kMomNT) k_cut_moments(MomDesc md, const CutGeoS* __restrict__ cg,
                                                         const CutSubS* __restrict__ cs,
                                                         const int* __restrict__ counts, int64_t cap,
                                                         T* __restrict__ mu) {
  constexpr int kMomEPB = mom_epb<D>(), kMomCHP = kMomPts / kMomEPB;
  extern __shared__ __align__(16) unsigned char mo_smem[];
  T* A = (T*)mo_smem;                // [kMomPts][NA]: w lambda0^e0 lambda1^e1
  T* B = A + kMomPts * md.NA;        // [kMomPts][NB]: lambda2^e2 lambda3^e3 (3D), lambda2^e2 (2D)
  __shared__ int np_s[kMomEPB];
  constexpr int NSLOT = (kMomEPB * mono_count(D + 1, kMaxMomDeg) + kMomNT - 1) / kMomNT;
  const int count = (int)min((int64_t)counts[1], cap);
  const int NA = md.NA, NB = md.NB;
  for (int batch = blockIdx.x; batch * kMomEPB < count; batch += gridDim.x) {
    const int base = batch * kMomEPB;
    for (int s = 0; s < md.nsets; s++) {
      const int dt = md.dt[s], d = md.deg[s], M = md.M[s];
      const int sd = dt == XG_IF ? D - 1 : D;
      const int nq = c_rules.cnt[sd][md.order[s]], offq = c_rules.off[sd][md.order[s]];
      __syncthreads();
      if (threadIdx.x < kMomEPB) {
        const int idx = base + threadIdx.x;
        np_s[threadIdx.x] = idx < count ? cg[idx].ns[dt] * nq : 0;
      }
      __syncthreads();
      int maxnp = 0;
#pragma unroll
      for (int k = 0; k < kMomEPB; k++) maxnp = max(maxnp, np_s[k]);
      Acc<T> acc[NSLOT];
#pragma unroll
      for (int r = 0; r < NSLOT; r++) acc[r].init();
      for (int c0 = 0; c0 < maxnp; c0 += kMomCHP) {
        if (threadIdx.x < kMomPts) {
          const int el = threadIdx.x / kMomCHP, qi = c0 + threadIdx.x % kMomCHP;
          if (qi < np_s[el]) {
            const int idx = base + el;
            const int sidx = qi / nq, bq = qi - sidx * nq;
            const Sub& sub = cs[idx].sub[dt][sidx];
            T lam[4], w;
            if constexpr (sizeof(T) == 4) {
              const float* ip = c_rules_f.x[offq + bq];
              float ow = 1.f, pt[3];
              for (int m = 0; m < sd; ++m) ow -= ip[m];
#pragma unroll
              for (int k = 0; k < 3; k++) pt[k] = ow * (float)sub.p[0].c[k];
              for (int m = 0; m < sd; ++m)
#pragma unroll
                for (int k = 0; k < 3; k++) pt[k] += ip[m] * (float)sub.p[m + 1].c[k];
              w = c_rules_f.w[offq + bq] * (float)cs[idx].vol[dt][sidx];
              if (dt == XG_IF) w *= (float)cg[idx].iffac;
              w *= (float)cg[idx].meas;
              float s3 = 0.f;
#pragma unroll
              for (int k = 0; k < D; k++) {
                lam[k] = pt[k];
                s3 += pt[k];
              }
              lam[D] = 1.f - s3;
            } else {
              double pt[3];
              plain_point(sub, sd + 1, c_rules.x[offq + bq], pt);
              w = c_rules.w[offq + bq] * cs[idx].vol[dt][sidx];
              if (dt == XG_IF) w *= cg[idx].iffac;
              w *= cg[idx].meas;
              double s3 = 0.0;
#pragma unroll
              for (int k = 0; k < D; k++) {
                lam[k] = pt[k];
                s3 += pt[k];
              }
              lam[D] = 1.0 - s3;
            }
            T* a = A + threadIdx.x * NA;
            T* b = B + threadIdx.x * NB;
            switch (d) {
              case 0: point_tables<0, D, T>(lam, w, a, b); break;
              case 1: point_tables<1, D, T>(lam, w, a, b); break;
              case 2: point_tables<2, D, T>(lam, w, a, b); break;
              case 3: point_tables<3, D, T>(lam, w, a, b); break;
              case 4: point_tables<4, D, T>(lam, w, a, b); break;
              case 5: point_tables<5, D, T>(lam, w, a, b); break;
              default: point_tables<6, D, T>(lam, w, a, b); break;
            }
          }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < NSLOT; r++) {
          const int t = threadIdx.x + r * kMomNT;
          if (t < kMomEPB * M) {
            const int el = t / M, m = t - el * M;
            const int n = min(kMomCHP, np_s[el] - c0);
            const int ab = c_mono[D - 2][m];
            const T* a = A + el * kMomCHP * NA + (ab & 255);
            const T* b = B + el * kMomCHP * NB + (ab >> 8);
            for (int j = 0; j < n; j++) acc[r].add(a[j * NA] * b[j * NB]);
          }
        }
        __syncthreads();
      }
#pragma unroll
      for (int r = 0; r < NSLOT; r++) {
        const int t = threadIdx.x + r * kMomNT;
        if (t < kMomEPB * M) {
          const int el = t / M, m = t - el * M;
          if (base + el < count) mu[(int64_t)(base + el) * md.MT + md.off[s] + m] = acc[r].get();
        }
      }
    }
  }
}

// per cut element: Gram matrix of the barycentric gradients, the weights of
// the first-derivative tables and the group coefficients
template <int D, typename T>
struct EntGeoS {
  T G[(D + 1) * (D + 2) / 2];
  T wpd[kMaxGroups][D + 1];  // phi_p d_b phi_q: cN1 nu_b + cC beta_b
  T wdp[kMaxGroups][D + 1];  // d_b phi_p phi_q: cN2 nu_b
  T cM[kMaxGroups], cL[kMaxGroups];
  int act;  // groups whose defined_on holds the element
  int idx, slot, elem;
  int gv[D + 1];
};

template <typename T>
__device__ __forceinline__ T tab_sum(const int32_t* __restrict__ ptr, const int32_t* __restrict__ ix,
                                     const T* __restrict__ cf, int k, const T* __restrict__ m) {
  T s = 0;
  const int t1 = __ldg(&ptr[k + 1]);
  for (int t = __ldg(&ptr[k]); t < t1; t++) s += __ldg(&cf[t]) * m[__ldg(&ix[t]) & 0xffff];
  return s;
}
template <typename T>
__device__ __forceinline__ T tab_sum_w(const int32_t* __restrict__ ptr, const int32_t* __restrict__ ix,
                                       const T* __restrict__ cf, int k, const T* __restrict__ m, const T* w) {
  T s = 0;
  const int t1 = __ldg(&ptr[k + 1]);
  for (int t = __ldg(&ptr[k]); t < t1; t++) {
    const int x = __ldg(&ix[t]);
    s += (__ldg(&cf[t]) * w[x >> 16]) * m[x & 0xffff];
  }
  return s;
}

template <int D, int K, bool SYM, typename T>
__global__ void __launch_bounds__(kEntNT) k_cut_entries(FormDesc form, MomDesc md, EntTabs tabs,
                                                         const CutGeoS* __restrict__ cg,
                                                         const int* __restrict__ counts, int64_t cap,
                                                         const T* __restrict__ mu, T* __restrict__ elmat, int* err,
                                                         const int32_t* __restrict__ rowslot) {
  constexpr int N = ndof_el(D, K), E = SYM ? tri_size(N) : N * N;
  __shared__ EntGeoS<D, T> eg[kEntEPB];
  __shared__ unsigned char ep[E], eq[E];
  entry_tables(N, SYM, ep, eq);
  const int count = (int)min((int64_t)counts[1], cap);
  const T* cf[4];
#pragma unroll
  for (int k = 0; k < 4; k++) cf[k] = (const T*)tabs.coef[k];
  for (int batch = blockIdx.x; batch * kEntEPB < count; batch += gridDim.x) {
    __syncthreads();
    if (threadIdx.x < kEntEPB) {
      EntGeoS<D, T>& S = eg[threadIdx.x];
      const int idx = batch * kEntEPB + threadIdx.x;
      S.idx = idx < count ? idx : -1;
      if (idx < count) {
        const CutGeoS& C = cg[idx];
        double g[D + 1][D], nu[D + 1];
#pragma unroll
        for (int a = 0; a <= D; a++) {
          double s = 0.0;
#pragma unroll
          for (int k = 0; k < D; k++) {
            g[a][k] = C.g[a][k];
            s += C.nrm[k] * g[a][k];
          }
          nu[a] = s;
        }
#pragma unroll
        for (int a = 0; a <= D; a++)
#pragma unroll
          for (int b = a; b <= D; b++) {
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < D; k++) s += g[a][k] * g[b][k];
            S.G[tri_index(a, b, D + 1)] = (T)s;
          }
        int act = 0;
        for (int q = 0; q < form.ngroups; q++) {
          const GroupDesc& Gq = form.g[q];
          if (!Gq.defined_on || tbit(Gq.defined_on, C.elem)) act |= 1 << q;
          const int used = Gq.used;
          S.cM[q] = (T)C.coef[q][0];
          S.cL[q] = (T)C.coef[q][1];
#pragma unroll
          for (int b = 0; b <= D; b++) {
            double pd = 0.0, dp = 0.0;
            if (used & (1 << XG_TERM_NGRADU_V)) pd = C.coef[q][2] * nu[b];
            if (used & (1 << XG_TERM_CONV)) {
              double s = 0.0;
#pragma unroll
              for (int k = 0; k < D; k++) s += Gq.b[k] * g[b][k];
              pd += C.coef[q][4] * s;
            }
            if (used & (1 << XG_TERM_U_NGRADV)) dp = C.coef[q][3] * nu[b];
            S.wpd[q][b] = (T)pd;
            S.wdp[q][b] = (T)dp;
          }
        }
        S.act = act;
        S.slot = C.slot;
        S.elem = C.elem;
#pragma unroll
        for (int v = 0; v <= D; v++) S.gv[v] = C.gv[v];
      }
    }
    __syncthreads();
    // element fastest: the lanes of a warp share the entry and its term lists
    for (int t = threadIdx.x; t < kEntEPB * E; t += kEntNT) {
      const int k = t / kEntEPB, el = t - k * kEntEPB;
      const EntGeoS<D, T>& S = eg[el];
      if (S.idx < 0) continue;
      const T* mue = mu + (int64_t)S.idx * md.MT;
      Acc<T> v;
      v.init();
      for (int q = 0; q < form.ngroups; q++) {
        if (!((S.act >> q) & 1)) continue;
        const int used = form.g[q].used;
        const T* m = mue + md.off[md.set_of[q]];
        if (used & (1 << XG_TERM_MASS)) v.add(S.cM[q] * tab_sum<T>(tabs.ptr[0], tabs.idx[0], cf[0], k, m));
        if (used & (1 << XG_TERM_LAPLACE))
          v.add(S.cL[q] * tab_sum_w<T>(tabs.ptr[1], tabs.idx[1], cf[1], k, m, S.G));
        if (used & ((1 << XG_TERM_NGRADU_V) | (1 << XG_TERM_CONV)))
          v.add(tab_sum_w<T>(tabs.ptr[2], tabs.idx[2], cf[2], k, m, S.wpd[q]));
        if (used & (1 << XG_TERM_U_NGRADV)) v.add(tab_sum_w<T>(tabs.ptr[3], tabs.idx[3], cf[3], k, m, S.wdp[q]));
      }
      T r = v.get();
      if (K == 3) r = neg_if(r, fn_sign<D, K>(ep[k], S.gv) != fn_sign<D, K>(eq[k], S.gv));
      if (!finite_bits(r)) set_err(err, XG_ERR_NONFINITE);
      store_out<T>(elmat, rowslot, S.elem, S.slot, N, ep[k], eq[k], r, SYM);
    }
  }
}

// ---- host side of the moment kernels (tables: xg_moments.cuh) --------------
int upload_mono() {
  uint16_t h[2][210] = {};
  for (int D = 2; D <= 3; D++) {
    const std::vector<Expo> ms = monomials(D + 1);
    for (size_t m = 0; m < ms.size(); m++) {
      const Expo& e = ms[m];
      const int ia = pair_index(e[0], e[1]), ib = D == 3 ? pair_index(e[2], e[3]) : e[2];
      h[D - 2][m] = (uint16_t)(ia | ib << 8);
    }
  }
  XG_CUDA(cudaMemcpyToSymbol(c_mono, h, sizeof(h)));
  return XG_OK;
}


// ============================================================================
// Facet-patch matrices (ghost penalty): patch rule = the volume rule of order
// 2*maxorder on each element mapped into the neighbour; contraction over the
// packed upper triangle of the (2N)^2 symmetric patch matrix.
// ============================================================================
template <int D, int K>
struct PaCfg {
  static constexpr int N = ndof_el(D, K);
  static constexpr int N2 = 2 * N;
  static constexpr int E = tri_size(N2);
  static constexpr int FPB = N2 <= 8 ? 16 : (N2 <= 20 ? 8 : 4);
  static constexpr int CH = 8;
  static constexpr int NT = N2 * FPB;
  static constexpr int NACC = (FPB * E + NT - 1) / NT;
};

// per-facet patch geometry in the kernel's precision (computed in FP64)
template <int D, typename T>
struct PaGeoS {
  T A12[D][D], c12[D];  // xi_2 = A12 xi_1 + c12 (element 1 -> element 2 reference coordinates)
  T A21[D][D], c21[D];
  T L21[D + 1][D + 1];  // lambda_2 = L21 lambda_1 (barycentric coordinates)
  T L12[D + 1][D + 1];  // lambda_1 = L12 lambda_2
  T det1, det2;
  int gv1[4], gv2[4];
  int facet;
  T coef[kMaxPatch];
};

template <typename T>
__device__ __forceinline__ T rule_x(int r, int k);
template <>
__device__ __forceinline__ double rule_x<double>(int r, int k) {
  return c_rules.x[r][k];
}
template <>
__device__ __forceinline__ float rule_x<float>(int r, int k) {
  return c_rules_f.x[r][k];
}
template <typename T>
__device__ __forceinline__ T rule_w(int r);
template <>
__device__ __forceinline__ double rule_w<double>(int r) {
  return c_rules.w[r];
}
template <>
__device__ __forceinline__ float rule_w<float>(int r) {
  return c_rules_f.w[r];
}

// Reference-coordinate map between the two elements of a patch.  For affine
// elements the low-order guess of MapPatchIntegrationPoint
// (symboliccutbfi.cpp:1747-1846) is the exact map and its Newton loop only
// adds a correction of rounding size, so the map is precomputed once per facet.
template <int D>
__device__ __forceinline__ void patch_map(const Geo<D>& from, const Geo<D>& to, double (*A)[D], double* c) {
#pragma unroll
  for (int i = 0; i < D; i++) {
#pragma unroll
    for (int k = 0; k < D; k++) {
      double s = 0;
#pragma unroll
      for (int j = 0; j < D; j++) s += to.Finv[i][j] * from.F[j][k];
      A[i][k] = s;
    }
    double s = 0;
#pragma unroll
    for (int j = 0; j < D; j++) s += to.Finv[i][j] * (from.x0[j] - to.x0[j]);
    c[i] = s;
  }
}

// Per active facet (thread per facet): the two element maps, the measures and
// the patch coefficients, read by k_patch.
template <int D, typename T>
__global__ void k_patch_geo(int ne, int nv, const int32_t* __restrict__ elv, const double* __restrict__ xyz,
                            int64_t nf, const int32_t* __restrict__ fel, FormDesc form,
                            const int32_t* __restrict__ list, const int* __restrict__ counts,
                            PaGeoS<D, T>* __restrict__ pgeo, int64_t cap_fa, int* err) {
  const int count = counts[2];
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < count; idx += gridDim.x * blockDim.x) {
    if (idx >= cap_fa) {
      set_err(err, XG_ERR_CAPACITY);
      continue;
    }
    PaGeoS<D, double> G;
    G.facet = list[idx];
    const int e1 = fel[G.facet], e2 = fel[nf + G.facet];
    double xv[D + 1][3];
#pragma unroll
    for (int v = 0; v <= D; v++) {
      const int vid = elv[(int64_t)v * ne + e1];
      G.gv1[v] = vid;
#pragma unroll
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
    }
    Geo<D> g1, g2;
    make_geo<D>(xv, g1);
#pragma unroll
    for (int v = 0; v <= D; v++) {
      const int vid = elv[(int64_t)v * ne + e2];
      G.gv2[v] = vid;
#pragma unroll
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? xyz[(int64_t)c * nv + vid] : 0.0;
    }
    make_geo<D>(xv, g2);
    patch_map<D>(g1, g2, G.A12, G.c12);
    patch_map<D>(g2, g1, G.A21, G.c21);
    G.det1 = fabs(g1.det);
    G.det2 = fabs(g2.det);
    double h = -1.0;
    for (int pp = 0; pp < kMaxPatch; pp++) G.coef[pp] = 0.0;
    for (int pp = 0; pp < form.npatch; pp++) {
      const PatchDesc& P = form.p[pp];
      const bool on = !P.defined_on || tbit(P.defined_on, G.facet);
      if (P.hpow != 0 && h < 0) h = mesh_h<D>(G.det1);
      G.coef[pp] = !on ? 0.0 : (P.hpow == 0 ? P.c : P.c * int_pow(h, P.hpow));
    }
    PaGeoS<D, T> O;
#pragma unroll
    for (int i = 0; i < D; i++) {
      O.c12[i] = (T)G.c12[i];
      O.c21[i] = (T)G.c21[i];
#pragma unroll
      for (int k = 0; k < D; k++) {
        O.A12[i][k] = (T)G.A12[i][k];
        O.A21[i][k] = (T)G.A21[i][k];
      }
    }
    // barycentric form of the maps: lambda_to[i] = sum_b L[i][b] lambda_from[b]
    // (xi_to = A xi_from + c with 1 = sum_b lambda_from[b])
#pragma unroll
    for (int b = 0; b <= D; b++) {
      double s12 = 0.0, s21 = 0.0;
#pragma unroll
      for (int i = 0; i < D; i++) {
        const double l21 = (b < D ? G.A12[i][b] : 0.0) + G.c12[i];
        const double l12 = (b < D ? G.A21[i][b] : 0.0) + G.c21[i];
        O.L21[i][b] = (T)l21;
        O.L12[i][b] = (T)l12;
        s12 += l21;
        s21 += l12;
      }
      O.L21[D][b] = (T)(1.0 - s12);
      O.L12[D][b] = (T)(1.0 - s21);
    }
    O.det1 = (T)G.det1;
    O.det2 = (T)G.det2;
    for (int pp = 0; pp < kMaxPatch; pp++) O.coef[pp] = (T)G.coef[pp];
    for (int v = 0; v < 4; v++) {
      O.gv1[v] = G.gv1[v];
      O.gv2[v] = G.gv2[v];
    }
    O.facet = G.facet;
    pgeo[idx] = O;
  }
}

template <int D, int K, typename T>
__global__ void __launch_bounds__(PaCfg<D, K>::NT) k_patch(
    FormDesc form, const PaGeoS<D, T>* __restrict__ pgeo, const int* __restrict__ counts,
    T* __restrict__ famat, int64_t cap_fa, int* err, int full_rows) {
  using C = PaCfg<D, K>;
  constexpr int N = C::N, N2 = C::N2, E = C::E, FPB = C::FPB, CH = C::CH, NT = C::NT, NACC = C::NACC;
  __shared__ PaGeoS<D, T> geo[FPB];
  __shared__ T pts[FPB][CH][2 * D + 3];  // barycentrics in element 1 and 2, weight
  __shared__ T S[FPB][CH][N2];   // s_a = phi1_a / -phi2_(a-N)
  __shared__ T SW[FPB][CH][N2];  // weighted
  __shared__ unsigned char ep[E], eq[E];
  entry_tables(N2, true, ep, eq);
  const int count = counts[2];
  const int lf = threadIdx.x / N2, a = threadIdx.x % N2;

  for (int batch = blockIdx.x; batch * FPB < count; batch += gridDim.x) {
    __syncthreads();
    if (threadIdx.x < FPB) {
      const int idx = batch * FPB + threadIdx.x;
      if (idx < count && idx < cap_fa) geo[threadIdx.x] = pgeo[idx];
      else geo[threadIdx.x].facet = -1;
    }
    __syncthreads();
    const PaGeoS<D, T>& G = geo[lf];
    const bool mine1 = a < N;
    const int desc = G.facet >= 0 ? fn_desc<D, K>(mine1 ? a : a - N, mine1 ? G.gv1 : G.gv2) : 0;
    Acc<T> acc[NACC];
#pragma unroll
    for (int m = 0; m < NACC; m++) acc[m].init();

    for (int pp = 0; pp < form.npatch; pp++) {
      const PatchDesc& P = form.p[pp];
      const int p = clamp_order(P.order);
      const int nq = c_rules.cnt[D][p], off = c_rules.off[D][p];
      for (int q0 = 0; q0 < 2 * nq; q0 += CH) {
        for (int qq = a; qq < CH; qq += N2) {
          const int qi = q0 + qq;
          T x1[3] = {(T)0.25, (T)0.25, (T)0.25}, x2[3] = {(T)0.25, (T)0.25, (T)0.25}, W = 0;
          if (qi < 2 * nq && G.facet >= 0) {
            const bool one = qi < nq;
            const int r = off + (one ? qi : qi - nq);
            T* xa = one ? x1 : x2;
            T* xb = one ? x2 : x1;
#pragma unroll
            for (int k = 0; k < D; k++) xa[k] = rule_x<T>(r, k);
#pragma unroll
            for (int i2 = 0; i2 < D; i2++) {
              T sacc = one ? G.c12[i2] : G.c21[i2];
#pragma unroll
              for (int k = 0; k < D; k++) sacc += (one ? G.A12[i2][k] : G.A21[i2][k]) * xa[k];
              xb[i2] = sacc;
            }
            W = rule_w<T>(r) * (one ? G.det1 : G.det2);
          }
          T s1 = 0, s2 = 0;
#pragma unroll
          for (int k = 0; k < D; k++) {
            pts[lf][qq][k] = x1[k];
            pts[lf][qq][D + 1 + k] = x2[k];
            s1 += x1[k];
            s2 += x2[k];
          }
          pts[lf][qq][D] = (T)1 - s1;
          pts[lf][qq][2 * D + 1] = (T)1 - s2;
          pts[lf][qq][2 * D + 2] = W * G.coef[pp];
        }
        __syncthreads();
#pragma unroll
        for (int qq = 0; qq < CH; qq++) {
          const T v = eval_fn_value<D, T>(desc, &pts[lf][qq][mine1 ? 0 : D + 1]);
          const T sv = mine1 ? v : -v;
          S[lf][qq][a] = sv;
          SW[lf][qq][a] = pts[lf][qq][2 * D + 2] * sv;
        }
        __syncthreads();
        const int nch = min(CH, 2 * nq - q0);
#pragma unroll
        for (int m = 0; m < NACC; m++) {
          const int t = threadIdx.x + m * NT;
          if (t < FPB * E) {
            const int fl = t / E, k = t % E, pa = ep[k], pb = eq[k];
            T v = 0;
            for (int qq = 0; qq < nch; qq++) v += SW[fl][qq][pa] * S[fl][qq][pb];
            acc[m].add(v);
          }
        }
        __syncthreads();
      }
    }
#pragma unroll
    for (int m = 0; m < NACC; m++) {
      const int t = threadIdx.x + m * NT;
      if (t < FPB * E) {
        const int fl = t / E, k = t % E;
        const int idx = batch * FPB + fl;
        if (geo[fl].facet >= 0) {
          if (idx >= cap_fa) {
            if (k == 0) set_err(err, XG_ERR_CAPACITY);
          } else {
            const T v = acc[m].get();
            if (!isfinite(v)) set_err(err, XG_ERR_NONFINITE);
            store_out<T>(famat, nullptr, idx, idx, N2, ep[k], eq[k], v, true, full_rows != 0);
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Facet patches by basis change (every patch term of order >= 2K).  The
// integrand (u1 - u2)(v1 - v2) has degree 2K on each element and the order-2K
// rule integrates it exactly, so with x = [x1; x2] the coefficients of both
// elements' functions:
//   on T1:  (S1 x1 - C21 x2)^T  |det F1| Mh  (S1 x1 - C21 x2)
//   on T2:  (C12 x1 - S2 x2)^T  |det F2| Mh  (C12 x1 - S2 x2)
// Mh = reference mass matrix of the canonical basis, S = the elements' edge
// orientation signs, C21 = the functions of T2 in the canonical basis of T1
// (exact, from their values at T1's nodes) and C12 likewise.  With
// W = Mh C the blocks of the patch matrix are
//   (1,1)  det1 S1 Mh S1 + det2 C12^T W12
//   (1,2)  -det1 S1 W21 - det2 (S2 W12)^T
//   (2,2)  det1 C21^T W21 + det2 S2 Mh S2
// the same integrals as the quadrature of k_patch, reassociated.
// ---------------------------------------------------------------------------
template <int D, int K>
struct PxCfg {
  static constexpr int N = ndof_el(D, K);
  static constexpr int E = tri_size(2 * N);
  static constexpr int FPB = N <= 10 ? 32 : 8;  // facets per block: the lanes of one unit of work
  static constexpr int NT = 256;
  static constexpr int NU = NT / FPB;           // units per pass of the block
};

// shared memory of k_patch_exact, facet index fastest (lanes = facets, so a
// warp runs one unit of work -- a node, a column, an entry -- for FPB facets
// without divergence: partially active warps would idle FP64 lanes)
template <int D, int K, typename T>
struct PxSmem {
  static constexpr int N = PxCfg<D, K>::N, E = PxCfg<D, K>::E, F = PxCfg<D, K>::FPB;
  T Ct[2][N][N][F];  // [0]: C21 (T2's functions in T1's canonical basis), [1]: C12
  // W = Mh C, written once C is complete, shares its storage with the maps and
  // node images, which are needed only to build C (two blocks fit an SM)
  union {
    T Wt[2][N][N][F];
    struct {
      T nodes[2][N][D + 1][F];
      T L[2][D + 1][D + 1][F];  // [0]: L21, [1]: L12
    } pre;
  };
  T det1[F], det2[F], c[F];
  int gv1[D + 1][F], gv2[D + 1][F];
  int idx[F];
  T Mh[N][N];
  int cnt[4];
  unsigned char perm[N];
  unsigned char ep[E], eq[E];
};

// One form's share of the basis-change patch work.
template <int D, typename T>
struct PxJob {
  const PaGeoS<D, T>* pgeo;
  const int* counts;  // [2] active facets
  const T* mhat;      // reference mass matrix of the element's order
  T* famat;
  int64_t cap_fa;
  int* err;
  int full_rows;
  int npatch;
  int K;
};

// per-block tables of the order: entry order, Mh, rows by canonical degree
template <int D, int K, typename T>
__device__ void px_init(PxSmem<D, K, T>& sm, const T* __restrict__ mhat) {
  using C = PxCfg<D, K>;
  constexpr int N = C::N, NT = C::NT;
  entry_tables(2 * N, true, sm.ep, sm.eq);
  for (int t = threadIdx.x; t < N * N; t += NT) sm.Mh[t / N][t % N] = mhat[t];
  if (threadIdx.x == 0) {
    int n = 0;
    sm.cnt[0] = 0;
    for (int d = 1; d <= 3; d++) {
      for (int k = 0; k < N; k++)
        if (canon_degree<D, K>(k) == d) sm.perm[n++] = (unsigned char)k;
      sm.cnt[d] = n;
    }
  }
}

// the patch matrices of F facets (batch `batch` of the job's active facets);
// the block's tables must hold the job's order (px_init)
template <int D, int K, typename T>
__device__ void px_batch(const PxJob<D, T>& J, int batch, PxSmem<D, K, T>& sm) {
  using C = PxCfg<D, K>;
  constexpr int N = C::N, E = C::E, F = C::FPB, NU = C::NU;
  const int f = threadIdx.x % F, u0 = threadIdx.x / F;
  const int count = J.counts[2];
  const int64_t cap_fa = J.cap_fa;
  const PaGeoS<D, T>* __restrict__ pgeo = J.pgeo;
  __syncthreads();
  if (threadIdx.x < F) {
    const int idx = batch * F + threadIdx.x;
    const bool ok = idx < count && idx < cap_fa;
    sm.idx[threadIdx.x] = ok ? idx : -1;
    if (ok) {
      const PaGeoS<D, T>& G = pgeo[idx];
#pragma unroll
      for (int i = 0; i <= D; i++)
#pragma unroll
        for (int b = 0; b <= D; b++) {
          sm.pre.L[0][i][b][threadIdx.x] = G.L21[i][b];
          sm.pre.L[1][i][b][threadIdx.x] = G.L12[i][b];
        }
      sm.det1[threadIdx.x] = G.det1;
      sm.det2[threadIdx.x] = G.det2;
      T c = 0;
      for (int pp = 0; pp < J.npatch; pp++) c += G.coef[pp];
      sm.c[threadIdx.x] = c;
#pragma unroll
      for (int v = 0; v <= D; v++) {
        sm.gv1[v][threadIdx.x] = G.gv1[v];
        sm.gv2[v][threadIdx.x] = G.gv2[v];
      }
    }
  }
  __syncthreads();
  const bool live = sm.idx[f] >= 0;
  // images of the canonical nodes under the barycentric maps
  for (int u = u0; u < 2 * N; u += NU) {
    const int sd = u / N, n = u % N;
    if (!live) continue;
    T out[D + 1];
    node_image<D, K, T>(n, &sm.pre.L[sd][0][0][f], (D + 1) * F, F, out);
#pragma unroll
    for (int i = 0; i <= D; i++) sm.pre.nodes[sd][n][i][f] = out[i];
  }
  __syncthreads();
  // column j of C: function j of the other element in this element's canonical basis
  for (int u = u0; u < 2 * N; u += NU) {
    const int sd = u / N, j = u % N;
    if (!live) continue;
    int gv[4] = {0, 0, 0, 0};
#pragma unroll
    for (int v = 0; v <= D; v++) gv[v] = sd == 0 ? sm.gv2[v][f] : sm.gv1[v][f];
    const int desc = fn_desc<D, K>(j, gv);
    T p[N];
#pragma unroll
    for (int n = 0; n < N; n++) {
      T lam[D + 1];
#pragma unroll
      for (int i = 0; i <= D; i++) lam[i] = sm.pre.nodes[sd][n][i][f];
      p[n] = eval_fn_value<D, T>(desc, lam);
    }
    nodal_to_hier<D, K, T>(p, fn_degree(desc), &sm.Ct[sd][0][j][f], N * F);
  }
  __syncthreads();
  // W = Mh C over the rows of degree <= the column's degree (the others are 0)
  for (int u = u0; u < 2 * N * N; u += NU) {
    const int r = u % N, j = (u / N) % N, sd = u / (N * N);
    if (!live) continue;
    const int nk = sm.cnt[canon_degree<D, K>(j)];
    T s = 0;
    for (int i = 0; i < nk; i++) {
      const int k = sm.perm[i];
      s += sm.Mh[r][k] * sm.Ct[sd][k][j][f];
    }
    sm.Wt[sd][r][j][f] = s;
  }
  __syncthreads();
  if (!live) return;
  const int idx = sm.idx[f];
  const T det1 = sm.det1[f], det2 = sm.det2[f], c = sm.c[f];
  for (int k = u0; k < E; k += NU) {
    const int a = sm.ep[k], b = sm.eq[k];
    Acc<T> v;
    v.init();
    if (b < N) {  // (1,1)
      int g1[4] = {0, 0, 0, 0};
#pragma unroll
      for (int q = 0; q <= D; q++) g1[q] = sm.gv1[q][f];
      const bool flip = K == 3 && fn_sign<D, K>(a, g1) != fn_sign<D, K>(b, g1);
      v.add(det1 * neg_if(sm.Mh[a][b], flip));
      const int nk = sm.cnt[canon_degree<D, K>(a)];
      T s = 0;
      for (int i = 0; i < nk; i++) {
        const int kk = sm.perm[i];
        s += sm.Ct[1][kk][a][f] * sm.Wt[1][kk][b][f];
      }
      v.add(det2 * s);
    } else if (a < N) {  // (1,2)
      const int bb = b - N;
      int g1[4] = {0, 0, 0, 0}, g2[4] = {0, 0, 0, 0};
#pragma unroll
      for (int q = 0; q <= D; q++) {
        g1[q] = sm.gv1[q][f];
        g2[q] = sm.gv2[q][f];
      }
      const T w1 = neg_if(sm.Wt[0][a][bb][f], K == 3 && fn_sign<D, K>(a, g1) < 0);
      const T w2 = neg_if(sm.Wt[1][bb][a][f], K == 3 && fn_sign<D, K>(bb, g2) < 0);
      v.add(neg_if(det1 * w1, true));
      v.add(neg_if(det2 * w2, true));
    } else {  // (2,2)
      const int aa = a - N, bb = b - N;
      const int nk = sm.cnt[canon_degree<D, K>(aa)];
      T s = 0;
      for (int i = 0; i < nk; i++) {
        const int kk = sm.perm[i];
        s += sm.Ct[0][kk][aa][f] * sm.Wt[0][kk][bb][f];
      }
      v.add(det1 * s);
      int g2[4] = {0, 0, 0, 0};
#pragma unroll
      for (int q = 0; q <= D; q++) g2[q] = sm.gv2[q][f];
      const bool flip = K == 3 && fn_sign<D, K>(aa, g2) != fn_sign<D, K>(bb, g2);
      v.add(det2 * neg_if(sm.Mh[aa][bb], flip));
    }
    const T r = c * v.get();
    if (!finite_bits(r)) set_err(J.err, XG_ERR_NONFINITE);
    store_out<T>(J.famat, nullptr, idx, idx, 2 * N, a, b, r, true, J.full_rows != 0);
  }
}

template <int D, int K, typename T>
__global__ void __launch_bounds__(256) k_patch_exact(PxJob<D, T> J) {
  using S = PxSmem<D, K, T>;
  extern __shared__ __align__(16) unsigned char px_raw[];
  S& sm = *reinterpret_cast<S*>(px_raw);
  px_init<D, K, T>(sm, J.mhat);
  constexpr int F = PxCfg<D, K>::FPB;
  for (int batch = blockIdx.x; batch * F < J.counts[2]; batch += gridDim.x) px_batch<D, K, T>(J, batch, sm);
}

// Several forms' patch matrices in one persistent launch (batched steps of
// several forms): the work items are (form, batch of facets), enumerated in
// the jobs' order -- the host sorts the jobs by decreasing cost per item, so
// the queue is cost-sorted and the most expensive items start first -- and
// every block takes its next item from a global counter (work stealing), so
// blocks that drew cheap items take more of them.  Each item is the same
// px_batch work as k_patch_exact: the results are bit-identical.
constexpr int kMaxPxJobs = 16;
template <int D, typename T>
struct PxJobs {
  PxJob<D, T> job[kMaxPxJobs];
  int n;
  int* queue;  // item counter, zero at launch
};

template <int D, typename T>
__global__ void __launch_bounds__(256) k_patch_exact_multi(const __grid_constant__ PxJobs<D, T> Q) {
  extern __shared__ __align__(16) unsigned char px_raw[];
  __shared__ long long first[kMaxPxJobs + 1];
  __shared__ int item_s;
  if (threadIdx.x == 0) {
    long long acc = 0;
    for (int j = 0; j < Q.n; j++) {
      first[j] = acc;
      const int K = Q.job[j].K;
      const int F = K == 1 ? PxCfg<D, 1>::FPB : (K == 2 ? PxCfg<D, 2>::FPB : PxCfg<D, 3>::FPB);
      const long long cnt = min((long long)Q.job[j].counts[2], (long long)Q.job[j].cap_fa);
      acc += (cnt + F - 1) / F;
    }
    first[Q.n] = acc;
  }
  __syncthreads();
  const long long total = first[Q.n];
  int cur = -1;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) item_s = atomicAdd(Q.queue, 1);
    __syncthreads();
    const long long item = item_s;
    if (item >= total) break;
    int j = 0;
    while (item >= first[j + 1]) j++;
    const int batch = (int)(item - first[j]);
    const PxJob<D, T>& J = Q.job[j];
    if (J.K == 1) {
      auto& sm = *reinterpret_cast<PxSmem<D, 1, T>*>(px_raw);
      if (cur != j) px_init<D, 1, T>(sm, J.mhat);
      px_batch<D, 1, T>(J, batch, sm);
    } else if (J.K == 2) {
      auto& sm = *reinterpret_cast<PxSmem<D, 2, T>*>(px_raw);
      if (cur != j) px_init<D, 2, T>(sm, J.mhat);
      px_batch<D, 2, T>(J, batch, sm);
    } else {
      auto& sm = *reinterpret_cast<PxSmem<D, 3, T>*>(px_raw);
      if (cur != j) px_init<D, 3, T>(sm, J.mhat);
      px_batch<D, 3, T>(J, batch, sm);
    }
    cur = j;
  }
}

// ============================================================================
// Scatter.  The columns of the row of dof r are the dofs of the active
// elements containing r and, for every active facet of an element containing
// r, the dofs of both elements of that facet patch.  At form creation the full
// pattern (every element and interior facet active) is built once: sorted
// columns of every dof row (hash + sort, k_row_count) and the position of
// every element column in its rows' full rows (k_fpos_el).  Per step, pass 1
// flags the active columns over the full-row positions, element- and
// facet-centric (k_row_clear, k_flag_elements, k_flag_facets), and counts
// them per row (k_row_flagcount); pass 2 (k_row_sum, one warp per active row)
// stages (position, value) pairs and adds them in the fixed order (adjacent
// elements ascending; per element its own matrix row, then its facets in local
// order, first then second element's columns) -- the sum order never depends
// on scheduling, no atomics -- and writes the flagged positions compressed.
// ============================================================================
struct ScatterArgs {
  int ne, nd, nfl;
  const int32_t* el_dofs;    // [ne][nd]
  const int32_t* el_facets;  // [ne][nfl]
  const int2* fel;           // [nf] first / second element
  const int32_t* adj_ptr;
  const int32_t* adj;
  const uint32_t* act_un;
  const uint32_t* act_cut;
  const uint32_t* act_fa;
  const int32_t* el_slot;    // valid for active elements
  const int32_t* fa_slot;    // valid for active facets
  const int32_t* rows;       // active dofs (row -> dof)
  const int32_t* dof_row;    // dof -> row (valid for active dofs)
  const int* counts;         // [3] = nrows
  int64_t cap_fa;
  const int64_t* full_ptr;   // per dof: offset of its row in tmp_cols (full-pattern row sizes)
  int32_t* tmp_cols;         // full-pattern columns of every dof row, sorted (written once at creation)
  const uint16_t* fpos_el;   // [ne][nd][nd] positions of element columns in the full rows
  uint16_t* pbuf;            // [cap_fa][2][nd][nd] positions of neighbour columns of active facets
  uint8_t* flags;            // [full_nnz] active columns of the active rows
  int el_sym;                // element matrices stored as packed upper triangles
  int nds, kt1;              // spatial dofs per element, time dofs (1 for spatial forms)
  double mt[9];              // time mass kt1 x kt1: patch value = mt[it][is] * spatial patch value
  int hs;                    // hash slots per warp (pow2, or 0)
  int maxu;                  // distinct-column capacity per warp (pow2)
  int ucn, accn;             // shared column ints / accumulator doubles per warp (0 or maxu)
  int stage;                 // staged (pos, value) pairs per warp
  int wbytes;                // shared bytes per warp
};

constexpr int kRowWarps = 8;
constexpr int kEnt = 32;  // adjacency entries per chunk

struct RowSm {
  int* hash;
  int* ucols;
  double* acc;
  double* sval;
  int* spos;
  int* ent_e;
  int* ent_i;
  int* ent_nb;     // [kEnt][4] other element of an active facet, -1 if inactive
  int* ent_fs;     // [kEnt][4] facet slot
  int* ent_first;  // [kEnt][4] 1 if the row's element is the facet's first element
  int* celem;      // [kEnt * 5]
  int* grp;        // [kEnt * 9] (entry << 4) | kind
  int* ent_slot;   // [kEnt] element-matrix slot of an active element
};

__host__ __device__ inline int row_smem_bytes(int hs, int ucn, int accn, int stage) {
  return hs * 4 + ucn * 4 + accn * 8 + stage * 8 + stage * 4 + kEnt * 4 * 2 + kEnt * 4 * 4 * 3 + kEnt * 5 * 4 +
         kEnt * 9 * 4 + kEnt * 4 + 16;
}

__device__ __forceinline__ RowSm row_sm(const ScatterArgs& A, unsigned char* base) {
  RowSm S;
  S.hash = (int*)base;
  S.ucols = S.hash + A.hs;
  S.acc = (double*)(S.ucols + A.ucn);  // hs, ucn are 0 or powers of two >= 32: 8-byte aligned
  S.sval = S.acc + A.accn;
  S.spos = (int*)(S.sval + A.stage);
  S.ent_e = S.spos + A.stage;
  S.ent_i = S.ent_e + kEnt;
  S.ent_nb = S.ent_i + kEnt;
  S.ent_fs = S.ent_nb + kEnt * 4;
  S.ent_first = S.ent_fs + kEnt * 4;
  S.celem = S.ent_first + kEnt * 4;
  S.grp = S.celem + kEnt * 5;
  S.ent_slot = S.grp + kEnt * 9;
  return S;
}

// (t / nd, t % nd) for t = lane, lane + 32, ... without an integer division per step
struct LaneIdx {
  int g, j, dg, dj, nd;
  __device__ __forceinline__ void init(int t, int nd_) {
    nd = nd_;
    g = t / nd;
    j = t - g * nd;
    dg = 32 / nd;
    dj = 32 - dg * nd;
  }
  __device__ __forceinline__ void next() {
    g += dg;
    j += dj;
    if (j >= nd) {
      j -= nd;
      g++;
    }
  }
};

__device__ __forceinline__ bool el_active(const ScatterArgs& A, int e) {
  return tbit32(A.act_un, e) || tbit32(A.act_cut, e);
}

// Loads adjacency entries [c0, c0+na) of the row into shared memory; returns the
// number of candidate elements written to S.celem.
__device__ int load_entries(const ScatterArgs& A, const RowSm& S, int c0, int na) {
  const int lane = threadIdx.x & 31;
  int ncand = 0;
  if (lane < na) {
    // three levels of independent loads (element; its facets; the active
    // facets' neighbours and slots) instead of one dependent chain per facet
    const int v = A.adj[c0 + lane];
    const int e = v >> 5, i = v & 31;
    const bool act = el_active(A, e);
    const int slot = A.el_slot[e];
    int f[4], fa[4];
#pragma unroll
    for (int lf = 0; lf < 4; lf++) f[lf] = lf < A.nfl ? A.el_facets[(int64_t)e * A.nfl + lf] : 0;
#pragma unroll
    for (int lf = 0; lf < 4; lf++) fa[lf] = lf < A.nfl && tbit32(A.act_fa, f[lf]);
    int2 pr[4];
    int fsl[4];
#pragma unroll
    for (int lf = 0; lf < 4; lf++) {
      pr[lf] = fa[lf] ? A.fel[f[lf]] : make_int2(-1, -1);
      fsl[lf] = fa[lf] ? A.fa_slot[f[lf]] : 0;
    }
    S.ent_e[lane] = act ? e : ~e;  // sign marks an inactive element
    S.ent_i[lane] = i;
    S.ent_slot[lane] = act ? slot : -1;
    int nf = 0;
#pragma unroll
    for (int lf = 0; lf < 4; lf++) {
      if (lf >= A.nfl) break;
      int nb = -1, first = 0;
      if (fa[lf]) {
        first = pr[lf].x == e;
        nb = first ? pr[lf].y : pr[lf].x;
        nf++;
      }
      S.ent_nb[lane * 4 + lf] = nb;
      S.ent_fs[lane * 4 + lf] = fa[lf] ? fsl[lf] : 0;
      S.ent_first[lane * 4 + lf] = first;
    }
    ncand = ((act || nf) ? 1 : 0) + nf;
  }
  int x = ncand;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  const int total = __shfl_sync(0xffffffffu, x, 31);
  if (lane < na && ncand) {
    int k = x - ncand;
    const int e = S.ent_e[lane] >= 0 ? S.ent_e[lane] : ~S.ent_e[lane];
    S.celem[k++] = e;
    for (int lf = 0; lf < A.nfl; lf++)
      if (S.ent_nb[lane * 4 + lf] >= 0) S.celem[k++] = S.ent_nb[lane * 4 + lf];
  }
  __syncwarp();
  return total;
}

__device__ __forceinline__ bool hash_insert(int* hash, int hs, int key) {
  unsigned h = ((unsigned)key * 2654435761u) & (unsigned)(hs - 1);
  for (int probe = 0; probe < hs; probe++) {
    int old = atomicCAS(&hash[h], 0, key + 1);
    if (old == 0 || old == key + 1) return true;
    h = (h + 1) & (unsigned)(hs - 1);
  }
  return false;  // table full: reported as a capacity error
}

// Builds the row's column set in the hash table; returns false on overflow.
__device__ bool row_columns(const ScatterArgs& A, const RowSm& S, int r) {
  const int lane = threadIdx.x & 31;
  for (int k = lane; k < A.hs; k += 32) S.hash[k] = 0;
  __syncwarp();
  const int a0 = A.adj_ptr[r], a1 = A.adj_ptr[r + 1];
  bool ok = true;
  for (int c0 = a0; c0 < a1; c0 += kEnt) {
    const int na = min(kEnt, a1 - c0);
    const int nc = load_entries(A, S, c0, na);
    // four independent dof loads in flight per lane before the inserts
    LaneIdx L;
    L.init(lane, A.nd);
    for (int t0 = lane; t0 < nc * A.nd; t0 += 128) {
      int key[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int t = t0 + 32 * q;
        key[q] = -1;
        if (t < nc * A.nd) key[q] = A.el_dofs[(int64_t)S.celem[L.g] * A.nd + L.j];
        L.next();
      }
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (key[q] >= 0) ok &= hash_insert(S.hash, A.hs, key[q]);
    }
    __syncwarp();
  }
  return __all_sync(0xffffffffu, ok);
}

// Occupied hash slots -> S.ucols (unordered); returns the count.
__device__ int hash_extract(const ScatterArgs& A, const RowSm& S, bool write) {
  const int lane = threadIdx.x & 31;
  int out = 0;
  for (int base = 0; base < A.hs; base += 32) {
    const int v = S.hash[base + lane];
    const unsigned m = __ballot_sync(0xffffffffu, v != 0);
    if (write && v != 0) {
      const int k = out + __popc(m & ((1u << lane) - 1));
      if (k < A.maxu) S.ucols[k] = v - 1;
    }
    out += __popc(m);
  }
  __syncwarp();
  return out;
}

__device__ void warp_bitonic_sort(int* buf, int n) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= n; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < n; i += 32) {
        int l = i ^ j;
        if (l > i) {
          int x = buf[i], y = buf[l];
          bool up = (i & k) == 0;
          if ((x > y) == up) {
            buf[i] = y;
            buf[l] = x;
          }
        }
      }
      __syncwarp();
    }
}

__device__ __forceinline__ int lower_bound_sm(const int* a, int n, int v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Pass 1: the row's distinct columns, sorted, into tmp_cols at the row's
// full-pattern offset, and the count.
__global__ void __launch_bounds__(kRowWarps * 32) k_row_count(ScatterArgs A, int64_t* rowcnt, int* err) {
  extern __shared__ __align__(16) unsigned char sm_rows[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const RowSm S = row_sm(A, sm_rows + (size_t)warp * A.wbytes);
  const int nrows = A.counts[3];
  for (int row = blockIdx.x * kRowWarps + warp; row < nrows; row += gridDim.x * kRowWarps) {
    const int r = A.rows[row];
    const bool ok = row_columns(A, S, r);
    int u = hash_extract(A, S, true);
    const int64_t fo = A.full_ptr[r], fcap = A.full_ptr[r + 1] - fo;
    if (!ok || u > A.maxu || u > fcap) {
      if (lane == 0) {
        set_err(err, XG_ERR_CAPACITY);
        rowcnt[row] = 0;
      }
      continue;
    }
    int m = 32;
    while (m < u) m <<= 1;
    for (int k = u + lane; k < m; k += 32) S.ucols[k] = 0x7fffffff;
    __syncwarp();
    warp_bitonic_sort(S.ucols, m);
    for (int k = lane; k < u; k += 32) A.tmp_cols[fo + k] = S.ucols[k];
    if (lane == 0) rowcnt[row] = u;
    __syncwarp();
  }
}

// Full-pattern probe (form creation): distinct columns per dof with every
// element and interior facet active; sizes the scatter buffers.
__global__ void __launch_bounds__(kRowWarps * 32) k_row_probe(ScatterArgs A, int64_t ndof, int64_t* rowcnt, int* err) {
  extern __shared__ __align__(16) unsigned char sm_rows[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const RowSm S = row_sm(A, sm_rows + (size_t)warp * A.wbytes);
  for (int64_t r = blockIdx.x * (int64_t)kRowWarps + warp; r < ndof; r += (int64_t)gridDim.x * kRowWarps) {
    const bool ok = row_columns(A, S, (int)r);
    const int u = hash_extract(A, S, false);
    if (lane == 0) {
      if (!ok) set_err(err, XG_ERR_CAPACITY);
      rowcnt[r] = u;
    }
  }
}

__global__ void k_fill_u32(uint32_t* p, int64_t n, uint32_t v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

// positions of element columns in the full-pattern rows: thread per (e, i, j)
__global__ void k_fpos_el(ScatterArgs A, uint16_t* __restrict__ fpos, int* err) {
  const int64_t nd = A.nd, n = (int64_t)A.ne * nd * nd;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / (nd * nd);
    const int i = (int)((t / nd) % nd), j = (int)(t % nd);
    const int r = A.el_dofs[e * nd + i], c = A.el_dofs[e * nd + j];
    const int64_t fo = A.full_ptr[r];
    const int len = (int)(A.full_ptr[r + 1] - fo);
    int lo = 0, hi = len;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (A.tmp_cols[fo + mid] < c) lo = mid + 1;
      else hi = mid;
    }
    if (lo >= len || A.tmp_cols[fo + lo] != c || lo > 65535) set_err(err, XG_ERR_CAPACITY);
    fpos[t] = (uint16_t)min(lo, 65535);
  }
}

// Pass 1 (per step), element- and facet-centric: the active columns of the
// active rows as byte flags over the rows' full-pattern positions.  Flag
// writes are idempotent (every writer stores 1), so no ordering is needed.
// (a) the active rows' flags are cleared (rows of earlier steps may hold
// flags); (b) every active element flags its columns in the rows of its dofs
// (static positions); (c) every active facet flags, in the rows of each
// element's dofs, the element's own columns and the other element's columns
// (found by a binary search of the sorted full row; the positions are kept
// for pass 2); (d) per row the flags are counted.
__global__ void __launch_bounds__(256) k_row_clear(ScatterArgs A) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nrows = A.counts[3];
  for (int row = warp; row < nrows; row += nwarps) {
    const int r = A.rows[row];
    const int64_t fo = A.full_ptr[r];
    const int len = (int)(A.full_ptr[r + 1] - fo);
    for (int k = lane; k < len; k += 32) A.flags[fo + k] = 0;
  }
}

__global__ void __launch_bounds__(256) k_flag_elements(ScatterArgs A, const int32_t* __restrict__ l_un,
                                                       const int32_t* __restrict__ l_cut) {
  const int nd = A.nd, nun = A.counts[0], ncut = A.counts[1];
  const int64_t total = (int64_t)(nun + ncut) * nd * nd;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t item = t / (nd * nd);
    const int ij = (int)(t - item * nd * nd), i = ij / nd;
    const int e = item < nun ? l_un[item] : l_cut[item - nun];
    const int r = A.el_dofs[(int64_t)e * nd + i];
    A.flags[A.full_ptr[r] + A.fpos_el[(int64_t)e * nd * nd + ij]] = 1;
  }
}

// thread per (active facet, side, local row i, local column j): binary search
// of the other element's dof j in the sorted full row of dof i
__global__ void __launch_bounds__(256) k_flag_facets(ScatterArgs A, const int32_t* __restrict__ l_fa, int* err) {
  const int nd = A.nd, nfa = A.counts[2];
  const int64_t total = (int64_t)nfa * 2 * nd * nd;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t fs = t / (2 * nd * nd);
    const int rem = (int)(t - fs * 2 * nd * nd), side = rem / (nd * nd), ij = rem - side * nd * nd;
    const int i = ij / nd, j = ij - i * nd;
    if (fs >= A.cap_fa) continue;  // reported by the patch kernels
    const int2 pr = A.fel[l_fa[fs]];
    const int er = side == 0 ? pr.x : pr.y, ec = side == 0 ? pr.y : pr.x;
    const int r = A.el_dofs[(int64_t)er * nd + i], c = A.el_dofs[(int64_t)ec * nd + j];
    const int64_t fo = A.full_ptr[r];
    const int len = (int)(A.full_ptr[r + 1] - fo);
    int lo = 0, hi = len;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (A.tmp_cols[fo + mid] < c) lo = mid + 1;
      else hi = mid;
    }
    if (lo >= len || A.tmp_cols[fo + lo] != c) {
      set_err(err, XG_ERR_CAPACITY);
      continue;
    }
    A.flags[fo + lo] = 1;
    A.pbuf[((fs * 2 + side) * nd + i) * nd + j] = (uint16_t)lo;
    // the row element's own columns, already flagged when it is active
    if (!el_active(A, er)) A.flags[fo + A.fpos_el[(int64_t)er * nd * nd + ij]] = 1;
  }
}

__global__ void __launch_bounds__(256) k_row_flagcount(ScatterArgs A, int64_t* __restrict__ rowcnt, int* err) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nrows = A.counts[3];
  for (int row = warp; row < nrows; row += nwarps) {
    const int r = A.rows[row];
    const int64_t fo = A.full_ptr[r];
    const int len = (int)(A.full_ptr[r + 1] - fo);
    int cnt = 0;
    for (int k = lane; k < len; k += 32) cnt += A.flags[fo + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0) {
      if (len > A.maxu) set_err(err, XG_ERR_CAPACITY);
      rowcnt[row] = cnt;
    }
  }
}

// Pass 2 (per step): values of each active row summed in a fixed order
// (adjacency order; per entry its element row, then its active facets) over
// the row's full-pattern positions, then written compressed to the active
// columns in ascending order.
template <typename T, bool SYM, bool ST, int QQ>
__global__ void __launch_bounds__(kRowWarps * 32) k_row_sum(ScatterArgs A, const T* __restrict__ elmat,
                                                             const T* __restrict__ famat,
                                                             const int64_t* __restrict__ rowptr,
                                                             int32_t* __restrict__ cols, double* __restrict__ vals,
                                                             int64_t cap_nnz, int* err) {
  extern __shared__ __align__(16) unsigned char sm_rows[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const RowSm S = row_sm(A, sm_rows + (size_t)warp * A.wbytes);
  const int nrows = A.counts[3];
  const int nd = A.nd;
  const int gpb = A.stage / nd;  // groups per staged batch
  for (int row = blockIdx.x * kRowWarps + warp; row < nrows; row += gridDim.x * kRowWarps) {
    const int r = A.rows[row];
    const int64_t rp = rowptr[row];
    const int u = (int)(rowptr[row + 1] - rp);
    const int64_t fo = A.full_ptr[r];
    const int len = (int)(A.full_ptr[r + 1] - fo);
    if (len > A.maxu || rp + u > cap_nnz) {
      if (lane == 0) set_err(err, XG_ERR_CAPACITY);
      continue;
    }
    for (int k = lane; k < len; k += 32) S.acc[k] = 0.0;
    __syncwarp();
    const int a0 = A.adj_ptr[r], a1 = A.adj_ptr[r + 1];
    for (int c0 = a0; c0 < a1; c0 += kEnt) {
      const int na = min(kEnt, a1 - c0);
      load_entries(A, S, c0, na);
      int ng = 0;
      {
        int cnt = 0;
        if (lane < na) {
          cnt = S.ent_e[lane] >= 0 ? 1 : 0;
          for (int lf = 0; lf < A.nfl; lf++) cnt += S.ent_nb[lane * 4 + lf] >= 0 ? 2 : 0;
        }
        int x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= o) x += y;
        }
        ng = __shfl_sync(0xffffffffu, x, 31);
        if (lane < na) {
          int k = x - cnt;
          if (S.ent_e[lane] >= 0) S.grp[k++] = (lane << 4) | 0;
          for (int lf = 0; lf < A.nfl; lf++)
            if (S.ent_nb[lane * 4 + lf] >= 0) {
              S.grp[k++] = (lane << 4) | (1 + 2 * lf);
              S.grp[k++] = (lane << 4) | (2 + 2 * lf);
            }
        }
        __syncwarp();
      }
      for (int g0 = 0; g0 < ng; g0 += gpb) {
        const int gb = min(gpb, ng - g0);
        LaneIdx L;
        L.init(lane, nd);
        // QQ (position, value) loads per lane in flight: 6 for rows of 10 or more
        // dofs per element, 4 below (measured; 8 is slower, registers)
        for (int t0 = lane; t0 < gb * nd; t0 += 32 * QQ) {
          double vq[QQ];
          int pq[QQ];
#pragma unroll
          for (int q = 0; q < QQ; q++) {
            const int t = t0 + 32 * q;
            const bool in = t < gb * nd;
            const int g = g0 + (in ? L.g : gb - 1), j = in ? L.j : nd - 1;
            L.next();
            const int a = S.grp[g] >> 4, kind = S.grp[g] & 15;
            const int ee = S.ent_e[a];
            const int e = ee >= 0 ? ee : ~ee, i = S.ent_i[a];
            const int64_t own = ((int64_t)e * nd + i) * nd + j;
            int pos;
            double v;
            if (kind == 0) {
              const int64_t eo = (int64_t)S.ent_slot[a];
              v = (double)load_entry<T>(elmat + eo * mat_stride<T>(nd, SYM), nd, i, j, SYM);
              pos = A.fpos_el[own];
            } else {
              // patch matrices are spatial: local space-time index = time dof * nds + spatial dof
              const int lf = (kind - 1) >> 1, h = (kind - 1) & 1;
              const int first = S.ent_first[a * 4 + lf], fs = S.ent_fs[a * 4 + lf];
              const int nds = A.nds, n2s = 2 * nds;
              int ir = 0, jr = i, ic = 0, jc = j;
              if (ST) {
                ir = i / nds;
                jr = i - ir * nds;
                ic = j / nds;
                jc = j - ic * nds;
              }
              const int prow = first ? jr : nds + jr, pcol = h * nds + jc;
              const bool self = (h == 0) == (first != 0);
              if (fs < A.cap_fa) {
                const double pv = (double)load_entry<T>(famat + (int64_t)fs * mat_stride<T>(n2s, true), n2s, prow,
                                                        pcol, true);
                v = ST ? A.mt[ir * A.kt1 + ic] * pv : pv;
                pos = self ? (int)A.fpos_el[own]
                           : (int)A.pbuf[(((int64_t)fs * 2 + (first ? 0 : 1)) * nd + i) * nd + j];
              } else {
                v = 0.0;
                pos = -1;
              }
            }
            vq[q] = v;
            pq[q] = in ? pos : -1;
          }
#pragma unroll
          for (int q = 0; q < QQ; q++) {
            const int t = t0 + 32 * q;
            if (t < gb * nd) {
              S.spos[t] = pq[q];
              S.sval[t] = vq[q];
            }
          }
        }
        __syncwarp();
        for (int g = 0; g < gb; g++) {
          if (lane < nd) {
            const int pos = S.spos[g * nd + lane];
            if (pos >= 0 && pos < len) S.acc[pos] += S.sval[g * nd + lane];
          }
          __syncwarp();
        }
      }
    }
    // compressed write: ascending active columns
    int base = 0;
    for (int k0 = 0; k0 < len; k0 += 32) {
      const int k = k0 + lane;
      const bool fl = k < len && A.flags[fo + k];
      const unsigned m = __ballot_sync(0xffffffffu, fl);
      if (fl) {
        const int c = base + __popc(m & ((1u << lane) - 1));
        if (c < u) {
          cols[rp + c] = A.dof_row[A.tmp_cols[fo + k]];
          vals[rp + c] = S.acc[k];
        }
      }
      base += __popc(m);
    }
    if (lane == 0 && base != u) set_err(err, XG_ERR_CAPACITY);
    __syncwarp();
  }
}


}  // namespace xg

using namespace xg;

// ============================================================================
// The form object
// ============================================================================
struct xg_form {
  xg_space* space = nullptr;
  xg_mesh* mesh = nullptr;
  int precision = XG_PREC_FP64;
  // terms on regions of several level sets (xg_mlset_form_create)
  bool ml = false;
  int ml_M = 0;
  std::vector<MlTermDev> ml_terms;
  MlTermDev* d_ml_terms = nullptr;
  int8_t* d_ml_tuples = nullptr;
  std::vector<xg_term> terms;
  std::vector<int> term_slot;  // group index (volume) or patch index
  // boundary terms (xg_form_set_bnd_terms) and the elements owning BND elements
  BndDesc bnd = {};
  int n_own = 0;
  int32_t* d_own = nullptr;  // [n_own] owners, [n_own + 1] pointers, [nbnd] BND elements
  // volume terms with a coefficient field (xg_form_set_coef_terms)
  CoefDesc cdesc = {};
  const double* d_patch_deform = nullptr;  // xg_form_set_deformation: patch terms on the deformed mesh
  cudaStream_t side = nullptr;             // the facet kernels' stream (forked from and joined into the step's)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool rows_marked = false;  // the step's active rows were marked in rows_front
  FormDesc desc;
  int needs_mask = 0;  // domains needing decompositions on cut elements
  int el_sym = 0;      // every volume group symmetric: packed element matrices
  double* d_tabs = nullptr;  // reference tables of the uncut kernel
  float* d_tabs_f = nullptr;  // their FP32 copies (mixed form)
  UncutTabs tabs = {};
  MomDesc md = {};              // moment sets of the cut element kernels
  EntTabs ent = {};             // their integer term tables
  int32_t* d_mtab_i = nullptr;  // term offsets and indices
  void* d_mtab_c = nullptr;     // term coefficients (kernel precision)
  void* d_mu = nullptr;         // [cap_cgeo][mu_MT] moments of the cut elements (per step)
  int64_t mu_MT = 0;
  size_t mo_smem = 0;
  int grid_mo = 0, grid_en = 0;
  bool patch_exact = false;     // every patch term integrates exactly: basis-change patch kernel
  void* d_mhat = nullptr;       // reference mass matrix of the canonical basis (kernel precision)
  int grid_px = 0;
  int64_t nw32_el = 0, nw32_fa = 0, nw32_dof = 0;
  int64_t cap_el = 0, cap_fa = 0;
  // workspace
  uint32_t* d_act_un = nullptr;
  uint32_t* d_act_cut = nullptr;
  uint32_t* d_act_fa = nullptr;
  uint32_t* d_dof_bits = nullptr;
  int32_t* d_l_un = nullptr;
  int32_t* d_l_cut = nullptr;
  int32_t* d_l_fa = nullptr;
  int32_t* d_cutlist = nullptr;  // [ne + 1] cut elements of the step's marking
  uint8_t* d_dof_flag = nullptr;  // [ndof] active-dof bytes (zero between steps)
  int32_t* d_el_slot = nullptr;
  int32_t* d_fa_slot = nullptr;
  int32_t* d_dof_row = nullptr;
  int64_t* d_rowcnt = nullptr;
  int* d_counts = nullptr;  // [n_uncut, n_cut, n_facets, n_rows]
  int* d_bsum = nullptr;    // compaction block sums
  int nbsum = 0;
  long long* d_bsum64 = nullptr;
  int nbsum64 = 0;
  void* d_elmat = nullptr;
  void* d_famat = nullptr;
  int* d_err = nullptr;
  int sc_hs = 0, sc_maxu = 0, sc_stage = 0, sc_wbytes = 0;
  size_t sc_smem = 0;
  int sm_wbytes = 0, grid_sm = 0;  // per-step summing pass
  size_t sm_smem = 0;
  int64_t full_nnz = 0;
  int64_t* d_full_ptr = nullptr;
  int32_t* d_tmp_cols = nullptr;  // full-pattern columns of every dof row (sorted), built at creation
  uint16_t* d_fpos_el = nullptr;  // [ne][nd][nd]: position of element column j in the full row of local row i
  uint16_t* d_pbuf = nullptr;     // [cap_fa][2][nd][nd]: neighbour-column positions of active facets (per step)
  uint8_t* d_flags = nullptr;     // [full_nnz]: active columns of each active row (per step)
  void* d_pgeo = nullptr;         // [cap_fa] per-facet patch geometry (per step)
  void* d_cgeo = nullptr;         // [cap_cgeo] per-cut-element geometry and sub-simplices (per step)
  void* d_csub = nullptr;
  int64_t cap_cgeo = 0;
  int max_unique = 0;
  int grid_el_un = 0, grid_el_cut = 0, grid_fa = 0, grid_sc = 0;
  // CutFEM step state
  uint8_t* d_dom = nullptr;
  double* d_ratio = nullptr;
  uint64_t* d_bits = nullptr;
  uint64_t* d_fbits = nullptr;
  uint64_t* d_fbits_sk = nullptr;  // [2][facet words]: skeleton facets of the CutFEM step (NEG, POS)
  bool has_patch = false;
  cudaEvent_t ev[8] = {};
  bool use_ev = false;
  // space-time forms
  bool st = false;
  StFormDesc stdesc = {};
  StTimeTabs st_tt = {};  // time sums of the uncut space-time kernel
  std::vector<xg_st_term> st_terms;
  double mt[9] = {1, 0, 0, 0, 0, 0, 0, 0, 0};  // time mass of the time rule (patch factor)
  // spatial forms: element rows in the row-major layout of xg_rows.h
  bool rows = false;
  bool defer_patch = false;  // batched graph: the basis-change patch kernel runs for several forms at once
  int32_t* d_el_rowslot = nullptr;  // [ne][nd]
  uint16_t* d_pos_rows = nullptr;   // [ne * nd][nd]
  uint16_t* d_nbpos = nullptr;      // [ne * nd * nfl][nd]
  int32_t* d_cand_fs = nullptr;     // [ne * nd * nfl]
  uint8_t* d_act_slot = nullptr;    // [ne * nd]
  int32_t* d_vcols = nullptr;       // [full_nnz]
  double* d_vvals = nullptr;        // [full_nnz]
  long long* d_bsum_rows = nullptr;
  int nbsum_rows = 0;
  int rows_W = 0, rows_copies = 1, rows_grid = 0, rows_warps = 8;
  size_t rows_smem = 0;
  // launch configuration chosen by the autotuner (xg_form_autotune)
  int tune_uncut_epb = 32;  // uncut elements per block: 16 or 32
  int grid_el_un16 = 0;
  int px_bps = 0;           // blocks per SM of the basis-change patch kernel (0: occupancy)
  int px_occ = 1;           // its occupancy limit (blocks per SM)
};

namespace {

int form_workspace(xg_form* f);
int apply_cached_tune(xg_form* f);

int form_free(xg_form* f) {
  void* ptrs[] = {f->d_full_ptr, f->d_tmp_cols, f->d_fpos_el, f->d_pbuf, f->d_flags, f->d_pgeo, f->d_cgeo, f->d_csub,
                  f->d_tabs, f->d_tabs_f, f->d_act_un, f->d_act_cut, f->d_act_fa, f->d_dof_bits, f->d_l_un, f->d_l_cut, f->d_l_fa,
                  f->d_el_slot, f->d_fa_slot, f->d_dof_row, f->d_rowcnt, f->d_counts, f->d_bsum, f->d_bsum64,
                  f->d_elmat, f->d_famat, f->d_err, f->d_dom, f->d_ratio, f->d_bits, f->d_fbits, f->d_fbits_sk,
                  f->d_mtab_i, f->d_mtab_c, f->d_mu, f->d_mhat, f->d_cutlist, f->d_dof_flag,
                  f->d_el_rowslot, f->d_pos_rows, f->d_nbpos, f->d_cand_fs, f->d_act_slot, f->d_vcols, f->d_vvals,
                  f->d_bsum_rows, f->d_ml_terms, f->d_ml_tuples, f->d_own};
  for (void* p : ptrs) cudaFree(p);
  if (f->side) cudaStreamDestroy(f->side);
  if (f->ev_fork) cudaEventDestroy(f->ev_fork);
  if (f->ev_join) cudaEventDestroy(f->ev_join);
  delete f;
  return XG_OK;
}

int default_order(int kind, int k) {
  switch (kind) {
    case XG_TERM_MASS: return 2 * k;
    case XG_TERM_LAPLACE: return 2 * k - 2;
    case XG_TERM_NGRADU_V:
    case XG_TERM_U_NGRADV:
    case XG_TERM_CONV: return 2 * k - 1;
    case XG_TERM_GHOST_MASS: return 2 * k;
    case XG_TERM_NGRADU_NGRADV: return 2 * k - 2;
  }
  return 2 * k;
}

// rebuild the group table from the term list
int build_desc(xg_form* f) {
  FormDesc& d = f->desc;
  std::memset(&d, 0, sizeof(d));
  f->term_slot.assign(f->terms.size(), -1);
  f->needs_mask = 0;
  f->has_patch = false;
  for (size_t t = 0; t < f->terms.size(); t++) {
    const xg_term& T = f->terms[t];
    const int order = T.order >= 0 ? T.order : default_order(T.kind, f->space->order);
    if (order > kMaxOrder) {
      set_last_error("xg_form: integration order above 8");
      return XG_ERR_UNSUPPORTED;
    }
    if (T.kind == XG_TERM_GHOST_MASS) {
      if (d.npatch >= kMaxPatch) return XG_ERR_UNSUPPORTED;
      PatchDesc& P = d.p[d.npatch];
      P.order = order;
      P.defined_on = T.d_defined_on;
      P.c = T.coef;
      P.hpow = T.hpow;
      f->term_slot[t] = d.npatch++;
      f->has_patch = true;
      continue;
    }
    if (T.kind >= XG_TERM_SKEL_JUMP && T.kind <= XG_TERM_SKEL_DN3) {
      // skeleton terms: grouped by (region, facet set), one facet rule per group
      const int kk = T.kind - XG_TERM_SKEL_JUMP;
      if (T.domain != XG_NEG && T.domain != XG_POS && T.domain != XG_WHOLE) {
        set_last_error("xg_form: skeleton terms run on XG_NEG, XG_POS or XG_WHOLE (codim-2 rules are not built)");
        return XG_ERR_UNSUPPORTED;
      }
      if (kk >= 3 && kk - 2 > f->space->order) {
        set_last_error("xg_form: normal-derivative order above the order of the space");
        return XG_ERR_ARG;
      }
      int g = -1;
      for (int q = 0; q < d.nskel; q++)
        if (d.s[q].region == T.domain && d.s[q].defined_on == T.d_defined_on && !((d.s[q].used >> kk) & 1)) g = q;
      if (g < 0) {
        if (d.nskel >= kMaxSkel) {
          set_last_error("xg_form: too many skeleton term groups");
          return XG_ERR_UNSUPPORTED;
        }
        g = d.nskel++;
        d.s[g].region = T.domain;
        d.s[g].defined_on = T.d_defined_on;
      }
      d.s[g].c[kk] = T.coef;
      d.s[g].hpow[kk] = T.hpow;
      d.s[g].used |= 1 << kk;
      f->term_slot[t] = g;
      f->has_patch = true;
      continue;
    }
    if (T.kind < 0 || T.kind > XG_TERM_CONV || T.domain < 0 || T.domain > 2) {
      set_last_error("xg_form: bad term kind or domain");
      return XG_ERR_ARG;
    }
    int g = -1;
    for (int q = 0; q < d.ngroups; q++) {
      const GroupDesc& G = d.g[q];
      bool same_b = T.kind != XG_TERM_CONV || !(G.used & (1 << XG_TERM_CONV)) ||
                    (G.b[0] == T.b[0] && G.b[1] == T.b[1] && G.b[2] == T.b[2]);
      if (G.domain == T.domain && G.order == order && G.defined_on == T.d_defined_on && same_b &&
          !(G.used & (1 << T.kind)))
        g = q;
    }
    if (g < 0) {
      if (d.ngroups >= kMaxGroups) {
        set_last_error("xg_form: too many term groups");
        return XG_ERR_UNSUPPORTED;
      }
      g = d.ngroups++;
      d.g[g].domain = T.domain;
      d.g[g].order = order;
      d.g[g].defined_on = T.d_defined_on;
    }
    GroupDesc& G = d.g[g];
    G.c[T.kind] = T.coef;
    G.hpow[T.kind] = T.hpow;
    G.used |= 1 << T.kind;

    if (T.kind == XG_TERM_CONV)
      for (int k = 0; k < 3; k++) G.b[k] = T.b[k];
    f->term_slot[t] = g;
    f->needs_mask |= 1 << T.domain;
  }
  f->el_sym = 1;
  for (int q = 0; q < d.ngroups; q++) {
    const GroupDesc& G = d.g[q];
    const int n1 = 1 << XG_TERM_NGRADU_V, n2 = 1 << XG_TERM_U_NGRADV;
    bool sym = !(G.used & (1 << XG_TERM_CONV));
    if ((G.used & n1) || (G.used & n2))
      sym = sym && (G.used & n1) && (G.used & n2) && G.c[XG_TERM_NGRADU_V] == G.c[XG_TERM_U_NGRADV] &&
            G.hpow[XG_TERM_NGRADU_V] == G.hpow[XG_TERM_U_NGRADV];
    if (!sym) f->el_sym = 0;
  }
  return XG_OK;
}

// Reference tables of the uncut kernel for every NEG/POS group: the group's
// rule on the reference simplex applied to products of the canonical basis
// (edge orientation by local vertex number).
template <int D, int K>
std::vector<double> uncut_tables(const FormDesc& d, bool sym, size_t offs[][3]) {
  constexpr int N = ndof_el(D, K);
  const int E = sym ? tri_size(N) : N * N;
  const int NG = D * (D + 1) / 2;
  const RuleTable& R = host_rules();
  std::vector<double> buf;
  int gv[4] = {0, 1, 2, 3};
  int desc[N];
  for (int i = 0; i < N; i++) desc[i] = fn_desc<D, K>(i, gv);
  double g[D + 1][D];
  for (int a = 0; a <= D; a++)
    for (int k = 0; k < D; k++) g[a][k] = a < D ? (a == k ? 1.0 : 0.0) : -1.0;
  for (int q = 0; q < d.ngroups; q++) {
    offs[q][0] = offs[q][1] = offs[q][2] = (size_t)-1;
    const GroupDesc& G = d.g[q];
    if (G.domain == XG_IF) continue;
    const int p = clamp_order(G.order), off = R.off[D][p], cnt = R.cnt[D][p];
    std::vector<double> phi((size_t)cnt * N), dphi((size_t)cnt * N * D);
    for (int x = 0; x < cnt; x++) {
      double lam[D + 1], s = 0;
      for (int a = 0; a < D; a++) {
        lam[a] = R.x[off + x][a];
        s += lam[a];
      }
      lam[D] = 1.0 - s;
      for (int i = 0; i < N; i++) {
        double gr[D];
        eval_fn<D, double>(desc[i], lam, g, phi[(size_t)x * N + i], gr);
        for (int k = 0; k < D; k++) dphi[((size_t)x * N + i) * D + k] = gr[k];
      }
    }
    auto entry = [&](int k, int& pp, int& qq) {
      if (sym) {
        pp = 0;
        int rem = k;
        while (rem >= N - pp) {
          rem -= N - pp;
          pp++;
        }
        qq = pp + rem;
      } else {
        pp = k / N;
        qq = k % N;
      }
    };
    if (G.used & (1 << XG_TERM_MASS)) {
      offs[q][0] = buf.size();
      for (int k = 0; k < E; k++) {
        int pp, qq;
        entry(k, pp, qq);
        double s = 0;
        for (int x = 0; x < cnt; x++) s += R.w[off + x] * phi[(size_t)x * N + pp] * phi[(size_t)x * N + qq];
        buf.push_back(s);
      }
    }
    if (G.used & (1 << XG_TERM_LAPLACE)) {
      offs[q][1] = buf.size();
      for (int a = 0; a < D; a++)
        for (int b = a; b < D; b++)
          for (int k = 0; k < E; k++) {
            int pp, qq;
            entry(k, pp, qq);
            double s = 0;
            for (int x = 0; x < cnt; x++) {
              const double* dp = &dphi[((size_t)x * N + pp) * D];
              const double* dq = &dphi[((size_t)x * N + qq) * D];
              double v = dp[a] * dq[b];
              if (a != b) v += dp[b] * dq[a];
              s += R.w[off + x] * v;
            }
            buf.push_back(s);
          }
    }
    if (G.used & (1 << XG_TERM_CONV)) {
      offs[q][2] = buf.size();
      for (int a = 0; a < D; a++)
        for (int k = 0; k < E; k++) {
          int pp, qq;
          entry(k, pp, qq);
          double s = 0;
          for (int x = 0; x < cnt; x++) s += R.w[off + x] * phi[(size_t)x * N + pp] * dphi[((size_t)x * N + qq) * D + a];
          buf.push_back(s);
        }
    }
    (void)NG;
  }
  return buf;
}

// Moment sets of the cut element kernels: groups of one domain whose rule is
// exact for their integrand (order >= degree) share one set, computed with the
// rule of the set's degree; a group whose rule is below its integrand degree
// keeps its own rule, so its moments reproduce that rule's sums.
void build_moment_desc(xg_form* f) {
  const int D = f->mesh->dim, K = f->space->order;
  MomDesc& md = f->md;
  std::memset(&md, 0, sizeof(md));
  bool exact[kMaxGroups] = {};
  for (int q = 0; q < f->desc.ngroups; q++) {
    const GroupDesc& G = f->desc.g[q];
    int deg = 0;
    if (G.used & (1 << XG_TERM_MASS)) deg = std::max(deg, 2 * K);
    if (G.used & (1 << XG_TERM_LAPLACE)) deg = std::max(deg, 2 * K - 2);
    if (G.used & ((1 << XG_TERM_NGRADU_V) | (1 << XG_TERM_U_NGRADV) | (1 << XG_TERM_CONV)))
      deg = std::max(deg, 2 * K - 1);
    const int p = clamp_order(G.order);
    const bool ex = p >= deg;
    int s = -1;
    for (int t = 0; t < md.nsets; t++)
      if (md.dt[t] == G.domain && exact[t] == ex && (ex || md.order[t] == p)) s = t;
    if (s < 0) {
      s = md.nsets++;
      md.dt[s] = G.domain;
      md.order[s] = p;
      exact[s] = ex;
    }
    md.deg[s] = std::max(md.deg[s], deg);
    md.set_of[q] = s;
  }
  md.NA = md.NB = 1;
  for (int s = 0; s < md.nsets; s++) {
    if (exact[s]) md.order[s] = md.deg[s];
    md.M[s] = mono_count(D + 1, md.deg[s]);
    md.off[s] = md.MT;
    md.MT += md.M[s];
    md.NA = std::max(md.NA, pair_count(md.deg[s]));
    md.NB = std::max(md.NB, D == 3 ? pair_count(md.deg[s]) : md.deg[s] + 1);
  }
  f->mo_smem = (size_t)kMomPts * (md.NA + md.NB) * (f->precision == XG_PREC_FP64 ? 8 : 4);
}

// Reference mass matrix of the canonical basis (unit |det F|) for the
// basis-change patch kernel, when every patch term's rule is exact (order >= 2K).
template <int D, int K>
std::vector<double> reference_mass() {
  constexpr int N = ndof_el(D, K);
  const RuleTable& R = host_rules();
  const int p = clamp_order(2 * K), off = R.off[D][p], cnt = R.cnt[D][p];
  int gv[4] = {0, 1, 2, 3};
  std::vector<double> M((size_t)N * N, 0.0);
  for (int x = 0; x < cnt; x++) {
    double lam[D + 1], s = 0;
    for (int a = 0; a < D; a++) {
      lam[a] = R.x[off + x][a];
      s += lam[a];
    }
    lam[D] = 1.0 - s;
    double phi[N];
    for (int i = 0; i < N; i++) phi[i] = eval_fn_value<D, double>(fn_desc<D, K>(i, gv), lam);
    for (int i = 0; i < N; i++)
      for (int j = 0; j < N; j++) M[(size_t)i * N + j] += R.w[off + x] * phi[i] * phi[j];
  }
  return M;
}

template <class K>
int grid_for(K kernel, int threads, size_t smem);

template <int D, int K, typename T>
int patch_exact_setup(xg_form* f) {
  auto kx = k_patch_exact<D, K, T>;
  const size_t smem = sizeof(PxSmem<D, K, T>);
  XG_CUDA(cudaFuncSetAttribute(kx, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  f->grid_px = grid_for(kx, PxCfg<D, K>::NT, smem);
  f->px_occ = std::max(1, f->grid_px / 152);
  return XG_OK;
}

template <typename T>
int patch_exact_setup_t(xg_form* f) {
  const int D = f->mesh->dim, K = f->space->order;
  if (D == 2) return K == 1 ? patch_exact_setup<2, 1, T>(f) : (K == 2 ? patch_exact_setup<2, 2, T>(f) : patch_exact_setup<2, 3, T>(f));
  return K == 1 ? patch_exact_setup<3, 1, T>(f) : (K == 2 ? patch_exact_setup<3, 2, T>(f) : patch_exact_setup<3, 3, T>(f));
}

int upload_patch_tables(xg_form* f) {
  const int D = f->mesh->dim, K = f->space->order;
  f->patch_exact = f->has_patch && f->desc.npatch > 0;
  for (int pp = 0; pp < f->desc.npatch; pp++)
    if (clamp_order(f->desc.p[pp].order) < 2 * K) f->patch_exact = false;
  cudaFree(f->d_mhat);
  f->d_mhat = nullptr;
  if (!f->patch_exact) return XG_OK;
  std::vector<double> M;
  if (D == 2) M = K == 1 ? reference_mass<2, 1>() : (K == 2 ? reference_mass<2, 2>() : reference_mass<2, 3>());
  else M = K == 1 ? reference_mass<3, 1>() : (K == 2 ? reference_mass<3, 2>() : reference_mass<3, 3>());
  const bool fp64 = f->precision == XG_PREC_FP64;
  std::vector<float> M32(M.begin(), M.end());
  XG_CUDA(cudaMalloc(&f->d_mhat, M.size() * (fp64 ? 8 : 4)));
  XG_CUDA(cudaMemcpy(f->d_mhat, fp64 ? (const void*)M.data() : (const void*)M32.data(), M.size() * (fp64 ? 8 : 4),
                     cudaMemcpyHostToDevice));
  return fp64 ? patch_exact_setup_t<double>(f) : patch_exact_setup_t<float>(f);
}

int upload_moment_tables(xg_form* f) {
  if (int st = upload_patch_tables(f)) return st;
  build_moment_desc(f);
  const int D = f->mesh->dim, K = f->space->order;
  const bool sym = f->el_sym;
  std::vector<int32_t> ptr[4], ix[4];
  std::vector<double> cf[4];
  if (D == 2) {
    if (K == 1) moment_tables<2, 1>(sym, ptr, ix, cf);
    else if (K == 2) moment_tables<2, 2>(sym, ptr, ix, cf);
    else moment_tables<2, 3>(sym, ptr, ix, cf);
  } else {
    if (K == 1) moment_tables<3, 1>(sym, ptr, ix, cf);
    else if (K == 2) moment_tables<3, 2>(sym, ptr, ix, cf);
    else moment_tables<3, 3>(sym, ptr, ix, cf);
  }
  std::vector<int32_t> ibuf;
  size_t ioff[4][2], coff[4], nc = 0;
  for (int k = 0; k < 4; k++) {
    ioff[k][0] = ibuf.size();
    ibuf.insert(ibuf.end(), ptr[k].begin(), ptr[k].end());
    ioff[k][1] = ibuf.size();
    ibuf.insert(ibuf.end(), ix[k].begin(), ix[k].end());
    coff[k] = nc;
    nc += cf[k].size();
  }
  const bool fp64 = f->precision == XG_PREC_FP64;
  std::vector<double> c64;
  std::vector<float> c32;
  for (int k = 0; k < 4; k++)
    for (double c : cf[k]) {
      c64.push_back(c);
      c32.push_back((float)c);
    }
  cudaFree(f->d_mtab_i);
  cudaFree(f->d_mtab_c);
  f->d_mtab_i = nullptr;
  f->d_mtab_c = nullptr;
  const size_t csz = fp64 ? 8 : 4;
  XG_CUDA(cudaMalloc((void**)&f->d_mtab_i, std::max<size_t>(ibuf.size(), 1) * 4));
  XG_CUDA(cudaMalloc(&f->d_mtab_c, std::max<size_t>(nc, 1) * csz));
  XG_CUDA(cudaMemcpy(f->d_mtab_i, ibuf.data(), ibuf.size() * 4, cudaMemcpyHostToDevice));
  if (nc)
    XG_CUDA(cudaMemcpy(f->d_mtab_c, fp64 ? (const void*)c64.data() : (const void*)c32.data(), nc * csz,
                       cudaMemcpyHostToDevice));
  for (int k = 0; k < 4; k++) {
    f->ent.ptr[k] = f->d_mtab_i + ioff[k][0];
    f->ent.idx[k] = f->d_mtab_i + ioff[k][1];
    f->ent.coef[k] = (const char*)f->d_mtab_c + coff[k] * csz;
  }
  if (f->mo_smem > 48 * 1024) {
    // the attribute is an upper bound shared by all forms: only ever raise it
    static std::mutex mu;
    static size_t raised[2][2] = {{48 * 1024, 48 * 1024}, {48 * 1024, 48 * 1024}};
    std::lock_guard<std::mutex> lock(mu);
    size_t& r = raised[D - 2][fp64 ? 0 : 1];
    if (f->mo_smem > r) {
      const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
      cudaError_t e;
      if (D == 2) e = fp64 ? cudaFuncSetAttribute(k_cut_moments<2, double>, at, (int)f->mo_smem)
                           : cudaFuncSetAttribute(k_cut_moments<2, float>, at, (int)f->mo_smem);
      else e = fp64 ? cudaFuncSetAttribute(k_cut_moments<3, double>, at, (int)f->mo_smem)
                    : cudaFuncSetAttribute(k_cut_moments<3, float>, at, (int)f->mo_smem);
      if (e) return cuda_fail(e, "xg_form: moment kernel shared memory");
      r = f->mo_smem;
    }
  }
  // the moment workspace grows if a rebuild needs more moments per element
  if (f->d_mu && f->md.MT > f->mu_MT) {
    cudaFree(f->d_mu);
    f->d_mu = nullptr;
    XG_CUDA(cudaMalloc(&f->d_mu, (size_t)f->cap_cgeo * f->md.MT * csz));
    f->mu_MT = f->md.MT;
  }
  return XG_OK;
}

// Tables of the uncut space-time kernel: the spatial reference tables of
// every group (the mass table also serves the d/dtau term) and the time sums
// of the form's time rule (or of the fixed time tref).
int st_uncut_tables(xg_form* f) {
  const StFormDesc& d = f->stdesc;
  const int D = f->mesh->dim, K = f->space->order, kt = f->space->kt;
  FormDesc tmp;
  std::memset(&tmp, 0, sizeof(tmp));
  tmp.ngroups = d.ngroups;
  for (int q = 0; q < d.ngroups; q++) {
    const int used = d.g[q].used;
    tmp.g[q].domain = d.g[q].domain;
    tmp.g[q].order = d.g[q].order;
    int u = 0;
    if (used & ((1 << XG_TERM_MASS) | (1 << XG_TERM_DT_U_V))) u |= 1 << XG_TERM_MASS;
    if (used & (1 << XG_TERM_LAPLACE)) u |= 1 << XG_TERM_LAPLACE;
    if (used & (1 << XG_TERM_CONV)) u |= 1 << XG_TERM_CONV;
    tmp.g[q].used = u;
  }
  size_t offs[kMaxGroups][3];
  std::vector<double> buf;
  if (D == 2) buf = K == 1 ? uncut_tables<2, 1>(tmp, false, offs) : uncut_tables<2, 2>(tmp, false, offs);
  else buf = K == 1 ? uncut_tables<3, 1>(tmp, false, offs) : uncut_tables<3, 2>(tmp, false, offs);
  cudaFree(f->d_tabs);
  f->d_tabs = nullptr;
  std::memset(&f->tabs, 0, sizeof(f->tabs));
  if (!buf.empty()) {
    XG_CUDA(cudaMalloc((void**)&f->d_tabs, buf.size() * sizeof(double)));
    XG_CUDA(cudaMemcpy(f->d_tabs, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice));
    for (int q = 0; q < d.ngroups; q++) {
      f->tabs.m[q] = offs[q][0] == (size_t)-1 ? nullptr : f->d_tabs + offs[q][0];
      f->tabs.t[q] = offs[q][1] == (size_t)-1 ? nullptr : f->d_tabs + offs[q][1];
      f->tabs.c[q] = offs[q][2] == (size_t)-1 ? nullptr : f->d_tabs + offs[q][2];
    }
  }
  StTimeTabs& T = f->st_tt;
  std::memset(&T, 0, sizeof(T));
  const RuleTable& R = host_rules();
  const int pt = clamp_order(d.order_time), offt = R.off[1][pt], nqt = R.cnt[1][pt];
  for (int q = 0; q < d.ngroups; q++) {
    const StGroupDesc& G = d.g[q];
    const bool fixed = G.tref >= 0.0;
    const int np = fixed ? 1 : nqt;
    for (int x = 0; x < np; x++) {
      const double tau = fixed ? G.tref : R.x[offt + x][0], w = fixed ? 1.0 : R.w[offt + x];
      double psi[3], dpsi[3];
      time_basis<double>(kt, tau, psi, dpsi);
      double bt[3] = {G.b[0], G.b[1], G.b[2]};
      if ((G.used & (1 << XG_TERM_CONV)) && G.omega != 0.0) {
        const double tp = G.t0 + G.dt * tau;
        const double cs = std::cos(G.omega * tp), sn = std::sin(G.omega * tp);
        for (int r = 0; r < 3; r++) bt[r] += G.bc[r] * cs + G.bs[r] * sn;
      }
      for (int a = 0; a <= kt; a++)
        for (int b = 0; b <= kt; b++) {
          const int ti = a * (kt + 1) + b;
          T.tm[q][ti] += w * psi[a] * psi[b];
          T.td[q][ti] += w * psi[a] * dpsi[b];
          for (int r = 0; r < 3; r++) T.tb[q][ti][r] += w * psi[a] * psi[b] * bt[r];
        }
    }
  }
  return XG_OK;
}

template <int D, int K, int KT, typename T>
int launch_st_uncut(xg_form* f, cudaStream_t s) {
  auto kern = k_st_elmat_uncut<D, K, KT, T>;
  if (!f->grid_el_un) f->grid_el_un = grid_for(kern, 256, 0);
  xg_mesh* m = f->mesh;
  StFormDesc d = f->stdesc;
  const int64_t nw = f->nw32_el / 2;
  for (int q = 0; q < d.ngroups; q++)
    d.g[q].defined_on = f->d_bits + (d.g[q].domain == XG_NEG ? XG_CDOM_HASNEG
                                                              : (d.g[q].domain == XG_IF ? XG_CDOM_IF : XG_CDOM_HASPOS)) *
                                        nw;
  kern<<<f->grid_el_un, 256, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, f->d_dom, d, f->tabs, f->st_tt, f->d_l_un,
                                     f->d_counts, (T*)f->d_elmat, f->d_err);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_st_elmat_uncut");
}

template <typename T>
int dispatch_st_uncut(xg_form* f, cudaStream_t s) {
  const int D = f->mesh->dim, K = f->space->order, KT = f->space->kt;
  if (D == 2) {
    if (K == 1) return KT == 1 ? launch_st_uncut<2, 1, 1, T>(f, s) : launch_st_uncut<2, 1, 2, T>(f, s);
    return KT == 1 ? launch_st_uncut<2, 2, 1, T>(f, s) : launch_st_uncut<2, 2, 2, T>(f, s);
  }
  if (K == 1) return KT == 1 ? launch_st_uncut<3, 1, 1, T>(f, s) : launch_st_uncut<3, 1, 2, T>(f, s);
  return KT == 1 ? launch_st_uncut<3, 2, 1, T>(f, s) : launch_st_uncut<3, 2, 2, T>(f, s);
}

int upload_tables(xg_form* f) {
  size_t offs[kMaxGroups][3];
  std::vector<double> buf;
  const int D = f->mesh->dim, K = f->space->order;
  const bool sym = f->el_sym;
  if (D == 2) {
    if (K == 1) buf = uncut_tables<2, 1>(f->desc, sym, offs);
    else if (K == 2) buf = uncut_tables<2, 2>(f->desc, sym, offs);
    else buf = uncut_tables<2, 3>(f->desc, sym, offs);
  } else {
    if (K == 1) buf = uncut_tables<3, 1>(f->desc, sym, offs);
    else if (K == 2) buf = uncut_tables<3, 2>(f->desc, sym, offs);
    else buf = uncut_tables<3, 3>(f->desc, sym, offs);
  }
  cudaFree(f->d_tabs);
  f->d_tabs = nullptr;
  cudaFree(f->d_tabs_f);
  f->d_tabs_f = nullptr;
  std::memset(&f->tabs, 0, sizeof(f->tabs));
  if (!buf.empty()) {
    XG_CUDA(cudaMalloc((void**)&f->d_tabs, buf.size() * sizeof(double)));
    XG_CUDA(cudaMemcpy(f->d_tabs, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<float> buf_f(buf.begin(), buf.end());
    XG_CUDA(cudaMalloc((void**)&f->d_tabs_f, buf_f.size() * sizeof(float)));
    XG_CUDA(cudaMemcpy(f->d_tabs_f, buf_f.data(), buf_f.size() * sizeof(float), cudaMemcpyHostToDevice));
    for (int q = 0; q < f->desc.ngroups; q++) {
      f->tabs.m[q] = offs[q][0] == (size_t)-1 ? nullptr : f->d_tabs + offs[q][0];
      f->tabs.t[q] = offs[q][1] == (size_t)-1 ? nullptr : f->d_tabs + offs[q][1];
      f->tabs.c[q] = offs[q][2] == (size_t)-1 ? nullptr : f->d_tabs + offs[q][2];
      f->tabs.mf[q] = offs[q][0] == (size_t)-1 ? nullptr : f->d_tabs_f + offs[q][0];
      f->tabs.tf[q] = offs[q][1] == (size_t)-1 ? nullptr : f->d_tabs_f + offs[q][1];
      f->tabs.cf[q] = offs[q][2] == (size_t)-1 ? nullptr : f->d_tabs_f + offs[q][2];
    }
    f->tabs.ok_f = 1;
  }
  return upload_moment_tables(f);
}

template <class K>
int grid_for(K kernel, int threads, size_t smem) {
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
  if (per < 1) per = 1;
  return nsm * per;
}

int compact(xg_form* f, const uint32_t* bits, int64_t nw32, int32_t* list, int32_t* slot, int* count_out,
            cudaStream_t s, const int* slot_base = nullptr) {
  const int nb = (int)((nw32 + kCChunk - 1) / kCChunk);
  if (nb > f->nbsum) return XG_ERR_CAPACITY;
  k_popc_blocks<<<nb, kCThreads, 0, s>>>(bits, nw32, f->d_bsum);
  k_scan_small<<<1, 1024, 0, s>>>(f->d_bsum, nb, count_out);
  k_write_list<<<nb, kCThreads, 0, s>>>(bits, nw32, f->d_bsum, list, slot, slot_base);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "compact");
}

template <int D, int K, bool SYM, typename T>
int launch_volume_sym(xg_form* f, const double* d_lset, const uint8_t* d_dom, cudaStream_t s) {
  using CC = CutCfg<D, K, SYM, T>;
  xg_mesh* m = f->mesh;
  auto ku = k_elmat_uncut<D, K, SYM, T, 32>;
  auto ku16 = k_elmat_uncut<D, K, SYM, T, 16>;
  auto kc = k_elmat_cut<D, K, SYM, T>;
  auto km = k_cut_moments<D, T>;
  auto kn = k_cut_entries<D, K, SYM, T>;
  if (!f->grid_el_un) {
    f->grid_el_un = grid_for(ku, 256, 0);
    f->grid_el_un16 = grid_for(ku16, 256, 0);
    f->grid_el_cut = grid_for(kc, CC::NT, 0);
    f->grid_mo = grid_for(km, kMomNT, f->mo_smem);
    f->grid_en = grid_for(kn, kEntNT, 0);
  }
  const int32_t* ers = f->rows ? f->d_el_rowslot : nullptr;  // spatial forms: element rows by row slot
  if (f->tune_uncut_epb == 16)
    ku16<<<f->grid_el_un16, 256, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, d_dom, f->desc, f->tabs, f->d_l_un,
                                         f->d_counts, (T*)f->d_elmat, f->d_err, ers);
  else
    ku<<<f->grid_el_un, 256, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, d_dom, f->desc, f->tabs, f->d_l_un,
                                     f->d_counts, (T*)f->d_elmat, f->d_err, ers);
  if (f->use_ev) cudaEventRecord(f->ev[3], s);
  k_cut_geo<D><<<152 * 4, 128, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, d_lset, f->desc, f->d_l_cut, f->d_counts,
                                       (CutGeoS*)f->d_cgeo, (CutSubS*)f->d_csub, f->cap_cgeo, f->d_err,
                                       f->needs_mask);
  km<<<f->grid_mo, kMomNT, f->mo_smem, s>>>(f->md, (const CutGeoS*)f->d_cgeo, (const CutSubS*)f->d_csub,
                                            f->d_counts, f->cap_cgeo, (T*)f->d_mu);
  kn<<<f->grid_en, kEntNT, 0, s>>>(f->desc, f->md, f->ent, (const CutGeoS*)f->d_cgeo, f->d_counts, f->cap_cgeo,
                                   (const T*)f->d_mu, (T*)f->d_elmat, f->d_err, ers);
  // cut elements beyond the workspace (none unless more than cap_cgeo are cut)
  kc<<<f->grid_el_cut, CC::NT, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, d_lset, f->desc, f->d_l_cut, f->d_counts,
                                      (T*)f->d_elmat, f->d_err, f->needs_mask, (const CutGeoS*)f->d_cgeo,
                                      (const CutSubS*)f->d_csub, f->cap_cgeo, (int)f->cap_cgeo, ers);
  if (f->use_ev) cudaEventRecord(f->ev[4], s);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_elmat");
}

template <int D, int K, typename T>
int launch_volume(xg_form* f, const double* d_lset, const uint8_t* d_dom, cudaStream_t s) {
  return f->el_sym ? launch_volume_sym<D, K, true, T>(f, d_lset, d_dom, s)
                   : launch_volume_sym<D, K, false, T>(f, d_lset, d_dom, s);
}

template <int D, typename T>
PxJob<D, T> px_job(xg_form* f) {
  PxJob<D, T> J;
  J.pgeo = (const PaGeoS<D, T>*)f->d_pgeo;
  J.counts = f->d_counts;
  J.mhat = (const T*)f->d_mhat;
  J.famat = (T*)f->d_famat;
  J.cap_fa = f->cap_fa;
  J.err = f->d_err;
  J.full_rows = f->rows ? 1 : 0;  // spatial forms: full patch rows in both precisions
  J.npatch = f->desc.npatch;
  J.K = f->space->order;
  return J;
}

template <int D, int K, typename T>
int launch_patch(xg_form* f, cudaStream_t s) {
  using C = PaCfg<D, K>;
  xg_mesh* m = f->mesh;
  auto kp = k_patch<D, K, T>;
  if (!f->grid_fa) f->grid_fa = grid_for(kp, C::NT, 0);
  PaGeoS<D, T>* pg = (PaGeoS<D, T>*)f->d_pgeo;
  const int frs = f->rows ? 1 : 0;  // spatial forms: full patch rows in both precisions
  k_patch_geo<D, T><<<152 * 8, 128, 0, s>>>(m->ne, m->nv, m->d_elv, m->d_xyz, m->nfacets, m->d_facet_els, f->desc,
                                         f->d_l_fa, f->d_counts, pg, f->cap_fa, f->d_err);
  if (f->patch_exact) {
    // batched steps of several forms run this part in one persistent launch
    // for all of them (k_patch_exact_multi)
    if (!f->defer_patch) {
      auto kx = k_patch_exact<D, K, T>;
      const size_t smem = sizeof(PxSmem<D, K, T>);
      kx<<<f->grid_px, PxCfg<D, K>::NT, smem, s>>>(px_job<D, T>(f));
    }
  } else {
    kp<<<f->grid_fa, C::NT, 0, s>>>(f->desc, pg, f->d_counts, (T*)f->d_famat, f->cap_fa, f->d_err, frs);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_patch");
}

template <typename T>
int dispatch_volume(xg_form* f, const double* d_lset, const uint8_t* d_dom, cudaStream_t s) {
  const int D = f->mesh->dim, K = f->space->order;
  if (D == 2) {
    if (K == 1) return launch_volume<2, 1, T>(f, d_lset, d_dom, s);
    if (K == 2) return launch_volume<2, 2, T>(f, d_lset, d_dom, s);
    return launch_volume<2, 3, T>(f, d_lset, d_dom, s);
  }
  if (K == 1) return launch_volume<3, 1, T>(f, d_lset, d_dom, s);
  if (K == 2) return launch_volume<3, 2, T>(f, d_lset, d_dom, s);
  return launch_volume<3, 3, T>(f, d_lset, d_dom, s);
}

template <typename T>
int dispatch_patch(xg_form* f, cudaStream_t s) {
  const int D = f->mesh->dim, K = f->space->order;
  if (D == 2) {
    if (K == 1) return launch_patch<2, 1, T>(f, s);
    if (K == 2) return launch_patch<2, 2, T>(f, s);
    return launch_patch<2, 3, T>(f, s);
  }
  if (K == 1) return launch_patch<3, 1, T>(f, s);
  if (K == 2) return launch_patch<3, 2, T>(f, s);
  return launch_patch<3, 3, T>(f, s);
}

ScatterArgs scatter_args(xg_form* f) {
  ScatterArgs A;
  xg_mesh* m = f->mesh;
  xg_space* sp = f->space;
  A.ne = m->ne;
  A.nd = sp->nd;
  A.nfl = m->dim + 1;
  A.el_dofs = sp->d_el_dofs_aos;
  A.el_facets = m->d_el_facets_aos;
  A.fel = m->d_facet_els_aos;
  A.adj_ptr = sp->d_dof_adj_ptr;
  A.adj = sp->d_dof_adj;
  A.act_un = f->d_act_un;
  A.act_cut = f->d_act_cut;
  A.act_fa = f->d_act_fa;
  A.el_slot = f->d_el_slot;
  A.fa_slot = f->d_fa_slot;
  A.rows = nullptr;
  A.dof_row = f->d_dof_row;
  A.counts = f->d_counts;
  A.cap_fa = f->cap_fa;
  A.el_sym = f->el_sym;
  A.nds = sp->nds;
  A.kt1 = sp->kt >= 0 ? sp->kt + 1 : 1;
  for (int k = 0; k < 9; k++) A.mt[k] = f->mt[k];
  A.full_ptr = f->d_full_ptr;
  A.tmp_cols = f->d_tmp_cols;
  A.fpos_el = f->d_fpos_el;
  A.pbuf = f->d_pbuf;
  A.flags = f->d_flags;
  A.hs = f->sc_hs;
  A.maxu = f->sc_maxu;
  A.ucn = f->sc_maxu;
  A.accn = 0;
  A.stage = 0;
  A.wbytes = f->sc_wbytes;
  return A;
}

RowsArgs rows_args(xg_form* f, const int32_t* rows) {
  RowsArgs R;
  xg_mesh* m = f->mesh;
  xg_space* sp = f->space;
  R.ne = m->ne;
  R.nd = sp->nd;
  R.nfl = m->dim + 1;
  R.n2 = 2 * sp->nd;
  R.W = f->rows_W;
  R.copies = f->rows_copies;
  R.warps = f->rows_warps;
  R.el_dofs = sp->d_el_dofs_aos;
  R.el_facets = m->d_el_facets_aos;
  R.fel = m->d_facet_els_aos;
  R.adj_ptr = sp->d_dof_adj_ptr;
  R.adj = sp->d_dof_adj;
  R.l_fa = f->d_l_fa;
  R.rows = rows;
  R.dof_row = f->d_dof_row;
  R.counts = f->d_counts;
  R.full_ptr = f->d_full_ptr;
  R.tmp_cols = f->d_tmp_cols;
  R.el_rowslot = f->d_el_rowslot;
  R.pos_rows = f->d_pos_rows;
  R.nbpos = f->has_patch ? f->d_nbpos : nullptr;
  R.act_slot = f->d_act_slot;
  R.cand_fs = f->has_patch ? f->d_cand_fs : nullptr;
  R.vcols = f->d_vcols;
  R.vvals = f->d_vvals;
  R.rowcnt = f->d_rowcnt;
  R.cap_fa = f->cap_fa;
  R.bsum = f->d_bsum_rows;
  R.nbsum = f->nbsum_rows;
  R.err = f->d_err;
  return R;
}

// active dofs -> rows (ascending) and dof -> row; spatial forms also mark the
// row slots of the active elements
int mark_rows(xg_form* f, xg_csr* out, cudaStream_t s) {
  xg_mesh* m = f->mesh;
  xg_space* sp = f->space;
  k_mark_dofs<<<152 * 8, 256, 0, s>>>(m->ne, sp->nd, sp->d_el_dofs_aos, f->d_l_un, f->d_l_cut, f->d_l_fa,
                                      f->d_counts, m->nfacets, m->d_facet_els, f->d_dof_flag, f->d_el_rowslot,
                                      f->rows ? f->d_act_slot : nullptr);
  k_pack_dofs<<<(unsigned)((f->nw32_dof * 32 + 255) / 256), 256, 0, s>>>(f->d_dof_flag, sp->ndof, f->d_dof_bits,
                                                                        f->nw32_dof);
  return compact(f, f->d_dof_bits, f->nw32_dof, out->d_row_dof, f->d_dof_row, f->d_counts + 3, s);
}

// active dofs -> rows, then the two scatter passes (space-time forms)
int scatter_phase(xg_form* f, xg_csr* out, cudaStream_t s) {
  xg_space* sp = f->space;
  int st;
  // 3. active dofs -> rows
  if ((st = mark_rows(f, out, s))) return st;
  // 4. pattern and values
  ScatterArgs A = scatter_args(f);
  A.rows = out->d_row_dof;
  k_row_clear<<<152 * 8, 256, 0, s>>>(A);
  k_flag_elements<<<152 * 16, 256, 0, s>>>(A, f->d_l_un, f->d_l_cut);
  if (f->has_patch) k_flag_facets<<<152 * 16, 256, 0, s>>>(A, f->d_l_fa, f->d_err);
  k_row_flagcount<<<152 * 8, 256, 0, s>>>(A, f->d_rowcnt, f->d_err);
  const int nb64 = (int)((sp->ndof + kSChunk - 1) / kSChunk);
  k_sum64_blocks<<<nb64, kSThreads, 0, s>>>(f->d_rowcnt, f->d_counts + 3, f->d_bsum64);
  k_scan64_small<<<1, 1024, 0, s>>>(f->d_bsum64, nb64);
  k_scan64_apply<<<nb64, kSThreads, 0, s>>>(f->d_rowcnt, f->d_counts + 3, f->d_bsum64, out->d_rowptr, out->d_counts,
                                            out->cap_nnz, f->d_err);
  if (f->use_ev) cudaEventRecord(f->ev[6], s);
  A.hs = 0;
  A.ucn = 0;
  A.accn = f->sc_maxu;
  A.stage = f->sc_stage;
  A.wbytes = f->sm_wbytes;
  const bool st_form = A.kt1 > 1;
#define XG_ROW_SUM(TT, SY, STF)                                                                                \
  do {                                                                                                       \
    if (sp->nd >= 10)                                                                                        \
      k_row_sum<TT, SY, STF, 6><<<f->grid_sm, kRowWarps * 32, f->sm_smem, s>>>(                              \
          A, (const TT*)f->d_elmat, (const TT*)f->d_famat, out->d_rowptr, out->d_cols, out->d_vals,          \
          out->cap_nnz, f->d_err);                                                                           \
    else                                                                                                     \
      k_row_sum<TT, SY, STF, 4><<<f->grid_sm, kRowWarps * 32, f->sm_smem, s>>>(                              \
          A, (const TT*)f->d_elmat, (const TT*)f->d_famat, out->d_rowptr, out->d_cols, out->d_vals,          \
          out->cap_nnz, f->d_err);                                                                           \
  } while (0)
  if (f->precision == XG_PREC_FP64) {
    if (st_form) XG_ROW_SUM(double, false, true);
    else if (A.el_sym) XG_ROW_SUM(double, true, false);
    else XG_ROW_SUM(double, false, false);
  } else {
    if (st_form) XG_ROW_SUM(float, false, true);
    else if (A.el_sym) XG_ROW_SUM(float, true, false);
    else XG_ROW_SUM(float, false, false);
  }
#undef XG_ROW_SUM
  if (f->use_ev) cudaEventRecord(f->ev[7], s);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "xg_form_assemble");
}


// Exact size of the largest pattern any level set can produce on this mesh
// (every element and interior facet active) and its widest row.
void full_pattern_stats(const xg_form* f, int64_t* nnz, int* max_unique, std::vector<int64_t>& row_ptr) {
  const xg_space* sp = f->space;
  const xg_mesh* m = f->mesh;
  const int nd = sp->nd, nfl = m->dim + 1, ne = m->ne;
  const int64_t ndof = sp->ndof;
  const std::vector<int32_t>& ed = sp->h_el_dofs;
  const std::vector<int32_t>& efa = m->dim == 2 ? m->h_el_edges : m->h_el_faces;
  const int efs = m->dim == 2 ? 3 : 4;
  std::vector<int32_t> ptr(ndof + 1, 0), adj(ed.size());
  for (size_t k = 0; k < ed.size(); k++) ptr[ed[k] + 1]++;
  for (int64_t r = 0; r < ndof; r++) ptr[r + 1] += ptr[r];
  {
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int e = 0; e < ne; e++)
      for (int k = 0; k < nd; k++) adj[fill[ed[(size_t)e * nd + k]]++] = e;
  }
  const int nth = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
  std::vector<int64_t> part(nth, 0);
  std::vector<int> pmax(nth, 0);
  row_ptr.assign(ndof + 1, 0);
  std::vector<std::thread> th;
  for (int t = 0; t < nth; t++)
    th.emplace_back([&, t]() {
      std::vector<int32_t> c;
      int64_t sum = 0;
      int mx = 0;
      for (int64_t r = t; r < ndof; r += nth) {
        c.clear();
        for (int a = ptr[r]; a < ptr[r + 1]; a++) {
          int e = adj[a];
          c.insert(c.end(), ed.begin() + (size_t)e * nd, ed.begin() + (size_t)(e + 1) * nd);
          if (f->has_patch)
            for (int lf = 0; lf < nfl; lf++) {
              int fc = efa[(size_t)e * efs + lf];
              int e2 = m->h_facet_els[2 * (size_t)fc] == e ? m->h_facet_els[2 * (size_t)fc + 1]
                                                            : m->h_facet_els[2 * (size_t)fc];
              if (e2 >= 0) c.insert(c.end(), ed.begin() + (size_t)e2 * nd, ed.begin() + (size_t)(e2 + 1) * nd);
            }
        }
        std::sort(c.begin(), c.end());
        int u = (int)(std::unique(c.begin(), c.end()) - c.begin());
        row_ptr[r + 1] = u;
        sum += u;
        mx = std::max(mx, u);
      }
      part[t] = sum;
      pmax[t] = mx;
    });
  for (auto& x : th) x.join();
  *nnz = 0;
  *max_unique = 0;
  for (int t = 0; t < nth; t++) {
    *nnz += part[t];
    *max_unique = std::max(*max_unique, pmax[t]);
  }
  for (int64_t r = 0; r < ndof; r++) row_ptr[r + 1] += row_ptr[r];
}

}  // namespace

extern "C" {

int xg_form_create(xg_space* space, const xg_term* terms, int32_t nterms, int precision, xg_form** out) {
  if (!space || !out || (nterms > 0 && !terms) || nterms < 0 ||
      (precision != XG_PREC_FP64 && precision != XG_PREC_MIXED)) {
    set_last_error("xg_form_create: bad arguments");
    return XG_ERR_ARG;
  }
  if (space->kt >= 0) {
    set_last_error("xg_form_create: space-time spaces take xg_st_form_create");
    return XG_ERR_ARG;
  }
  *out = nullptr;
  auto* f = new xg_form();
  f->space = space;
  f->mesh = space->mesh;
  f->precision = precision;
  f->terms.assign(terms, terms + nterms);
  int st = build_desc(f);
  if (!st) st = upload_tables(f);
  if (!st) st = form_workspace(f);
  if (!st) st = apply_cached_tune(f);
  if (st) {
    form_free(f);
    return st;
  }
  *out = f;
  return XG_OK;
}

}  // extern "C"

namespace {

// Full pattern (every element and interior facet active) on the GPU: exact
// distinct-column count per dof -> row offsets of the column scratch, its
// size and the widest row.  Returns XG_ERR_CAPACITY if a row does not fit the
// probe's hash table (the caller then counts on the host).
int full_pattern_probe(xg_form* f, std::vector<int64_t>& full_ptr) {
  xg_mesh* m = f->mesh;
  xg_space* sp = f->space;
  const int64_t ndof = sp->ndof;
  int32_t* d_rows = nullptr;
  std::vector<int32_t> iota(ndof);
  for (int64_t i = 0; i < ndof; i++) iota[i] = (int32_t)i;
  XG_CUDA(cudaMalloc((void**)&d_rows, sizeof(int32_t) * (ndof > 0 ? ndof : 1)));
  cudaError_t e = cudaMemcpy(d_rows, iota.data(), sizeof(int32_t) * ndof, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(f->d_act_cut, 0, f->nw32_el * 4);
  if (e != cudaSuccess) {
    cudaFree(d_rows);
    return cuda_fail(e, "full_pattern_probe");
  }
  k_fill_u32<<<152 * 4, 256>>>(f->d_act_un, f->nw32_el, 0xffffffffu);
  if (f->has_patch) {
    FormDesc all = {};
    all.npatch = 1;
    k_active_facets<<<(unsigned)((f->nw32_fa * 32 + 255) / 256), 256>>>(m->nfacets, m->d_facet_els, all, f->d_act_fa,
                                                                         f->nw32_fa);
  } else {
    cudaMemset(f->d_act_fa, 0, f->nw32_fa * 4);
  }
  ScatterArgs A = scatter_args(f);
  A.rows = d_rows;
  A.hs = 4096;
  A.maxu = 0;
  A.ucn = 0;
  A.accn = 0;
  A.stage = 0;
  A.wbytes = (row_smem_bytes(A.hs, 0, 0, 0) + 15) & ~15;
  const size_t smem = (size_t)kRowWarps * A.wbytes;
  cudaFuncSetAttribute(k_row_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int grid = grid_for(k_row_probe, kRowWarps * 32, smem);
  k_row_probe<<<grid, kRowWarps * 32, smem>>>(A, ndof, f->d_rowcnt, f->d_err);
  std::vector<int64_t> cnt(ndof);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(cnt.data(), f->d_rowcnt, sizeof(int64_t) * ndof, cudaMemcpyDeviceToHost);
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&herr, f->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d_rows);
  if (e != cudaSuccess) return cuda_fail(e, "full_pattern_probe");
  if (herr) return XG_ERR_CAPACITY;
  full_ptr.assign(ndof + 1, 0);
  int mx = 0;
  for (int64_t r = 0; r < ndof; r++) {
    full_ptr[r + 1] = full_ptr[r] + cnt[r];
    mx = std::max(mx, (int)cnt[r]);
  }
  f->full_nnz = full_ptr[ndof];
  f->max_unique = mx;
  return XG_OK;
}

// Static scatter structure (form creation): the sorted full-pattern columns of
// every dof row (the row pass with every element and interior facet active),
// the full-row positions of every element's columns, and the per-step buffers.
// The activity bits still hold the all-active state of the probe.
int full_pattern_build(xg_form* f) {
  xg_mesh* m = f->mesh;
  xg_space* sp = f->space;
  const int64_t ndof = sp->ndof;
  const int64_t nd = sp->nd;
  auto A_ = [&](void** p, size_t bytes) { return cudaMalloc(p, bytes ? bytes : 16); };
  // the per-row scatter of space-time forms keeps element-column positions by
  // element; the row layout of spatial forms by row slot (rows_static_build)
  cudaError_t e = A_(f->rows ? (void**)&f->d_pos_rows : (void**)&f->d_fpos_el, (size_t)m->ne * nd * nd * 2);
  if (!e && !f->rows) e = A_((void**)&f->d_pbuf, f->has_patch ? (size_t)f->cap_fa * 2 * nd * nd * 2 : 16);
  if (!e && !f->rows) e = A_((void**)&f->d_flags, (size_t)f->full_nnz);
  int32_t* d_rows = nullptr;
  if (!e) e = A_((void**)&d_rows, sizeof(int32_t) * (size_t)std::max<int64_t>(ndof, 1));
  if (e) {
    cudaFree(d_rows);
    return cuda_fail(e, "xg_form_create");
  }
  std::vector<int32_t> iota(ndof);
  for (int64_t i = 0; i < ndof; i++) iota[i] = (int32_t)i;
  int cnt[8] = {0, 0, 0, (int)ndof, 0, 0, 0, 0};
  e = cudaMemcpy(d_rows, iota.data(), sizeof(int32_t) * ndof, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(f->d_counts, cnt, sizeof(cnt), cudaMemcpyHostToDevice);
  if (!e) e = cudaMemset(f->d_err, 0, sizeof(int));
  if (e) {
    cudaFree(d_rows);
    return cuda_fail(e, "xg_form_create");
  }
  ScatterArgs A = scatter_args(f);
  A.rows = d_rows;
  k_row_count<<<f->grid_sc, kRowWarps * 32, f->sc_smem>>>(A, f->d_rowcnt, f->d_err);
  if (f->rows) {
    const int rst = rows_static_build(rows_args(f, nullptr), f->has_patch, nullptr);
    if (rst) {
      cudaFree(d_rows);
      return rst;
    }
  } else {
    const int64_t nt = (int64_t)m->ne * nd * nd;
    k_fpos_el<<<(unsigned)std::min<int64_t>((nt + 255) / 256, 152 * 64), 256>>>(A, f->d_fpos_el, f->d_err);
  }
  e = cudaGetLastError();
  int herr = 0;
  if (!e) e = cudaMemcpy(&herr, f->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  std::memset(cnt, 0, sizeof(cnt));
  if (!e) e = cudaMemcpy(f->d_counts, cnt, sizeof(cnt), cudaMemcpyHostToDevice);
  if (!e) e = cudaMemset(f->d_err, 0, sizeof(int));
  cudaFree(d_rows);
  if (e) return cuda_fail(e, "xg_form_create");
  if (herr) {
    set_last_error("xg_form_create: full pattern does not fit the scatter buffers");
    return XG_ERR_CAPACITY;
  }
  return XG_OK;
}

// largest compaction scratch of the row scatter (bytes); see xg_rows.h
constexpr double kRowsScratchBytes = 8.0 * (1 << 30);

// device workspace of a form, sized for the whole mesh
int form_workspace(xg_form* f) {
  xg_space* space = f->space;
  const int precision = f->precision;
  xg_mesh* m = f->mesh;
  const int nd = space->nd;
  const size_t esz = precision == XG_PREC_FP64 ? sizeof(double) : sizeof(float);
  f->nw32_el = 2 * ((m->ne + 63) / 64);
  f->nw32_fa = 2 * ((m->nfacets + 63) / 64);
  f->nw32_dof = 2 * ((space->ndof + 63) / 64);
  f->cap_el = m->ne;
  // facet-patch workspace: all facets when small, else a quarter of them
  const int nds = space->nds;  // patch matrices are spatial (space-time forms apply the time factor in the scatter)
  f->rows = !f->st;
  const size_t fa_stride = precision == XG_PREC_FP64 || f->rows ? (size_t)(2 * nds) * (2 * nds)
                                                                 : (size_t)tri_size(2 * nds);
  const size_t fa_bytes = (size_t)m->nfacets * fa_stride * esz;
  // forms with skeleton terms (discontinuous-Galerkin skeletons touch most
  // facets) keep a slot for every facet up to 48 GiB
  const size_t fa_budget = f->desc.nskel > 0 ? ((size_t)48 << 30) : ((size_t)4 << 30);
  f->cap_fa = fa_bytes <= fa_budget ? m->nfacets : std::max<int64_t>(m->nfacets / 4, 1);
  int64_t maxw = std::max(f->nw32_el, std::max(f->nw32_fa, f->nw32_dof));
  f->nbsum = (int)((maxw + kCChunk - 1) / kCChunk) + 1;
  f->nbsum64 = (int)((space->ndof + kSChunk - 1) / kSChunk) + 1;
  // scatter buffers sized by the widest row of the full pattern (probed on the
  // GPU below, after the workspace exists)
  std::vector<int64_t> full_ptr;
  auto A = [&](void** p, size_t bytes) { return cudaMalloc(p, bytes ? bytes : 16); };
  cudaError_t e = cudaSuccess;
  e = e ? e : A((void**)&f->d_act_un, f->nw32_el * 4);
  e = e ? e : A((void**)&f->d_act_cut, f->nw32_el * 4);
  e = e ? e : A((void**)&f->d_act_fa, f->nw32_fa * 4);
  e = e ? e : A((void**)&f->d_dof_bits, f->nw32_dof * 4);
  e = e ? e : A((void**)&f->d_l_un, (size_t)m->ne * 4);
  e = e ? e : A((void**)&f->d_l_cut, (size_t)m->ne * 4);
  e = e ? e : A((void**)&f->d_l_fa, (size_t)m->nfacets * 4);
  e = e ? e : A((void**)&f->d_cutlist, ((size_t)m->ne + 1) * 4);
  e = e ? e : A((void**)&f->d_dof_flag, (size_t)space->ndof);
  e = e ? e : A((void**)&f->d_el_slot, (size_t)m->ne * 4);
  e = e ? e : A((void**)&f->d_fa_slot, (size_t)m->nfacets * 4);
  e = e ? e : A((void**)&f->d_dof_row, (size_t)space->ndof * 4);
  e = e ? e : A((void**)&f->d_rowcnt, (size_t)space->ndof * 8);
  e = e ? e : A((void**)&f->d_counts, 8 * sizeof(int));
  e = e ? e : A((void**)&f->d_bsum, (size_t)f->nbsum * 4);
  e = e ? e : A((void**)&f->d_bsum64, (size_t)f->nbsum64 * 8);
  e = e ? e : A(&f->d_elmat, (size_t)f->cap_el * nd * nd * esz);
  e = e ? e : A(&f->d_famat, f->has_patch ? (size_t)f->cap_fa * fa_stride * esz : 16);
  e = e ? e : A(&f->d_pgeo, f->has_patch ? (size_t)f->cap_fa * sizeof(PaGeoS<3, double>) : 16);
  // cut elements beyond this capacity set themselves up inside the element kernel
  f->cap_cgeo = std::min<int64_t>(m->ne, std::max<int64_t>(65536, m->ne / 8));
  // test hook: a smaller cut workspace sends the remaining cut elements through
  // the quadrature-point kernel
  if (const char* cap_env = std::getenv("XG_CUT_WORKSPACE")) {
    const long long v = std::atoll(cap_env);
    if (v > 0) f->cap_cgeo = std::min<int64_t>(f->cap_cgeo, v);
  }
  e = e ? e : A(&f->d_cgeo, (size_t)f->cap_cgeo * sizeof(CutGeoS));
  e = e ? e : A(&f->d_csub, (size_t)f->cap_cgeo * sizeof(CutSubS));
  f->mu_MT = std::max(f->md.MT, 1);
  e = e ? e : A(&f->d_mu, (size_t)f->cap_cgeo * f->mu_MT * esz);
  e = e ? e : A((void**)&f->d_err, sizeof(int));
  e = e ? e : A((void**)&f->d_dom, (size_t)m->ne);
  e = e ? e : A((void**)&f->d_ratio, (size_t)m->ne * 8);
  e = e ? e : A((void**)&f->d_bits, (size_t)8 * (f->nw32_el / 2) * 8);
  e = e ? e : A((void**)&f->d_fbits, (size_t)(f->nw32_fa / 2) * 8);
  // CutFEM step: the skeleton facet sets (HASNEG | HASNEG, HASPOS | HASPOS)
  e = e ? e : A((void**)&f->d_fbits_sk, f->desc.nskel ? (size_t)2 * (f->nw32_fa / 2) * 8 : 16);
  if (e == cudaSuccess) e = cudaMemset(f->d_err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(f->d_dof_flag, 0, (size_t)space->ndof);
  if (e == cudaSuccess) e = cudaMemset(f->d_counts, 0, 8 * sizeof(int));
  if (e != cudaSuccess) return cuda_fail(e, "xg_form_create");
  int pst = full_pattern_probe(f, full_ptr);
  if (pst == XG_ERR_CAPACITY) {
    cudaMemset(f->d_err, 0, sizeof(int));
    full_pattern_stats(f, &f->full_nnz, &f->max_unique, full_ptr);  // very wide rows: exact host count
  } else if (pst) {
    return pst;
  }
  {
    int maxu = 32;
    while (maxu < f->max_unique) maxu <<= 1;
    f->sc_maxu = maxu;
    f->sc_hs = 2 * maxu;
    f->sc_stage = nd * std::max(1, 192 / nd);
    f->sc_wbytes = (row_smem_bytes(f->sc_hs, f->sc_maxu, 0, 0) + 15) & ~15;
    f->sc_smem = (size_t)kRowWarps * f->sc_wbytes;
  }
  e = A((void**)&f->d_full_ptr, (size_t)(space->ndof + 1) * 8);
  e = e ? e : A((void**)&f->d_tmp_cols, (size_t)f->full_nnz * 4);
  if (e == cudaSuccess)
    e = cudaMemcpy(f->d_full_ptr, full_ptr.data(), (size_t)(space->ndof + 1) * 8, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "xg_form_create");
  {
    // the attribute is an upper bound shared by all forms: only ever raise it
    static std::mutex mu;
    static size_t raised = 48 * 1024;
    std::lock_guard<std::mutex> lock(mu);
    if (f->sc_smem > raised) {
      if (cudaFuncSetAttribute(k_row_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f->sc_smem)) {
        set_last_error("xg_form_create: scatter shared memory too large for this mesh");
        return XG_ERR_CAPACITY;
      }
      raised = f->sc_smem;
    }
  }
  f->grid_sc = grid_for(k_row_count, kRowWarps * 32, f->sc_smem);
  // per-step scatter kernels, each with its own shared layout: the marking pass
  // holds the full row's columns and its flags (in the hash region, maxu
  // bytes), the summing pass the accumulators and the staged values
  f->sm_wbytes = (row_smem_bytes(0, 0, f->sc_maxu, f->sc_stage) + 15) & ~15;
  f->sm_smem = (size_t)kRowWarps * f->sm_wbytes;
  {
    static std::mutex mu;
    static size_t raised_sm = 48 * 1024;
    std::lock_guard<std::mutex> lock(mu);
    bool bad = false;
    if (f->sm_smem > raised_sm) {
      const int sm = (int)f->sm_smem;
      const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
      bad |= cudaFuncSetAttribute(k_row_sum<double, false, false, 4>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<double, true, false, 4>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<double, false, true, 4>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<float, false, false, 4>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<float, true, false, 4>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<float, false, true, 4>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<double, false, false, 6>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<double, true, false, 6>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<double, false, true, 6>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<float, false, false, 6>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<float, true, false, 6>, at, sm) != 0;
      bad |= cudaFuncSetAttribute(k_row_sum<float, false, true, 6>, at, sm) != 0;
      raised_sm = f->sm_smem;
    }
    if (bad) {
      set_last_error("xg_form_create: scatter shared memory too large for this mesh");
      return XG_ERR_CAPACITY;
    }
  }
  f->grid_sm = grid_for(k_row_sum<double, false, false, 4>, kRowWarps * 32, f->sm_smem);
  if (f->rows) {
    const int64_t ndof = space->ndof, ncand = (int64_t)m->ne * nd * (m->dim + 1);
    f->rows_W = (f->max_unique + 31) / 32;
    f->rows_copies = std::min(4, std::max(1, 32 / nd));
    f->nbsum_rows = (int)((ndof + 2047) / 2048) + 2;
    e = A((void**)&f->d_el_rowslot, (size_t)m->ne * nd * 4);
    e = e ? e : A((void**)&f->d_nbpos, f->has_patch ? (size_t)ncand * nd * 2 : 16);
    e = e ? e : A((void**)&f->d_cand_fs, f->has_patch ? (size_t)ncand * 4 : 16);
    e = e ? e : A((void**)&f->d_act_slot, (size_t)m->ne * nd);
    // compaction scratch by full-pattern offset while it stays modest; larger
    // forms count their rows first and sum straight into the output
    double budget = kRowsScratchBytes;
    // test hook: a smaller budget sends the form through the direct path
    if (const char* sb = std::getenv("XG_ROWS_SCRATCH_BYTES")) budget = std::atof(sb);
    if ((double)f->full_nnz * 12.0 <= budget) {
      e = e ? e : A((void**)&f->d_vcols, (size_t)f->full_nnz * 4);
      e = e ? e : A((void**)&f->d_vvals, (size_t)f->full_nnz * 8);
    }
    e = e ? e : A((void**)&f->d_bsum_rows, (size_t)f->nbsum_rows * 8);
    if (e == cudaSuccess) e = cudaMemset(f->d_act_slot, 0, (size_t)m->ne * nd);
    if (e != cudaSuccess) return cuda_fail(e, "xg_form_create");
    const RowsArgs R = rows_args(f, nullptr);
    f->rows_smem = rows_accum_smem(R);
    f->rows_grid = std::min(rows_accum_grid(R, true, f->rows_smem), rows_accum_grid(R, false, f->rows_smem));
    if (!f->rows_grid) {
      set_last_error("xg_form_create: row-pass shared memory too large for this mesh");
      return XG_ERR_CAPACITY;
    }
  }
  return full_pattern_build(f);
}

}  // namespace

extern "C" {

int xg_form_destroy(xg_form* f) {
  if (!f) return XG_OK;
  return form_free(f);
}

int xg_form_set_defined_on(xg_form* f, int32_t t, const uint64_t* d_defined_on) {
  if (!f || t < 0 || t >= (int)f->terms.size()) return XG_ERR_ARG;
  f->terms[t].d_defined_on = d_defined_on;
  int st = build_desc(f);
  return st ? st : upload_tables(f);
}

int xg_form_set_bnd_terms(xg_form* f, const xg_bterm* terms, int32_t nterms) {
  if (!f || nterms < 0 || (nterms > 0 && !terms)) return XG_ERR_ARG;
  if (nterms > kMaxBnd) {
    set_last_error("xg_form_set_bnd_terms: at most 8 boundary terms");
    return XG_ERR_CAPACITY;
  }
  xg_mesh* m = f->mesh;
  if (nterms > 0 && (!f->rows || f->ml || m->tensor)) {
    set_last_error("xg_form_set_bnd_terms: boundary terms need a spatial form on a simplex mesh");
    return XG_ERR_UNSUPPORTED;
  }
  BndDesc d = {};
  for (int t = 0; t < nterms; t++) {
    const xg_bterm& T = terms[t];
    if (T.kind != XG_TERM_MASS || (T.domain != XG_NEG && T.domain != XG_POS && T.domain != XG_IF) ||
        T.order > kMaxOrder) {
      set_last_error("xg_form_set_bnd_terms: mass terms on NEG, POS or IF of order <= 8");
      return XG_ERR_ARG;
    }
    if (T.domain == XG_IF && m->dim == 3) {
      set_last_error("xg_form_set_bnd_terms: IF on boundary triangles (3D) is not supported");
      return XG_ERR_UNSUPPORTED;
    }
    BndTermDev& B = d.t[d.n++];
    B.domain = T.domain;
    B.order = T.order >= 0 ? T.order : 2 * f->space->order;
    B.hpow = T.hpow;
    B.coef = T.coef;
    B.defined_on = T.d_defined_on;
  }
  if (nterms > 0 && !f->d_own && m->nbnd > 0) {
    // owners ascending, their BND elements ascending (the boundary facets in
    // facet order; the owner is the facet's first element)
    const int64_t nb = m->nbnd;
    std::vector<int32_t> cnt(m->ne, 0);
    for (int64_t b = 0; b < nb; b++) cnt[m->h_facet_els[2 * (int64_t)m->h_bnd_facets[b]]]++;
    std::vector<int32_t> own, ptr(1, 0), pos(m->ne, -1);
    for (int e = 0; e < m->ne; e++)
      if (cnt[e]) {
        pos[e] = ptr.back();
        own.push_back(e);
        ptr.push_back(ptr.back() + cnt[e]);
      }
    std::vector<int32_t> lst(nb);
    for (int64_t b = 0; b < nb; b++) lst[pos[m->h_facet_els[2 * (int64_t)m->h_bnd_facets[b]]]++] = (int32_t)b;
    const int no = (int)own.size();
    std::vector<int32_t> h(own);
    h.insert(h.end(), ptr.begin(), ptr.end());
    h.insert(h.end(), lst.begin(), lst.end());
    XG_CUDA(cudaSetDevice(m->device));
    XG_CUDA(cudaMalloc((void**)&f->d_own, h.size() * sizeof(int32_t)));
    XG_CUDA(cudaMemcpy(f->d_own, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    f->n_own = no;
  }
  f->bnd = d;
  return XG_OK;
}

int xg_form_set_coef_terms(xg_form* f, const xg_cterm* terms, int32_t nterms) {
  if (!f || nterms < 0 || (nterms > 0 && !terms)) return XG_ERR_ARG;
  if (nterms > kMaxCoef) {
    set_last_error("xg_form_set_coef_terms: at most 8 coefficient terms");
    return XG_ERR_CAPACITY;
  }
  xg_mesh* m = f->mesh;
  if (nterms > 0 && (!f->rows || f->ml || m->tensor)) {
    set_last_error("xg_form_set_coef_terms: coefficient terms need a spatial form on a simplex mesh");
    return XG_ERR_UNSUPPORTED;
  }
  CoefDesc d = {};
  for (int t = 0; t < nterms; t++) {
    const xg_cterm& T = terms[t];
    const bool kind_ok = T.kind == XG_TERM_MASS || T.kind == XG_TERM_LAPLACE || T.kind == XG_TERM_NGRADU_V ||
                         T.kind == XG_TERM_U_NGRADV || T.kind == XG_TERM_CONV || T.kind == XG_TERM_NGRADU_NGRADV;
    if (!kind_ok || (T.domain != XG_NEG && T.domain != XG_POS && T.domain != XG_IF && T.domain != XG_WHOLE) ||
        T.order > kMaxOrder || T.e[0] < 0 || T.e[1] < 0 || T.e[2] < 0) {
      set_last_error("xg_form_set_coef_terms: kinds MASS, LAPLACE, NGRADU_V, U_NGRADV, CONV, NGRADU_NGRADV on NEG, "
                     "POS, IF or WHOLE, order <= 8, exponents >= 0");
      return XG_ERR_ARG;
    }
    const xg_space* g = T.gf_space;
    if (g && (!T.d_gf || g->mesh != m || g->kt >= 0 || g->ndof != g->ndof_s || g->order < 1 || g->order > 3 ||
              g->nd != ndof_el(m->dim, g->order))) {
      set_last_error("xg_form_set_coef_terms: the coefficient is a GridFunction of an H1 space of order 1..3 "
                     "on the form's mesh");
      return XG_ERR_ARG;
    }
    CoefTermDev& C = d.t[d.n++];
    C.kind = T.kind;
    C.domain = T.domain;
    C.order = T.order >= 0 ? T.order : default_order(T.kind, f->space->order);
    C.hpow = T.hpow;
    C.coef = T.coef;
    for (int k = 0; k < 3; k++) {
      C.b[k] = T.b[k];
      C.e[k] = T.e[k];
    }
    C.gf_order = g ? g->order : 0;
    C.gf_dofs = g ? g->d_el_dofs : nullptr;
    C.gf = g ? T.d_gf : nullptr;
    C.defined_on = T.d_defined_on;
    C.gdef = T.d_deform;
  }
  f->cdesc = d;
  return XG_OK;
}

int xg_form_set_deformation(xg_form* f, const double* d_gdef) {
  if (!f) return XG_ERR_ARG;
  if (d_gdef && (!f->rows || f->ml || f->mesh->tensor)) {
    set_last_error("xg_form_set_deformation: spatial forms on simplex meshes");
    return XG_ERR_UNSUPPORTED;
  }
  f->d_patch_deform = d_gdef;
  return XG_OK;
}

int xg_form_capacity(const xg_form* f, int64_t* o) {
  if (!f || !o) return XG_ERR_ARG;
  // the largest pattern any level set can produce on this mesh (every element
  // and every interior facet active), computed at creation
  o[0] = f->space->ndof;
  o[1] = f->full_nnz;
  return XG_OK;
}

int xg_form_check(xg_form* f) {
  if (!f) return XG_ERR_ARG;
  int h = 0;
  XG_CUDA(cudaMemcpy(&h, f->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  XG_CUDA(cudaMemset(f->d_err, 0, sizeof(int)));
  if (h) set_last_error(std::string("device error: ") + xg_status_string(h));
  return h;
}

}  // extern "C"

namespace {
int rows_front(xg_form* f, const double* d_lset, const uint8_t* d_dom, xg_csr* out, cudaStream_t s);
int rows_front_facets(xg_form* f, const double* d_lset, cudaStream_t s);
int rows_back(xg_form* f, xg_csr* out, cudaStream_t s);
int assemble_front(xg_form* f, const double* d_lset, const uint8_t* d_dom, xg_csr* out, void* stream);
}  // namespace

extern "C" {

int xg_form_assemble(xg_form* f, const double* d_lset, const uint8_t* d_dom, xg_csr* out, void* stream) {
  if (!out || !out->d_row_dof || !out->d_rowptr || !out->d_cols || !out->d_vals || !out->d_counts) return XG_ERR_ARG;
  if (f && f->ml) {
    set_last_error("xg_form_assemble: forms on several level sets take xg_mlset_form_assemble");
    return XG_ERR_ARG;
  }
  int st = assemble_front(f, d_lset, d_dom, out, stream);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  return f->rows ? rows_back(f, out, s) : scatter_phase(f, out, s);
}

}  // extern "C"

namespace {

// skeleton terms of the active facets, after the facet-patch terms (which
// write the facet matrices; without them this kernel writes)
int launch_skel(xg_form* f, const double* d_lset, cudaStream_t s) {
  xg_mesh* m = f->mesh;
  SkelLaunch A;
  A.dim = m->dim;
  A.order = f->space->order;
  A.ne = m->ne;
  A.nv = m->nv;
  A.elv = m->d_elv;
  A.xyz = m->d_xyz;
  A.nf = m->nfacets;
  A.fel = m->d_facet_els;
  A.lset = d_lset;
  A.l_fa = f->d_l_fa;
  A.counts = f->d_counts;
  A.famat = f->d_famat;
  A.cap_fa = f->cap_fa;
  A.accumulate = f->desc.npatch > 0 ? 1 : 0;
  A.fp64 = f->precision == XG_PREC_FP64 ? 1 : 0;
  A.err = f->d_err;
  return skel_launch(A, f->desc, s);
}

// boundary terms: the owners of BND elements and their element rows
BndFormLaunch bnd_args(xg_form* f, const double* d_lset) {
  xg_mesh* m = f->mesh;
  BndFormLaunch L;
  L.dim = m->dim;
  L.order = f->space->order;
  L.ne = m->ne;
  L.nv = m->nv;
  L.elv = m->d_elv;
  L.xyz = m->d_xyz;
  L.lset = d_lset;
  L.nbnd = m->nbnd;
  L.bnd_v = m->d_bnd_v;
  L.n_own = f->n_own;
  L.own_el = f->d_own;
  L.own_ptr = f->d_own + f->n_own;
  L.own_bnd = f->d_own + 2 * f->n_own + 1;
  L.d = f->bnd;
  L.act_un = f->d_act_un;
  L.act_cut = f->d_act_cut;
  L.rowslot = f->d_el_rowslot;
  L.elmat = f->d_elmat;
  L.fp64 = f->precision == XG_PREC_FP64 ? 1 : 0;
  L.err = f->d_err;
  return L;
}

// coefficient terms: their active elements and their element rows
CoefFormLaunch coef_args(xg_form* f, const double* d_lset, const uint8_t* d_dom) {
  xg_mesh* m = f->mesh;
  CoefFormLaunch L;
  L.dim = m->dim;
  L.order = f->space->order;
  L.ne = m->ne;
  L.nv = m->nv;
  L.elv = m->d_elv;
  L.xyz = m->d_xyz;
  L.el_edges = m->d_el_edges;
  L.lset = d_lset;
  L.dom = d_dom;
  L.d = f->cdesc;
  L.act_un = f->d_act_un;
  L.act_cut = f->d_act_cut;
  L.nw32 = f->nw32_el;
  L.l_un = f->d_l_un;
  L.l_cut = f->d_l_cut;
  L.counts = f->d_counts;
  L.rowslot = f->d_el_rowslot;
  L.elmat = f->d_elmat;
  L.fp64 = f->precision == XG_PREC_FP64 ? 1 : 0;
  L.err = f->d_err;
  return L;
}

// the element and patch kernels of one step (spatial forms: the element rows
// at their static slots and the patch matrices by facet slot; the patch
// matrices are left out when the form's patches run in a batched launch)
int rows_front(xg_form* f, const double* d_lset, const uint8_t* d_dom, xg_csr* out, cudaStream_t s) {
  const bool fp64 = f->precision == XG_PREC_FP64;
  int st;
  // the facet kernels (patch, skeleton) write the facet matrices, the element
  // kernels the element rows: without stage events they run on a second
  // stream of the form, forked from and joined back into s (in a captured
  // step they become concurrent branches of the graph)
  const bool fork = !f->use_ev && f->has_patch && (f->desc.npatch > 0 || f->desc.nskel > 0);
  f->rows_marked = false;
  cudaStream_t sf = s;
  if (fork) {
    if (!f->side) {
      XG_CUDA(cudaStreamCreateWithFlags(&f->side, cudaStreamNonBlocking));
      XG_CUDA(cudaEventCreateWithFlags(&f->ev_fork, cudaEventDisableTiming));
      XG_CUDA(cudaEventCreateWithFlags(&f->ev_join, cudaEventDisableTiming));
    }
    XG_CUDA(cudaEventRecord(f->ev_fork, s));
    XG_CUDA(cudaStreamWaitEvent(f->side, f->ev_fork, 0));
    sf = f->side;
    if ((st = rows_front_facets(f, d_lset, sf))) return st;
  }
  if ((st = fp64 ? dispatch_volume<double>(f, d_lset, d_dom, s) : dispatch_volume<float>(f, d_lset, d_dom, s)))
    return st;
  if (f->bnd.n > 0 && (st = bnd_elmat_launch(bnd_args(f, d_lset), s))) return st;
  if (f->cdesc.n > 0 && (st = coef_elmat_launch(coef_args(f, d_lset, d_dom), s))) return st;
  if (fork) {
    // the active rows need only the lists: they are marked while the facet
    // kernels run (rows_back then skips this pass)
    if ((st = mark_rows(f, out, s))) return st;
    f->rows_marked = true;
    XG_CUDA(cudaEventRecord(f->ev_join, sf));
    XG_CUDA(cudaStreamWaitEvent(s, f->ev_join, 0));
  } else if ((st = rows_front_facets(f, d_lset, s))) {
    return st;
  }
  if (f->use_ev) cudaEventRecord(f->ev[5], s);
  return XG_OK;
}

// the facet kernels of one step: the patch matrices (affine: the basis-change
// or quadrature kernels; deformed: k_patch_def), then the skeleton terms
int rows_front_facets(xg_form* f, const double* d_lset, cudaStream_t s) {
  const bool fp64 = f->precision == XG_PREC_FP64;
  int st;
  if (f->has_patch && f->desc.npatch > 0) {
    if (f->d_patch_deform) {
      xg_mesh* m = f->mesh;
      PatchDefLaunch P;
      P.dim = m->dim;
      P.order = f->space->order;
      P.ne = m->ne;
      P.nv = m->nv;
      P.elv = m->d_elv;
      P.xyz = m->d_xyz;
      P.el_edges = m->d_el_edges;
      P.gdef = f->d_patch_deform;
      P.nf = m->nfacets;
      P.fel = m->d_facet_els;
      P.l_fa = f->d_l_fa;
      P.counts = f->d_counts;
      P.npatch = f->desc.npatch;
      for (int q = 0; q < kMaxPatch; q++) P.p[q] = f->desc.p[q];
      P.famat = f->d_famat;
      P.cap_fa = f->cap_fa;
      P.fp64 = fp64 ? 1 : 0;
      P.err = f->d_err;
      if ((st = patch_def_launch(P, s))) return st;
    } else if ((st = fp64 ? dispatch_patch<double>(f, s) : dispatch_patch<float>(f, s))) {
      return st;
    }
  }
  if (f->desc.nskel > 0 && (st = launch_skel(f, d_lset, s))) return st;
  return XG_OK;
}

// active rows, then the fixed-order row sums and the compressed output
int rows_back(xg_form* f, xg_csr* out, cudaStream_t s) {
  int st;
  if (!f->rows_marked && (st = mark_rows(f, out, s))) return st;
  f->rows_marked = false;
  if (f->use_ev) cudaEventRecord(f->ev[6], s);
  st = rows_scatter(rows_args(f, out->d_row_dof), f->space->ndof, f->has_patch, f->precision == XG_PREC_FP64,
                    f->d_elmat, f->d_famat, out->d_rowptr, out->d_counts, out->d_cols, out->d_vals, out->cap_nnz,
                    f->rows_grid, f->rows_smem, s);
  if (f->use_ev) cudaEventRecord(f->ev[7], s);
  return st;
}

// checks, active sets and lists, and (spatial forms) the element and patch
// kernels; space-time-shaped forms also their element and patch matrices
int assemble_front(xg_form* f, const double* d_lset, const uint8_t* d_dom, xg_csr* out, void* stream) {
  if (!f || !d_lset || !d_dom || !out || !out->d_row_dof || !out->d_rowptr || !out->d_cols || !out->d_vals ||
      !out->d_counts)
    return XG_ERR_ARG;
  if (out->cap_rows < f->space->ndof) {
    set_last_error("xg_form_assemble: cap_rows below ndof");
    return XG_ERR_CAPACITY;
  }
  cudaStream_t s = (cudaStream_t)stream;
  xg_mesh* m = f->mesh;
  int st;
  // 1. active elements / facets and their lists
  k_active_elements<<<(unsigned)((f->nw32_el * 32 + 255) / 256), 256, 0, s>>>(m->ne, d_dom, f->desc, f->d_act_un,
                                                                              f->d_act_cut, f->nw32_el);
  if (f->bnd.n > 0 && (st = bnd_active_launch(bnd_args(f, d_lset), s))) return st;
  if (f->cdesc.n > 0 && (st = coef_active_launch(coef_args(f, d_lset, d_dom), s))) return st;
  if ((st = compact(f, f->d_act_un, f->nw32_el, f->d_l_un, f->d_el_slot, f->d_counts + 0, s))) return st;
  if ((st = compact(f, f->d_act_cut, f->nw32_el, f->d_l_cut, f->d_el_slot, f->d_counts + 1, s, f->d_counts + 0)))
    return st;
  if (f->has_patch) {
    k_active_facets<<<(unsigned)((f->nw32_fa * 32 + 255) / 256), 256, 0, s>>>(m->nfacets, m->d_facet_els, f->desc,
                                                                              f->d_act_fa, f->nw32_fa);
    if ((st = compact(f, f->d_act_fa, f->nw32_fa, f->d_l_fa, f->d_fa_slot, f->d_counts + 2, s))) return st;
  } else {
    XG_CUDA(cudaMemsetAsync(f->d_act_fa, 0, f->nw32_fa * 4, s));
    XG_CUDA(cudaMemsetAsync(f->d_counts + 2, 0, sizeof(int), s));
  }
  if (f->use_ev) cudaEventRecord(f->ev[2], s);
  if (f->rows) return rows_front(f, d_lset, d_dom, out, s);
  // 2. element and patch matrices (the cut list's slots follow the uncut list's)
  if (f->precision == XG_PREC_FP64) {
    if ((st = dispatch_volume<double>(f, d_lset, d_dom, s))) return st;
    if (f->has_patch && (st = dispatch_patch<double>(f, s))) return st;
  } else {
    if ((st = dispatch_volume<float>(f, d_lset, d_dom, s))) return st;
    if (f->has_patch && (st = dispatch_patch<float>(f, s))) return st;
  }
  if (f->use_ev) cudaEventRecord(f->ev[5], s);
  return XG_OK;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {
// marking, the form's effective element / facet sets, and the front of the
// assembly (up to the element and patch kernels)
int cutfem_front(xg_form* f, const double* d_lset, xg_csr* out, void* stream) {
  if (!f || !d_lset || !out) return XG_ERR_ARG;
  xg_mesh* m = f->mesh;
  if (f->use_ev) cudaEventRecord(f->ev[0], (cudaStream_t)stream);
  int st = cutinfo_update_ws(m, d_lset, f->d_dom, f->d_ratio, f->d_bits, f->d_cutlist, stream);
  if (st) return st;
  const int64_t nw = f->nw32_el / 2;
  const uint64_t* hasneg = f->d_bits + XG_CDOM_HASNEG * nw;
  const uint64_t* ifb = f->d_bits + XG_CDOM_IF * nw;
  const uint64_t* haspos = f->d_bits + XG_CDOM_HASPOS * nw;
  if (f->has_patch) {
    st = xg_facets_with_neighbor_types(m, hasneg, ifb, 1, 1, 1, f->d_fbits, stream);
    if (st) return st;
  }
  uint64_t* fb_neg = f->d_fbits_sk;
  uint64_t* fb_pos = f->d_fbits_sk + f->nw32_fa / 2;
  bool sk_neg = false, sk_pos = false;
  for (int q = 0; q < f->desc.nskel; q++) {
    sk_neg |= f->desc.s[q].region == XG_NEG;
    sk_pos |= f->desc.s[q].region == XG_POS;
  }
  if (sk_neg && (st = xg_facets_with_neighbor_types(m, hasneg, hasneg, 1, 1, 1, fb_neg, stream))) return st;
  if (sk_pos && (st = xg_facets_with_neighbor_types(m, haspos, haspos, 1, 1, 1, fb_pos, stream))) return st;
  // effective element / facet sets of the CutFEM form
  FormDesc saved = f->desc;
  for (int q = 0; q < f->desc.ngroups; q++) {
    GroupDesc& G = f->desc.g[q];
    G.defined_on = G.domain == XG_NEG ? hasneg : (G.domain == XG_IF ? ifb : haspos);
  }
  for (int p = 0; p < f->desc.npatch; p++) f->desc.p[p].defined_on = f->d_fbits;
  // skeleton terms (demos/fictdom_dg.py:100-135): facets inside the domain's
  // elements, whole-facet terms on the ghost facets
  for (int q = 0; q < f->desc.nskel; q++) {
    SkelDesc& S = f->desc.s[q];
    S.defined_on = S.region == XG_NEG ? fb_neg : (S.region == XG_POS ? fb_pos : f->d_fbits);
  }
  if (f->use_ev) cudaEventRecord(f->ev[1], (cudaStream_t)stream);
  st = assemble_front(f, d_lset, f->d_dom, out, stream);
  f->desc = saved;
  return st;
}

}  // namespace

extern "C" {

int xg_cutfem_step(xg_form* f, const double* d_lset, xg_csr* out, void* stream) {
  if (!f || !d_lset || !out) return XG_ERR_ARG;
  if (f->ml) {
    set_last_error("xg_cutfem_step: forms on several level sets take xg_mlset_form_assemble");
    return XG_ERR_ARG;
  }
  int st = cutfem_front(f, d_lset, out, stream);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  return f->rows ? rows_back(f, out, s) : scatter_phase(f, out, s);
}

int xg_form_stage_events(xg_form* f, void* const* events, int n) {
  if (!f || (n != 0 && n != 8) || (n == 8 && !events)) return XG_ERR_ARG;
  f->use_ev = n == 8;
  for (int i = 0; i < 8; i++) f->ev[i] = n == 8 ? (cudaEvent_t)events[i] : nullptr;
  return XG_OK;
}

int xg_st_form_create(xg_space* space, int kt_lset, int order_time, const xg_st_term* terms, int32_t nterms,
                      int precision, xg_form** out) {
  if (!space || !out || space->kt < 1 || space->kt > 2 || space->order > 2 || kt_lset < 0 || kt_lset > 2 ||
      order_time < 0 || order_time > 7 || (nterms > 0 && !terms) || nterms < 0 ||
      (precision != XG_PREC_FP64 && precision != XG_PREC_MIXED)) {
    set_last_error("xg_st_form_create: space-time space of space order 1..2 and time order 1..2, level set time "
                   "order 0..2, time rule order 0..7");
    return XG_ERR_ARG;
  }
  *out = nullptr;
  auto* f = new xg_form();
  f->space = space;
  f->mesh = space->mesh;
  f->precision = precision;
  f->st = true;
  f->st_terms.assign(terms, terms + nterms);
  std::memset(&f->desc, 0, sizeof(f->desc));
  StFormDesc& d = f->stdesc;
  std::memset(&d, 0, sizeof(d));
  d.kt_l = kt_lset;
  d.order_time = order_time;
  const int k = space->order;
  for (int t = 0; t < nterms; t++) {
    const xg_st_term& T = terms[t];
    const xg_term& B = T.base;
    if (B.kind == XG_TERM_GHOST_MASS) {
      if (f->desc.npatch >= kMaxPatch) {
        form_free(f);
        return XG_ERR_UNSUPPORTED;
      }
      PatchDesc& P = f->desc.p[f->desc.npatch++];
      P.order = B.order >= 0 ? B.order : 2 * k;
      P.defined_on = B.d_defined_on;
      P.c = B.coef;
      P.hpow = B.hpow;
      f->has_patch = true;
      continue;
    }
    if (!(B.kind == XG_TERM_MASS || B.kind == XG_TERM_LAPLACE || B.kind == XG_TERM_CONV || B.kind == XG_TERM_DT_U_V) ||
        B.domain < 0 || B.domain > 2) {
      form_free(f);
      set_last_error("xg_st_form_create: space-time terms are MASS, LAPLACE, CONV, DT_U_V and GHOST_MASS");
      return XG_ERR_UNSUPPORTED;
    }
    const int order = B.order >= 0 ? B.order
                                   : (B.kind == XG_TERM_LAPLACE ? 2 * k - 2 : (B.kind == XG_TERM_CONV ? 2 * k - 1 : 2 * k));
    if (order > kMaxOrder) {
      form_free(f);
      return XG_ERR_UNSUPPORTED;
    }
    int g = -1;
    for (int q = 0; q < d.ngroups; q++) {
      const StGroupDesc& G = d.g[q];
      bool same_conv = B.kind != XG_TERM_CONV || !(G.used & (1 << XG_TERM_CONV)) ||
                       (std::memcmp(G.b, B.b, sizeof(G.b)) == 0 && std::memcmp(G.bc, T.bc, sizeof(G.bc)) == 0 &&
                        std::memcmp(G.bs, T.bs, sizeof(G.bs)) == 0 && G.omega == T.omega && G.t0 == T.t0 &&
                        G.dt == T.dt);
      if (G.domain == B.domain && G.order == order && G.defined_on == B.d_defined_on &&
          (G.tref < 0) == (T.tref < 0) && (T.tref < 0 || G.tref == T.tref) && same_conv && !(G.used & (1 << B.kind)))
        g = q;
    }
    if (g < 0) {
      if (d.ngroups >= kMaxGroups) {
        form_free(f);
        set_last_error("xg_st_form_create: too many term groups");
        return XG_ERR_UNSUPPORTED;
      }
      g = d.ngroups++;
      d.g[g].domain = B.domain;
      d.g[g].order = order;
      d.g[g].defined_on = B.d_defined_on;
      d.g[g].tref = T.tref < 0 ? -1.0 : T.tref;
    }
    StGroupDesc& G = d.g[g];
    G.c[B.kind] = B.coef;
    G.hpow[B.kind] = B.hpow;
    G.used |= 1 << B.kind;
    if (B.kind == XG_TERM_CONV) {
      for (int c = 0; c < 3; c++) {
        G.b[c] = B.b[c];
        G.bc[c] = T.bc[c];
        G.bs[c] = T.bs[c];
      }
      G.omega = T.omega;
      G.t0 = T.t0;
      G.dt = T.dt;
    }
  }
  // time mass of the time rule: factor of the space-time facet patches
  {
    const RuleTable& R = host_rules();
    const int p = clamp_order(order_time), kt = space->kt;
    for (int a = 0; a < 9; a++) f->mt[a] = 0.0;
    for (int q = 0; q < R.cnt[1][p]; q++) {
      double psi[3], dpsi[3];
      time_basis<double>(kt, R.x[R.off[1][p] + q][0], psi, dpsi);
      for (int a = 0; a <= kt; a++)
        for (int b = 0; b <= kt; b++) f->mt[a * (kt + 1) + b] += R.w[R.off[1][p] + q] * psi[a] * psi[b];
    }
  }
  f->el_sym = 0;
  int st = st_uncut_tables(f);
  if (!st) st = form_workspace(f);
  if (st) {
    form_free(f);
    return st;
  }
  *out = f;
  return XG_OK;
}

int xg_st_cutfem_step(xg_form* f, const double* d_lset_st, xg_csr* out, void* stream) {
  if (!f || !f->st || !d_lset_st || !out || !out->d_row_dof || !out->d_rowptr || !out->d_cols || !out->d_vals ||
      !out->d_counts)
    return XG_ERR_ARG;
  if (out->cap_rows < f->space->ndof) return XG_ERR_CAPACITY;
  cudaStream_t s = (cudaStream_t)stream;
  xg_mesh* m = f->mesh;
  if (f->use_ev) cudaEventRecord(f->ev[0], s);
  int st = cutinfo_update_st_ws(m, d_lset_st, f->stdesc.kt_l, f->d_dom, f->d_ratio, f->d_bits, f->d_cutlist, stream);
  if (st) return st;
  const int64_t nw = f->nw32_el / 2;
  const uint64_t* hasneg = f->d_bits + XG_CDOM_HASNEG * nw;
  const uint64_t* ifb = f->d_bits + XG_CDOM_IF * nw;
  const uint64_t* haspos = f->d_bits + XG_CDOM_HASPOS * nw;
  if (f->has_patch && (st = xg_facets_with_neighbor_types(m, hasneg, ifb, 1, 1, 1, f->d_fbits, stream))) return st;
  StFormDesc d = f->stdesc;
  for (int q = 0; q < d.ngroups; q++)
    d.g[q].defined_on = d.g[q].domain == XG_NEG ? hasneg : (d.g[q].domain == XG_IF ? ifb : haspos);
  FormDesc pd = f->desc;
  for (int p = 0; p < pd.npatch; p++) pd.p[p].defined_on = f->d_fbits;
  if (f->use_ev) cudaEventRecord(f->ev[1], s);
  // work lists: elements uncut in the slab, then the cut ones (slots after the uncut ones)
  k_active_st<<<(unsigned)((f->nw32_el * 32 + 255) / 256), 256, 0, s>>>(m->ne, f->d_dom, d, f->d_act_un,
                                                                        f->d_act_cut, f->nw32_el);
  if ((st = compact(f, f->d_act_un, f->nw32_el, f->d_l_un, f->d_el_slot, f->d_counts + 0, s))) return st;
  if ((st = compact(f, f->d_act_cut, f->nw32_el, f->d_l_cut, f->d_el_slot, f->d_counts + 1, s, f->d_counts + 0)))
    return st;
  FormDesc saved = f->desc;
  f->desc = pd;
  if (f->has_patch) {
    k_active_facets<<<(unsigned)((f->nw32_fa * 32 + 255) / 256), 256, 0, s>>>(m->nfacets, m->d_facet_els, f->desc,
                                                                              f->d_act_fa, f->nw32_fa);
    st = compact(f, f->d_act_fa, f->nw32_fa, f->d_l_fa, f->d_fa_slot, f->d_counts + 2, s);
  } else {
    cudaMemsetAsync(f->d_act_fa, 0, f->nw32_fa * 4, s);
    cudaMemsetAsync(f->d_counts + 2, 0, sizeof(int), s);
  }
  if (f->use_ev) cudaEventRecord(f->ev[2], s);
  if (!st) {
    StLaunch L;
    L.D = m->dim;
    L.K = f->space->order;
    L.KT = f->space->kt;
    L.precision = f->precision;
    L.ne = m->ne;
    L.nv = m->nv;
    L.elv = m->d_elv;
    L.xyz = m->d_xyz;
    L.lset_st = d_lset_st;
    L.desc = d;
    L.list = f->d_l_cut;
    L.count = f->d_counts + 1;
    L.slot_base = f->d_counts + 0;
    L.elmat = f->d_elmat;
    L.err = f->d_err;
    st = f->precision == XG_PREC_FP64 ? dispatch_st_uncut<double>(f, s) : dispatch_st_uncut<float>(f, s);
    if (f->use_ev) cudaEventRecord(f->ev[3], s);
    if (!st) st = launch_st_elmat(L, s);
  }
  if (f->use_ev) cudaEventRecord(f->ev[4], s);
  if (!st && f->has_patch)
    st = f->precision == XG_PREC_FP64 ? dispatch_patch<double>(f, s) : dispatch_patch<float>(f, s);
  f->desc = saved;
  if (st) return st;
  if (f->use_ev) cudaEventRecord(f->ev[5], s);
  return scatter_phase(f, out, s);
}

int xg_cutfem_marking(xg_form* f, const uint8_t** d_dom, const double** d_ratio, const uint64_t** d_bits,
                      const uint64_t** d_facets) {
  if (!f) return XG_ERR_ARG;
  if (d_dom) *d_dom = f->d_dom;
  if (d_ratio) *d_ratio = f->d_ratio;
  if (d_bits) *d_bits = f->d_bits;
  if (d_facets) *d_facets = f->d_fbits;
  return XG_OK;
}

}  // extern "C"

// ============================================================================
// Autotuner.  Per (device, dimension, order, precision) it times, on the
// caller's form and level set, the launch choices that do not change any
// result bit: elements per block of the uncut element kernel (16 or 32),
// blocks per SM of the basis-change patch kernel (1 .. its occupancy) and
// rows per block (4 or 8 warps) of the row passes; and the row sums'
// accumulator copies (1 .. min(4, 32 / dofs per element)), which fix the
// summation order of the row sums (every configuration is deterministic; the
// chosen one is used for every later step and form of that key).  Each
// choice is the fastest median of three steps of its own stage (CUDA events
// on the launching stream), searched one knob at a time; the table is cached
// per process and applied to forms created afterwards.
// ============================================================================
namespace {

struct TuneRec {
  int uncut_epb = 32, rows_warps = 8, rows_copies = 1, px_bps = 0;
  float ms_uncut = 0, ms_rows = 0, ms_patch = 0;
};
std::mutex g_tune_mu;
std::map<std::string, TuneRec> g_tune;

std::string tune_key(const xg_form* f) {
  int dev = 0;
  cudaGetDevice(&dev);
  return std::to_string(dev) + "/d" + std::to_string(f->mesh->dim) + "/k" + std::to_string(f->space->order) + "/" +
         (f->precision == XG_PREC_FP64 ? "fp64" : "mixed");
}

int apply_tune(xg_form* f, const TuneRec& t) {
  f->tune_uncut_epb = t.uncut_epb;
  f->rows_warps = t.rows_warps;
  f->rows_copies = t.rows_copies;
  const RowsArgs R = rows_args(f, nullptr);
  const size_t smem = rows_accum_smem(R);
  const int grid = rows_accum_grid(R, f->precision == XG_PREC_FP64, smem);
  if (!grid) return XG_ERR_CAPACITY;
  f->rows_smem = smem;
  f->rows_grid = grid;
  if (t.px_bps > 0) f->grid_px = 152 * std::min(t.px_bps, f->px_occ);
  f->px_bps = t.px_bps;
  return XG_OK;
}

int apply_cached_tune(xg_form* f) {
  if (f->st || !f->rows) return XG_OK;
  TuneRec t;
  bool found = false;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(tune_key(f));
    if (it != g_tune.end()) {
      t = it->second;
      found = true;
    }
  }
  return found ? apply_tune(f, t) : XG_OK;
}

}  // namespace

extern "C" {

int xg_form_autotune(xg_form* f, const double* d_lset, xg_csr* out, void* stream) {
  if (!f || !d_lset || !out) return XG_ERR_ARG;
  if (f->st || !f->rows) return XG_OK;  // space-time forms keep their fixed launches
  const std::string key = tune_key(f);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return apply_tune(f, it->second);
  }
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t ev[8];
  for (int i = 0; i < 8; i++)
    if (cudaEventCreate(&ev[i]) != cudaSuccess) {
      for (int k = 0; k < i; k++) cudaEventDestroy(ev[k]);
      return cuda_fail(cudaGetLastError(), "xg_form_autotune");
    }
  const bool use_ev = f->use_ev;
  cudaEvent_t saved_ev[8];
  for (int i = 0; i < 8; i++) {
    saved_ev[i] = f->ev[i];
    f->ev[i] = ev[i];
  }
  f->use_ev = true;
  int st = XG_OK;
  // median time (ms) of stage a -> b over kReps steps
  constexpr int kReps = 5;
  auto stage = [&](int a, int b) -> float {
    float t[kReps];
    for (int r = 0; r < kReps && !st; r++) {
      if ((st = xg_cutfem_step(f, d_lset, out, stream))) break;
      if (cudaStreamSynchronize(s) != cudaSuccess) {
        st = cuda_fail(cudaGetLastError(), "xg_form_autotune");
        break;
      }
      if ((st = xg_form_check(f))) break;
      cudaEventElapsedTime(&t[r], ev[a], ev[b]);
    }
    if (st) return 1e30f;
    std::sort(t, t + kReps);
    return t[kReps / 2];
  };
  // a choice replaces the incumbent only when it is faster by more than 3 %
  // (the medians of different choices differ by noise of about that size)
  constexpr float kGain = 0.97f;
  TuneRec best;
  best.rows_copies = f->rows_copies;
  best.rows_warps = f->rows_warps;
  if ((st = apply_tune(f, best)) == XG_OK) stage(0, 7);  // warm-up
  // uncut elements per block
  if (!st) {
    float bt = 1e30f;
    for (int epb : {32, 16}) {
      TuneRec t = best;
      t.uncut_epb = epb;
      if ((st = apply_tune(f, t))) break;
      const float ms = stage(2, 3);
      if (ms < kGain * bt) {
        bt = ms;
        best.uncut_epb = epb;
        best.ms_uncut = ms;
      }
    }
  }
  // row passes: rows per block, accumulator copies
  if (!st) {
    float bt = 1e30f;
    const int cmax = std::min(4, std::max(1, 32 / f->space->nd));
    // the incumbent (the form's default) first
    std::vector<std::pair<int, int>> cand = {{best.rows_warps, best.rows_copies}};
    for (int w : {4, 8})
      for (int c = 1; c <= cmax; c++)
        if (w != best.rows_warps || c != best.rows_copies) cand.push_back({w, c});
    for (const auto& wc : cand) {
      if (st) break;
      {
        const int w = wc.first, c = wc.second;
        TuneRec t = best;
        t.rows_warps = w;
        t.rows_copies = c;
        if (apply_tune(f, t)) continue;  // shared memory too large for this choice
        const float ms = stage(6, 7);
        if (ms < kGain * bt) {
          bt = ms;
          best.rows_warps = w;
          best.rows_copies = c;
          best.ms_rows = ms;
        }
      }
    }
  }
  // basis-change patch kernel: blocks per SM
  if (!st && f->has_patch && f->patch_exact) {
    float bt = 1e30f;
    // the incumbent (occupancy) first, then fewer blocks per SM
    for (int b = f->px_occ; b >= 1 && !st; b--) {
      TuneRec t = best;
      t.px_bps = b;
      if ((st = apply_tune(f, t))) break;
      const float ms = stage(4, 5);
      if (ms < kGain * bt) {
        bt = ms;
        best.px_bps = b;
        best.ms_patch = ms;
      }
    }
  }
  for (int i = 0; i < 8; i++) {
    f->ev[i] = saved_ev[i];
    cudaEventDestroy(ev[i]);
  }
  f->use_ev = use_ev;
  if (st) return st;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[key] = best;
  }
  return apply_tune(f, best);
}

int64_t xg_autotune_table(char* buf, int64_t cap) {
  std::string j = "{";
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    bool first = true;
    for (const auto& kv : g_tune) {
      const TuneRec& t = kv.second;
      char line[512];
      std::snprintf(line, sizeof(line),
                    "%s\"%s\": {\"uncut_elements_per_block\": %d, \"row_pass_rows_per_block\": %d, "
                    "\"row_pass_accumulator_copies\": %d, \"patch_blocks_per_sm\": %d, \"ms_uncut\": %.4f, "
                    "\"ms_rows\": %.4f, \"ms_patch\": %.4f}",
                    first ? "" : ", ", kv.first.c_str(), t.uncut_epb, t.rows_warps, t.rows_copies, t.px_bps,
                    t.ms_uncut, t.ms_rows, t.ms_patch);
      j += line;
      first = false;
    }
  }
  j += "}";
  if (buf && cap > 0) {
    const int64_t n = std::min<int64_t>(cap - 1, (int64_t)j.size());
    std::memcpy(buf, j.data(), (size_t)n);
    buf[n] = 0;
  }
  return (int64_t)j.size() + 1;
}

}  // extern "C"

struct xg_step_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t kernels = 0;
  int* d_queue = nullptr;  // work counters of the batched patch launches
};

namespace {

// work per item of the basis-change patch kernel (relative): facets per item
// x patch entries x the basis size of the contractions
int64_t px_item_cost(int D, int K) {
  const int N = D == 2 ? (K + 1) * (K + 2) / 2 : (K + 1) * (K + 2) * (K + 3) / 6;
  const int F = N <= 10 ? 32 : 8;
  return (int64_t)F * (2 * N) * (2 * N) * N;
}

// The basis-change patch matrices of several forms (same dimension and
// precision, spatial, kernels deferred by their steps) in one persistent
// launch per kMaxPxJobs forms: jobs ordered by decreasing cost per item.
template <int D, typename T>
int launch_patch_multi_t(std::vector<xg_form*> fs, int* d_queue, cudaStream_t s) {
  std::stable_sort(fs.begin(), fs.end(), [](xg_form* a, xg_form* b) {
    return px_item_cost(D, a->space->order) > px_item_cost(D, b->space->order);
  });
  const void* kern = (const void*)k_patch_exact_multi<D, T>;
  const size_t smem = std::max(sizeof(PxSmem<D, 1, T>), std::max(sizeof(PxSmem<D, 2, T>), sizeof(PxSmem<D, 3, T>)));
  {
    static std::mutex mu;
    static bool raised = false;
    std::lock_guard<std::mutex> lock(mu);
    if (!raised) {
      XG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      raised = true;
    }
  }
  static int grid = 0;
  if (!grid) grid = grid_for(k_patch_exact_multi<D, T>, 256, smem);
  for (size_t c0 = 0; c0 < fs.size(); c0 += kMaxPxJobs) {
    PxJobs<D, T> Q;
    std::memset(&Q, 0, sizeof(Q));
    Q.n = (int)std::min<size_t>(kMaxPxJobs, fs.size() - c0);
    Q.queue = d_queue + c0 / kMaxPxJobs;
    for (int j = 0; j < Q.n; j++) Q.job[j] = px_job<D, T>(fs[c0 + j]);
    XG_CUDA(cudaMemsetAsync(Q.queue, 0, sizeof(int), s));
    void* args[] = {&Q};
    XG_CUDA(cudaLaunchKernel(kern, dim3(grid), dim3(256), args, smem, s));
  }
  return XG_OK;
}

// groups the forms by (dimension, precision); d_queue holds one counter per
// kMaxPxJobs forms of each group (at most forms.size() in all)
int launch_patch_multi(const std::vector<xg_form*>& forms, int* d_queue, cudaStream_t s) {
  int used = 0;
  for (int D = 2; D <= 3; D++)
    for (int fp = 0; fp < 2; fp++) {
      std::vector<xg_form*> g;
      for (xg_form* f : forms)
        if (f->mesh->dim == D && (f->precision == XG_PREC_FP64) == (fp == 1)) g.push_back(f);
      if (g.empty()) continue;
      int st;
      if (D == 2) st = fp ? launch_patch_multi_t<2, double>(g, d_queue + used, s)
                          : launch_patch_multi_t<2, float>(g, d_queue + used, s);
      else st = fp ? launch_patch_multi_t<3, double>(g, d_queue + used, s)
                   : launch_patch_multi_t<3, float>(g, d_queue + used, s);
      if (st) return st;
      used += (int)((g.size() + kMaxPxJobs - 1) / kMaxPxJobs);
    }
  return XG_OK;
}

}  // namespace

extern "C" {

int xg_step_graph_destroy(xg_step_graph* g) {
  if (!g) return XG_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  cudaFree(g->d_queue);
  delete g;
  return XG_OK;
}

int xg_step_graph_create(xg_form* const* forms, const double* const* d_lsets, const xg_csr* outs, int32_t n,
                         xg_step_graph** out) {
  if (!forms || !d_lsets || !outs || !out || n <= 0) return XG_ERR_ARG;
  *out = nullptr;
  // one branch per distinct form; entries of the same form stay in list order
  std::vector<xg_form*> distinct;
  std::vector<int> branch(n);
  for (int i = 0; i < n; i++) {
    if (!forms[i] || !d_lsets[i]) return XG_ERR_ARG;
    auto it = std::find(distinct.begin(), distinct.end(), forms[i]);
    branch[i] = (int)(it - distinct.begin());
    if (it == distinct.end()) distinct.push_back(forms[i]);
  }
  for (size_t a = 0; a < distinct.size(); a++)
    for (size_t b = a + 1; b < distinct.size(); b++)
      for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
          if (forms[i] == distinct[a] && forms[j] == distinct[b] && outs[i].d_vals == outs[j].d_vals) {
            set_last_error("xg_step_graph_create: distinct forms must write distinct outputs");
            return XG_ERR_ARG;
          }
  const int nb = (int)distinct.size();
  // Forms whose patch matrices come from the basis-change kernel share one
  // persistent, work-stealing launch (k_patch_exact_multi) when each form
  // takes one step in the graph: every branch runs its step up to the patch
  // geometry, the batched launch waits for all of them, and every branch's
  // row sums wait for it.
  std::vector<xg_form*> multi;
  if (nb == n)
    for (xg_form* f : distinct)
      if (f->rows && f->has_patch && f->patch_exact && f->desc.npatch > 0 && f->desc.nskel == 0 && !f->d_patch_deform)
        multi.push_back(f);
  if (multi.size() < 2) multi.clear();
  int* d_queue = nullptr;
  if (!multi.empty()) XG_CUDA(cudaMalloc((void**)&d_queue, multi.size() * sizeof(int)));
  std::vector<cudaStream_t> streams(nb, nullptr);
  std::vector<cudaEvent_t> done(nb, nullptr), front(nb, nullptr);
  cudaEvent_t fork = nullptr, batched = nullptr;
  std::vector<xg_csr> o(outs, outs + n);
  std::vector<bool> use_ev(nb);
  auto release = [&]() {
    for (int b = 0; b < nb; b++) {
      if (streams[b]) cudaStreamDestroy(streams[b]);
      if (done[b]) cudaEventDestroy(done[b]);
      if (front[b]) cudaEventDestroy(front[b]);
      distinct[b]->use_ev = use_ev[b];
      distinct[b]->defer_patch = false;
    }
    if (fork) cudaEventDestroy(fork);
    if (batched) cudaEventDestroy(batched);
  };
  cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&batched, cudaEventDisableTiming);
  for (int b = 0; b < nb && e == cudaSuccess; b++) {
    use_ev[b] = distinct[b]->use_ev;
    distinct[b]->use_ev = false;
    e = cudaStreamCreateWithFlags(&streams[b], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&front[b], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    release();
    cudaFree(d_queue);
    return cuda_fail(e, "xg_step_graph_create");
  }
  for (xg_form* f : multi) f->defer_patch = true;
  // capture on branch 0's stream; the others fork from it and join back
  cudaStream_t s0 = streams[0];
  e = cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) e = cudaEventRecord(fork, s0);
  for (int b = 1; b < nb && e == cudaSuccess; b++) e = cudaStreamWaitEvent(streams[b], fork, 0);
  int st = XG_OK;
  if (multi.empty()) {
    for (int i = 0; i < n && e == cudaSuccess && !st; i++) {
      xg_form* f = forms[i];
      void* s = (void*)streams[branch[i]];
      st = f->st ? xg_st_cutfem_step(f, d_lsets[i], &o[i], s) : xg_cutfem_step(f, d_lsets[i], &o[i], s);
    }
  } else {
    // fronts on their branches (entries are distinct forms: entry i is branch i)
    for (int i = 0; i < n && e == cudaSuccess && !st; i++) {
      xg_form* f = forms[i];
      void* s = (void*)streams[branch[i]];
      if (f->st) st = xg_st_cutfem_step(f, d_lsets[i], &o[i], s);
      else if (f->rows) st = cutfem_front(f, d_lsets[i], &o[i], s);
      else st = xg_cutfem_step(f, d_lsets[i], &o[i], s);
    }
    for (int b = 1; b < nb && e == cudaSuccess; b++) {
      e = cudaEventRecord(front[b], streams[b]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s0, front[b], 0);
    }
    if (e == cudaSuccess && !st) st = launch_patch_multi(multi, d_queue, s0);
    if (e == cudaSuccess && !st) e = cudaEventRecord(batched, s0);
    for (int b = 1; b < nb && e == cudaSuccess; b++) e = cudaStreamWaitEvent(streams[b], batched, 0);
    // the row sums of the spatial forms
    for (int i = 0; i < n && e == cudaSuccess && !st; i++) {
      xg_form* f = forms[i];
      if (f->rows && !f->st) st = rows_back(f, &o[i], streams[branch[i]]);
    }
  }
  for (int b = 1; b < nb && e == cudaSuccess; b++) {
    e = cudaEventRecord(done[b], streams[b]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s0, done[b], 0);
  }
  cudaGraph_t graph = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(s0, &graph);
  if (e == cudaSuccess) e = e2;
  auto* g = new xg_step_graph();
  g->graph = graph;
  g->d_queue = d_queue;
  if (e == cudaSuccess && !st) e = cudaGraphInstantiate(&g->exec, graph, 0);
  if (e == cudaSuccess && !st) {
    size_t nn = 0;
    e = cudaGraphGetNodes(graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (e == cudaSuccess && nn) e = cudaGraphGetNodes(graph, nodes.data(), &nn);
    for (size_t k = 0; k < nn && e == cudaSuccess; k++) {
      cudaGraphNodeType t;
      e = cudaGraphNodeGetType(nodes[k], &t);
      if (e == cudaSuccess && t == cudaGraphNodeTypeKernel) g->kernels++;
    }
  }
  release();
  if (st || e != cudaSuccess) {
    xg_step_graph_destroy(g);
    cudaGetLastError();
    return st ? st : cuda_fail(e, "xg_step_graph_create");
  }
  *out = g;
  return XG_OK;
}

int xg_step_graph_kernel_count(const xg_step_graph* g, int64_t* out) {
  if (!g || !out) return XG_ERR_ARG;
  *out = g->kernels;
  return XG_OK;
}

int xg_step_graph_launch(xg_step_graph* g, void* stream) {
  if (!g || !g->exec) return XG_ERR_ARG;
  XG_CUDA(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  return XG_OK;
}

}  // extern "C"

// ============================================================================
// Bilinear forms on regions of several level sets (xg_mlset_form_*): the
// element matrices of the region terms by their multi-level-set rules
// (csrc/xg_mlform.cu), the facet-patch terms and the row scatter of the
// spatial forms.
// ============================================================================
namespace {

// active elements: in the element set of some region term (all without one)
__global__ void k_ml_active(int ne, const MlTermDev* __restrict__ terms, int nterms, uint32_t* bits, int64_t nw32) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool act = false;
  if (e < ne)
    for (int t = 0; t < nterms; t++)
      if (!terms[t].defined_on || tbit(terms[t].defined_on, e)) act = true;
  const unsigned m = __ballot_sync(0xffffffffu, act);
  if ((threadIdx.x & 31) == 0 && (e >> 5) < nw32) bits[e >> 5] = m;
}

}  // namespace

extern "C" {

int xg_mlset_form_create(xg_space* space, int32_t M, const xg_mlterm* terms, int32_t nterms,
                         const xg_term* patch_terms, int32_t npatch, int precision, xg_form** out) {
  if (!space || !out || M < 1 || M > 8 || nterms < 1 || !terms || npatch < 0 || (npatch > 0 && !patch_terms) ||
      (precision != XG_PREC_FP64 && precision != XG_PREC_MIXED)) {
    set_last_error("xg_mlset_form_create: bad arguments (1 <= M <= 8, at least one region term)");
    return XG_ERR_ARG;
  }
  if (space->kt >= 0 || space->mesh->tensor) {
    set_last_error("xg_mlset_form_create: spatial spaces on simplex meshes");
    return XG_ERR_UNSUPPORTED;
  }
  for (int t = 0; t < npatch; t++)
    if (patch_terms[t].kind != XG_TERM_GHOST_MASS) {
      set_last_error("xg_mlset_form_create: the patch terms are XG_TERM_GHOST_MASS");
      return XG_ERR_ARG;
    }
  std::vector<MlTermDev> mt(nterms);
  std::vector<int8_t> tup;
  for (int t = 0; t < nterms; t++) {
    const xg_mlterm& T = terms[t];
    if (T.kind < XG_TERM_MASS || T.kind > XG_TERM_CONV || T.ntup < 1 || T.ntup > 256 || !T.h_tuples ||
        T.normal_lset < 0 || T.normal_lset >= M) {
      set_last_error("xg_mlset_form_create: bad region term (kind MASS..CONV, 1..256 tuples, normal level set)");
      return XG_ERR_ARG;
    }
    const int order = T.order >= 0 ? T.order : default_order(T.kind, space->order);
    if (order > kMaxOrder) {
      set_last_error("xg_mlset_form_create: integration order above 8");
      return XG_ERR_UNSUPPORTED;
    }
    MlTermDev& D = mt[t];
    D.kind = T.kind;
    D.order = order;
    D.hpow = T.hpow;
    D.normal_lset = T.normal_lset;
    D.ntup = T.ntup;
    D.tup_off = (int)tup.size();
    D.coef = T.coef;
    for (int k = 0; k < 3; k++) D.b[k] = T.b[k];
    D.defined_on = T.d_defined_on;
    for (int k = 0; k < T.ntup * M; k++) {
      const int8_t v = T.h_tuples[k];
      if (v != XG_NEG && v != XG_POS && v != XG_IF) {
        set_last_error("xg_mlset_form_create: domain tuples hold XG_NEG / XG_POS / XG_IF");
        return XG_ERR_ARG;
      }
      tup.push_back(v);
    }
  }
  int st = ensure_device_rules();
  if (st) return st;
  *out = nullptr;
  auto* f = new xg_form();
  f->space = space;
  f->mesh = space->mesh;
  f->precision = precision;
  f->terms.assign(patch_terms, patch_terms + npatch);
  f->ml = true;
  f->ml_M = M;
  f->ml_terms = mt;
  st = build_desc(f);
  if (!st) st = upload_tables(f);
  if (!st) st = form_workspace(f);
  if (!st) st = apply_cached_tune(f);
  if (!st) {
    cudaError_t e = cudaMalloc((void**)&f->d_ml_terms, mt.size() * sizeof(MlTermDev));
    if (e == cudaSuccess) e = cudaMalloc((void**)&f->d_ml_tuples, tup.size());
    if (e == cudaSuccess)
      e = cudaMemcpy(f->d_ml_terms, mt.data(), mt.size() * sizeof(MlTermDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(f->d_ml_tuples, tup.data(), tup.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) st = cuda_fail(e, "xg_mlset_form_create");
  }
  if (st) {
    form_free(f);
    return st;
  }
  *out = f;
  return XG_OK;
}

int xg_mlset_form_assemble(xg_form* f, const double* d_lsets, xg_csr* out, void* stream) {
  if (!f || !f->ml || !d_lsets || !out || !out->d_row_dof || !out->d_rowptr || !out->d_cols || !out->d_vals ||
      !out->d_counts)
    return XG_ERR_ARG;
  if (out->cap_rows < f->space->ndof) {
    set_last_error("xg_mlset_form_assemble: cap_rows below ndof");
    return XG_ERR_CAPACITY;
  }
  cudaStream_t s = (cudaStream_t)stream;
  xg_mesh* m = f->mesh;
  int st;
  // active elements (all in the second list) and facets
  XG_CUDA(cudaMemsetAsync(f->d_act_un, 0, f->nw32_el * 4, s));
  k_ml_active<<<(unsigned)((f->nw32_el * 32 + 255) / 256), 256, 0, s>>>(m->ne, f->d_ml_terms, (int)f->ml_terms.size(),
                                                                        f->d_act_cut, f->nw32_el);
  if ((st = compact(f, f->d_act_un, f->nw32_el, f->d_l_un, f->d_el_slot, f->d_counts + 0, s))) return st;
  if ((st = compact(f, f->d_act_cut, f->nw32_el, f->d_l_cut, f->d_el_slot, f->d_counts + 1, s, f->d_counts + 0)))
    return st;
  if (f->has_patch) {
    k_active_facets<<<(unsigned)((f->nw32_fa * 32 + 255) / 256), 256, 0, s>>>(m->nfacets, m->d_facet_els, f->desc,
                                                                              f->d_act_fa, f->nw32_fa);
    if ((st = compact(f, f->d_act_fa, f->nw32_fa, f->d_l_fa, f->d_fa_slot, f->d_counts + 2, s))) return st;
  } else {
    XG_CUDA(cudaMemsetAsync(f->d_act_fa, 0, f->nw32_fa * 4, s));
    XG_CUDA(cudaMemsetAsync(f->d_counts + 2, 0, sizeof(int), s));
  }
  MlFormLaunch L;
  L.dim = m->dim;
  L.order = f->space->order;
  L.M = f->ml_M;
  L.ne = m->ne;
  L.nv = m->nv;
  L.elv = m->d_elv;
  L.xyz = m->d_xyz;
  L.lsets = d_lsets;
  L.terms = f->d_ml_terms;
  L.nterms = (int)f->ml_terms.size();
  L.tuples = f->d_ml_tuples;
  L.list = f->d_l_cut;
  L.counts = f->d_counts;
  L.rowslot = f->d_el_rowslot;
  L.elmat = f->d_elmat;
  L.fp64 = f->precision == XG_PREC_FP64 ? 1 : 0;
  L.err = f->d_err;
  if ((st = mlform_launch(L, s))) return st;
  const bool fp64 = f->precision == XG_PREC_FP64;
  if (f->has_patch && (st = fp64 ? dispatch_patch<double>(f, s) : dispatch_patch<float>(f, s))) return st;
  return rows_back(f, out, s);
}

}  // extern "C"

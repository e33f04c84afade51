// Spatial scatter over the row-major contribution layout (xg_rows.h).
//
// Per step, after the active lists, the element kernels (element rows at
// their static slots), the patch kernels (patch matrices by active-facet
// slot) and the active rows (the dof marking also marks the adjacency slots
// of the active elements):
//   k_fa_mark     thread per (active facet, patch row p): the candidate of
//                 the row's element and facet records the patch row
//   k_rows_accum  warp per active row: its element rows (adjacency order) and
//                 patch rows (candidate order, each as its two halves: the
//                 own element's columns, then the neighbour's) are added in
//                 FP64 into per-warp accumulators in shared memory (several
//                 rows per warp instruction, each into its own accumulator
//                 copy; the copies are added in a fixed order); every added
//                 position is flagged, and the flagged columns (global dof
//                 numbers) and their sums are written compacted at the row's
//                 full-pattern offset (the copies merged 32 positions per
//                 warp instruction), and counted
//   scan          row pointers of the output
//   k_rows_copy   warp per active row: the compacted row into the output,
//                 columns mapped to row numbers.
// Forms whose full pattern is too large for the compaction scratch run
// k_rows_count (the same flags, counted) and the scan first; k_rows_accum
// then writes each row straight into the output.
// No atomics touch values: the sums are formed in the same order on every run.
#include <algorithm>
#include <map>
#include <mutex>

#include "xg_internal.h"
#include "xg_rows.h"

namespace xg {
namespace {

constexpr int kSThreads = 256;
constexpr int kSPer = 8;
constexpr int kSChunk = kSThreads * kSPer;
constexpr int kQL = 4;          // warp instructions' loads in flight in the accumulation loops
constexpr int kCandBatch = 128;  // patch-row candidates of a row loaded at once

// FP32 -> FP64 on the integer pipe (GB300 issues the conversion instruction
// on its narrow FP64 pipe, which the row sums already load).  Exact for
// normal numbers, zeros, infinities and NaNs; FP32 subnormals (below 1.2e-38
// in magnitude) become signed zeros.
__device__ __forceinline__ double to_f64(double x) { return x; }
__device__ __forceinline__ double to_f64(float x) {
  const unsigned u = __float_as_uint(x), e = (u >> 23) & 0xffu, sign = u & 0x80000000u;
  const unsigned m_hi = (u & 0x7fffffu) >> 3, m_lo = u << 29;
  const unsigned ebits = e == 0xffu ? 0x7ff00000u : (e + 896u) << 20;
  const unsigned hi = e == 0 ? sign : sign | ebits | m_hi;
  const unsigned lo = e == 0 ? 0u : m_lo;
  return __hiloint2double((int)hi, (int)lo);
}

// position of column c in the sorted full row at fo (length len), -1 if absent
__device__ __forceinline__ int full_search(const int32_t* __restrict__ cols, int64_t fo, int len, int c) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cols[fo + mid] < c) lo = mid + 1;
    else hi = mid;
  }
  return (lo < len && cols[fo + lo] == c) ? lo : -1;
}

// ---- form creation ---------------------------------------------------------------
__global__ void k_el_rowslot(RowsArgs A, int64_t nadj) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < nadj; a += (int64_t)gridDim.x * blockDim.x) {
    const int v = A.adj[a];
    A.el_rowslot[(int64_t)(v >> 5) * A.nd + (v & 31)] = (int32_t)a;
  }
}

// thread per (adjacency slot a, column j): position of the element's column j
// in the full row of its dof i
__global__ void k_pos_rows(RowsArgs A, int64_t nadj) {
  const int nd = A.nd;
  const int64_t n = nadj * nd;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = t / nd;
    const int j = (int)(t - a * nd);
    const int v = A.adj[a];
    const int64_t e = v >> 5;
    const int r = A.el_dofs[e * nd + (v & 31)], c = A.el_dofs[e * nd + j];
    const int64_t fo = A.full_ptr[r];
    const int pos = full_search(A.tmp_cols, fo, (int)(A.full_ptr[r + 1] - fo), c);
    if (pos < 0 || pos > 65535) set_err(A.err, XG_ERR_CAPACITY);
    A.pos_rows[t] = (uint16_t)(pos < 0 ? 0 : min(pos, 65535));
  }
}

// thread per (candidate c = a * nfl + lf, column j): position of column j of
// the element across facet lf in the full row of the adjacency entry's dof
// (0xffff across a boundary facet: never read)
__global__ void k_nbpos(RowsArgs A, int64_t ncand) {
  const int nd = A.nd, nfl = A.nfl;
  const int64_t n = ncand * nd;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / nd;
    const int j = (int)(t - c * nd);
    const int64_t a = c / nfl;
    const int lf = (int)(c - a * nfl);
    const int v = A.adj[a];
    const int e = v >> 5;
    const int f = A.el_facets[(int64_t)e * nfl + lf];
    const int2 pr = A.fel[f];
    const int e2 = pr.x == e ? pr.y : pr.x;
    uint16_t out = 0xffff;
    if (e2 >= 0) {
      const int r = A.el_dofs[(int64_t)e * nd + (v & 31)], col = A.el_dofs[(int64_t)e2 * nd + j];
      const int64_t fo = A.full_ptr[r];
      const int pos = full_search(A.tmp_cols, fo, (int)(A.full_ptr[r + 1] - fo), col);
      if (pos < 0 || pos > 65534) set_err(A.err, XG_ERR_CAPACITY);
      else out = (uint16_t)pos;
    }
    A.nbpos[t] = out;
  }
}

__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

// ---- per step ----------------------------------------------------------------------
// thread per (active facet slot fs, patch row p): cand_fs of the candidate
// (row p's element and dof, the facet's local index in that element)
__global__ void __launch_bounds__(256) k_fa_mark(RowsArgs A) {
  const int nd = A.nd, n2 = A.n2, nfl = A.nfl;
  const int64_t nfa = min((int64_t)A.counts[2], A.cap_fa), n = nfa * n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t fs = t / n2;
    const int p = (int)(t - fs * n2), side = p >= nd, i = p - side * nd;
    const int f = A.l_fa[fs];
    const int2 pr = A.fel[f];
    const int e = side ? pr.y : pr.x;
    int lf = -1;
    if (e >= 0)
      for (int q = 0; q < nfl; q++)
        if (A.el_facets[(int64_t)e * nfl + q] == f) lf = q;
    if (lf < 0) {
      set_err(A.err, XG_ERR_ARG);
      continue;
    }
    const int64_t c = (int64_t)A.el_rowslot[(int64_t)e * nd + i] * nfl + lf;
    A.cand_fs[c] = (int32_t)t;
  }
}

// ND dofs per element, NFL facets per element (compile time: the index
// arithmetic of the inner loops divides by them)
template <typename T, int ND, int NFL, bool DIRECT>
__global__ void __launch_bounds__(kRowsMaxWarps * 32) k_rows_accum(RowsArgs A, const T* __restrict__ elrows,
                                                                 const T* __restrict__ farows,
                                                                 const int64_t* __restrict__ rowptr,
                                                                 int32_t* __restrict__ cols, double* __restrict__ vals,
                                                                 int64_t cap_nnz) {
  constexpr int N2 = 2 * ND;
  extern __shared__ __align__(16) unsigned char sm_acc[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int LEN = A.W * 32, C = A.copies;
  double* acc = (double*)sm_acc + (size_t)warp * C * LEN;
  int* clist = (int*)((double*)sm_acc + (size_t)A.warps * C * LEN) + (size_t)warp * (2 * kCandBatch + LEN / 4);
  int* cpi = clist + kCandBatch;                            // [kCandBatch] patch rows of the batch's candidates
  unsigned char* fl = (unsigned char*)(cpi + kCandBatch);  // [LEN] touched positions of the row
  for (int k = lane; k < C * LEN; k += 32) acc[k] = 0.0;
  for (int k = lane; k < LEN; k += 32) fl[k] = 0;
  __syncwarp();
  const int nrows = A.counts[3];
  const int ce = min(C, max(1, 32 / ND));
  const int cl = lane / ND, jl = lane - cl * ND;
  const bool on = cl < ce;
  const unsigned below = (1u << lane) - 1;
  const int stride = gridDim.x * A.warps;
  int row = blockIdx.x * A.warps + warp;
  int r = row < nrows ? A.rows[row] : 0;
  for (; row < nrows; row += stride) {
    const int64_t fo = A.full_ptr[r];
    const int len = (int)(A.full_ptr[r + 1] - fo), nw = (len + 31) >> 5;
    const int a0 = A.adj_ptr[r], a1 = A.adj_ptr[r + 1];
    const int r_next = row + stride < nrows ? A.rows[row + stride] : 0;  // next row's dof, in flight
    // DIRECT: the row's place in the output, from the counting pass and the scan
    const int64_t rp = DIRECT ? rowptr[row] : 0;
    const int64_t ucnt = DIRECT ? rowptr[row + 1] - rp : 0;
    if (nw > A.W || (DIRECT && rp + ucnt > cap_nnz)) {
      if (lane == 0) {
        set_err(A.err, XG_ERR_CAPACITY);
        if (!DIRECT) A.rowcnt[row] = 0;
      }
      r = r_next;
      continue;
    }
    // element rows: every adjacency entry's row is loaded (contiguous), the
    // active ones (this step's bytes, cleared after) are added
    const int nent = a1 - a0;
    for (int k0 = 0; k0 < nent; k0 += ce * kQL) {
      double v[kQL];
      int p[kQL];
#pragma unroll
      for (int q = 0; q < kQL; q++) {
        const int k = k0 + q * ce + cl;
        p[q] = -1;
        v[q] = 0.0;
        if (on && k < nent) {
          const int64_t a = a0 + k, o = a * ND + jl;
          const bool act = A.act_slot[a] != 0;
          v[q] = to_f64(elrows[o]);
          const int pp = A.pos_rows[o];
          p[q] = act ? pp : -1;
        }
      }
#pragma unroll
      for (int q = 0; q < kQL; q++)
        if (k0 + q * ce < nent)  // warp-uniform: waves past the row's entries issue no FP64 add
          if (p[q] >= 0 && p[q] < len) {
            acc[cl * LEN + p[q]] += v[q];
            fl[p[q]] = 1;
          }
    }
    __syncwarp();
    for (int k = lane; k < nent; k += 32) A.act_slot[a0 + k] = 0;  // cleared for the next step
    // patch rows: the row's candidates in order, each patch row as its own
    // element's half, then the neighbour's half (a dof of the common facet is
    // in both halves: the halves never share an instruction's copy)
    const int64_t cb = (int64_t)a0 * NFL, cend = A.cand_fs ? (int64_t)a1 * NFL : cb;  // no patch terms: none
    for (int64_t c0 = cb; c0 < cend; c0 += kCandBatch) {
      int pi[kCandBatch / 32];
#pragma unroll
      for (int u = 0; u < kCandBatch / 32; u++) {
        const int64_t c = c0 + 32 * u + lane;
        pi[u] = c < cend ? A.cand_fs[c] : -1;
      }
      int nact = 0;
#pragma unroll
      for (int u = 0; u < kCandBatch / 32; u++) {
        const unsigned m = __ballot_sync(0xffffffffu, pi[u] >= 0);
        if (pi[u] >= 0) {
          const int k = nact + __popc(m & below);
          clist[k] = (int)(c0 - cb) + 32 * u + lane;
          cpi[k] = pi[u];
          A.cand_fs[c0 + 32 * u + lane] = -1;  // cleared for the next step
        }
        nact += __popc(m);
      }
      __syncwarp();
      const int nh = 2 * nact;
      for (int k0 = 0; k0 < nh; k0 += ce * kQL) {
        double v[kQL];
        int p[kQL];
#pragma unroll
        for (int q = 0; q < kQL; q++) {
          const int hk = k0 + q * ce + cl;
          p[q] = -1;
          v[q] = 0.0;
          if (on && hk < nh) {
            const int k = hk >> 1, h = hk & 1;
            const int prow = cpi[k];
            const int64_t cc = cb + clist[k];
            const int side = (prow % N2) >= ND;
            const int col0 = (h == 0) == (side == 0) ? 0 : ND;  // own half at side * ND
            v[q] = to_f64(farows[(int64_t)prow * N2 + col0 + jl]);
            p[q] = h == 0 ? A.pos_rows[(cc / NFL) * ND + jl] : A.nbpos[cc * ND + jl];
          }
        }
#pragma unroll
        for (int q = 0; q < kQL; q++)
          if (k0 + q * ce < nh)  // warp-uniform, as above
            if (p[q] >= 0 && p[q] < len) {
              acc[cl * LEN + p[q]] += v[q];
              fl[p[q]] = 1;
            }
      }
      __syncwarp();
    }
    __syncwarp();
    // flagged columns in ascending order (collected into a position list,
    // 32 merged per warp instruction), compacted at the row's full offset as
    // global dof numbers (k_rows_copy maps them to rows); the copies added in
    // order and cleared, the flags cleared
    int* plist = clist;  // [2 kCandBatch] (the candidate lists are free here)
    constexpr int PL = 2 * kCandBatch;
    int base = 0, nl = 0;
    auto flush = [&]() {
      __syncwarp();
      for (int i = lane; i < nl; i += 32) {
        const int k = plist[i];
        const int col = A.tmp_cols[fo + k];
        double s = acc[k];
        acc[k] = 0.0;
        for (int cc = 1; cc < C; cc++) {
          s += acc[cc * LEN + k];
          acc[cc * LEN + k] = 0.0;
        }
        if (DIRECT) {
          if (base + i < ucnt) {
            cols[rp + base + i] = A.dof_row[col];
            vals[rp + base + i] = s;
          }
        } else {
          A.vcols[fo + base + i] = col;
          A.vvals[fo + base + i] = s;
        }
      }
      base += nl;
      nl = 0;
      __syncwarp();
    };
    for (int w0 = 0; w0 < nw; w0 += 4) {
      if (nl > PL - 128) flush();
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int k = 32 * (w0 + u) + lane;
        const bool set = w0 + u < nw && fl[k];
        const unsigned bits = __ballot_sync(0xffffffffu, set);
        if (set) {
          plist[nl + __popc(bits & below)] = k;
          fl[k] = 0;
        }
        nl += __popc(bits);
      }
    }
    flush();
    if (lane == 0) {
      if (DIRECT) {
        if (base != ucnt) set_err(A.err, XG_ERR_CAPACITY);
      } else {
        A.rowcnt[row] = base;
      }
    }
    __syncwarp();
    r = r_next;
  }
}

// Counting pass of the direct path (forms whose full pattern is too large
// for the compaction scratch): the same positions as k_rows_accum, flagged
// per row and counted; nothing is cleared (the accumulation pass clears).
template <int ND, int NFL>
__global__ void __launch_bounds__(kRowsMaxWarps * 32) k_rows_count(RowsArgs A) {
  extern __shared__ __align__(16) unsigned char sm_cnt[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int LEN = A.W * 32;
  int* clist = (int*)sm_cnt + (size_t)warp * (2 * kCandBatch + LEN / 4);
  int* cpi = clist + kCandBatch;
  unsigned char* fl = (unsigned char*)(cpi + kCandBatch);
  for (int k = lane; k < LEN; k += 32) fl[k] = 0;
  __syncwarp();
  const int nrows = A.counts[3];
  const unsigned below = (1u << lane) - 1;
  for (int row = blockIdx.x * A.warps + warp; row < nrows; row += gridDim.x * A.warps) {
    const int r = A.rows[row];
    const int64_t fo = A.full_ptr[r];
    const int len = (int)(A.full_ptr[r + 1] - fo), nw = (len + 31) >> 5;
    const int a0 = A.adj_ptr[r], a1 = A.adj_ptr[r + 1];
    if (nw > A.W) {
      if (lane == 0) {
        set_err(A.err, XG_ERR_CAPACITY);
        A.rowcnt[row] = 0;
      }
      continue;
    }
    const int n = (a1 - a0) * ND;
    for (int t = lane; t < n; t += 32) {
      const int k = t / ND;
      const int64_t a = a0 + k;
      if (A.act_slot[a]) {
        const int p = A.pos_rows[a * ND + (t - k * ND)];
        if (p < len) fl[p] = 1;
      }
    }
    const int64_t cb = (int64_t)a0 * NFL, cend = A.cand_fs ? (int64_t)a1 * NFL : cb;
    for (int64_t c0 = cb; c0 < cend; c0 += kCandBatch) {
      int pi[kCandBatch / 32];
#pragma unroll
      for (int u = 0; u < kCandBatch / 32; u++) {
        const int64_t c = c0 + 32 * u + lane;
        pi[u] = c < cend ? A.cand_fs[c] : -1;
      }
      int nact = 0;
#pragma unroll
      for (int u = 0; u < kCandBatch / 32; u++) {
        const unsigned m = __ballot_sync(0xffffffffu, pi[u] >= 0);
        if (pi[u] >= 0) {
          const int k = nact + __popc(m & below);
          clist[k] = (int)(c0 - cb) + 32 * u + lane;
          cpi[k] = pi[u];
        }
        nact += __popc(m);
      }
      __syncwarp();
      const int nt = nact * 2 * ND;
      for (int t = lane; t < nt; t += 32) {
        const int hk = t / ND, j = t - hk * ND, k = hk >> 1;
        const int64_t cc = cb + clist[k];
        const int p = (hk & 1) == 0 ? A.pos_rows[(cc / NFL) * ND + j] : A.nbpos[cc * ND + j];
        if (p < len) fl[p] = 1;
      }
      __syncwarp();
    }
    __syncwarp();
    int cnt = 0;
    for (int w = 0; w < nw; w++) {
      const int k = 32 * w + lane;
      const bool set = fl[k] != 0;
      if (set) fl[k] = 0;
      cnt += __popc(__ballot_sync(0xffffffffu, set));
    }
    if (lane == 0) A.rowcnt[row] = cnt;
    __syncwarp();
  }
}

// ---- exclusive scan of the row counts (n = counts[3]) --------------------------------
__device__ __forceinline__ long long block_scan_ll(long long v, long long* total, long long* sm) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[wid] = x;
  __syncthreads();
  if (wid == 0) {
    long long t = lane < nw ? sm[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    sm[lane] = t;
  }
  __syncthreads();
  const long long base = wid > 0 ? sm[wid - 1] : 0;
  if (total) *total = sm[nw - 1];
  __syncthreads();
  return base + x - v;
}

__global__ void k_scan_blocks(const int64_t* __restrict__ cnt, const int* __restrict__ n_ptr,
                              long long* __restrict__ bs) {
  __shared__ long long sm[32];
  const int n = *n_ptr;
  const int64_t i0 = (int64_t)blockIdx.x * kSChunk + (int64_t)threadIdx.x * kSPer;
  long long s = 0;
  for (int k = 0; k < kSPer; k++)
    if (i0 + k < n) s += cnt[i0 + k];
  long long tot;
  block_scan_ll(s, &tot, sm);
  if (threadIdx.x == 0) bs[blockIdx.x] = tot;
}

// one block: exclusive scan of bs[0, nb) in place
__global__ void k_scan_top(long long* bs, int nb) {
  __shared__ long long sm[32];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const long long x = i < nb ? bs[i] : 0;
    long long tot;
    const long long ex = block_scan_ll(x, &tot, sm);
    if (i < nb) bs[i] = ex + carry;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
}

// rowptr (+ counts_out {n, total}); capacity against cap_nnz
__global__ void k_scan_apply(const int64_t* __restrict__ cnt, const int* __restrict__ n_ptr,
                             const long long* __restrict__ bs, int64_t* __restrict__ rowptr,
                             int64_t* __restrict__ counts_out, int64_t cap_nnz, int* err) {
  __shared__ long long sm[32];
  const int n = *n_ptr;
  const int64_t i0 = (int64_t)blockIdx.x * kSChunk + (int64_t)threadIdx.x * kSPer;
  long long c[kSPer];
  long long s = 0;
  for (int k = 0; k < kSPer; k++) {
    c[k] = (i0 + k < n) ? cnt[i0 + k] : 0;
    s += c[k];
  }
  long long pos = bs[blockIdx.x] + block_scan_ll(s, nullptr, sm);
  for (int k = 0; k < kSPer; k++) {
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

// warp per active row: the compacted row into the output (rows beyond the
// output capacity are skipped; the scan reported it)
__global__ void __launch_bounds__(256) k_rows_copy(RowsArgs A, const int64_t* __restrict__ rowptr,
                                                   int32_t* __restrict__ cols, double* __restrict__ vals,
                                                   int64_t cap_nnz) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nrows = A.counts[3];
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nrows; row += nwarps) {
    const int64_t fo = A.full_ptr[A.rows[row]];
    const int64_t rp = rowptr[row], u = rowptr[row + 1] - rp;
    if (rp + u > cap_nnz) continue;
    for (int64_t k = lane; k < u; k += 32) {
      cols[rp + k] = A.dof_row[A.vcols[fo + k]];
      vals[rp + k] = A.vvals[fo + k];
    }
  }
}

int grid_of(const void* kernel, int threads, size_t smem) {
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
  return nsm * std::max(per, 1);
}

unsigned blocks_for(int64_t n, int64_t cap) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, cap));
}

// the accumulation / counting kernels of the element type (dofs per element,
// facets per element)
template <typename T, bool DIRECT>
const void* accum_kernel(int nd, int nfl) {
  if (nfl == 3) {
    if (nd == 3) return (const void*)k_rows_accum<T, 3, 3, DIRECT>;
    if (nd == 6) return (const void*)k_rows_accum<T, 6, 3, DIRECT>;
    if (nd == 10) return (const void*)k_rows_accum<T, 10, 3, DIRECT>;
  } else if (nfl == 4) {
    if (nd == 4) return (const void*)k_rows_accum<T, 4, 4, DIRECT>;
    if (nd == 10) return (const void*)k_rows_accum<T, 10, 4, DIRECT>;
    if (nd == 20) return (const void*)k_rows_accum<T, 20, 4, DIRECT>;
  }
  return nullptr;
}
const void* accum_kernel_of(bool fp64, bool direct, int nd, int nfl) {
  if (fp64) return direct ? accum_kernel<double, true>(nd, nfl) : accum_kernel<double, false>(nd, nfl);
  return direct ? accum_kernel<float, true>(nd, nfl) : accum_kernel<float, false>(nd, nfl);
}
const void* count_kernel(int nd, int nfl) {
  if (nfl == 3) {
    if (nd == 3) return (const void*)k_rows_count<3, 3>;
    if (nd == 6) return (const void*)k_rows_count<6, 3>;
    if (nd == 10) return (const void*)k_rows_count<10, 3>;
  } else if (nfl == 4) {
    if (nd == 4) return (const void*)k_rows_count<4, 4>;
    if (nd == 10) return (const void*)k_rows_count<10, 4>;
    if (nd == 20) return (const void*)k_rows_count<20, 4>;
  }
  return nullptr;
}

}  // namespace

int rows_static_build(const RowsArgs& A, bool has_patch, cudaStream_t s) {
  const int64_t nadj = (int64_t)A.ne * A.nd;
  if (nadj == 0) return XG_OK;
  k_el_rowslot<<<blocks_for(nadj, 152 * 32), 256, 0, s>>>(A, nadj);
  k_pos_rows<<<blocks_for(nadj * A.nd, 152 * 64), 256, 0, s>>>(A, nadj);
  if (has_patch) {
    const int64_t ncand = nadj * A.nfl;
    k_nbpos<<<blocks_for(ncand * A.nd, 152 * 64), 256, 0, s>>>(A, ncand);
    k_fill_i32<<<blocks_for(ncand, 152 * 32), 256, 0, s>>>(A.cand_fs, ncand, -1);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "rows_static_build");
}

size_t rows_accum_smem(const RowsArgs& A) {
  return (size_t)A.warps *
         ((size_t)A.copies * A.W * 32 * sizeof(double) + (2 * kCandBatch + A.W * 8) * sizeof(int));
}

int rows_accum_grid(const RowsArgs& A, bool fp64, size_t smem) {
  const bool direct = A.vcols == nullptr;
  const void* k = accum_kernel_of(fp64, direct, A.nd, A.nfl);
  const void* kc = count_kernel(A.nd, A.nfl);
  if (!k || !kc) return 0;
  {
    // the attribute is an upper bound shared by all forms: only ever raise it
    static std::mutex mu;
    static std::map<const void*, size_t> raised;
    std::lock_guard<std::mutex> lock(mu);
    for (const void* kk : {k, kc}) {
      size_t& cur = raised[kk];
      if (cur == 0) cur = 48 * 1024;
      if (smem > cur) {
        if (cudaFuncSetAttribute(kk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
          cudaGetLastError();
          return 0;
        }
        cur = smem;
      }
    }
  }
  return grid_of(k, A.warps * 32, smem);
}

int rows_scatter(const RowsArgs& A, int64_t ndof, bool has_patch, bool fp64, const void* elrows,
                 const void* farows, int64_t* out_rowptr, int64_t* out_counts, int32_t* cols, double* vals,
                 int64_t cap_nnz, int grid, size_t smem, cudaStream_t s) {
  const bool direct = A.vcols == nullptr;  // no compaction scratch: count, scan, then sum into the output
  const void* k = accum_kernel_of(fp64, direct, A.nd, A.nfl);
  const void* kc = count_kernel(A.nd, A.nfl);
  if (!k || !kc) {
    set_last_error("rows_scatter: unsupported element type");
    return XG_ERR_UNSUPPORTED;
  }
  const int nb = (int)std::max<int64_t>(1, (ndof + kSChunk - 1) / kSChunk);
  if (nb > A.nbsum) {
    set_last_error("rows_scatter: scan workspace too small");
    return XG_ERR_CAPACITY;
  }
  if (has_patch) k_fa_mark<<<152 * 8, 256, 0, s>>>(A);
  RowsArgs a = A;
  if (direct) {
    void* cargs[] = {&a};
    cudaError_t e = cudaLaunchKernel(kc, dim3(grid), dim3(A.warps * 32), cargs, smem, s);
    if (e != cudaSuccess) return cuda_fail(e, "k_rows_count");
  }
  void* args[] = {&a, const_cast<void**>(&elrows), const_cast<void**>(&farows), &out_rowptr, &cols, &vals, &cap_nnz};
  if (!direct) {
    cudaError_t e = cudaLaunchKernel(k, dim3(grid), dim3(A.warps * 32), args, smem, s);
    if (e != cudaSuccess) return cuda_fail(e, "k_rows_accum");
  }
  k_scan_blocks<<<nb, kSThreads, 0, s>>>(A.rowcnt, A.counts + 3, A.bsum);
  k_scan_top<<<1, 1024, 0, s>>>(A.bsum, nb);
  k_scan_apply<<<nb, kSThreads, 0, s>>>(A.rowcnt, A.counts + 3, A.bsum, out_rowptr, out_counts, cap_nnz, A.err);
  if (direct) {
    cudaError_t e = cudaLaunchKernel(k, dim3(grid), dim3(A.warps * 32), args, smem, s);
    if (e != cudaSuccess) return cuda_fail(e, "k_rows_accum");
  } else {
    k_rows_copy<<<152 * 16, 256, 0, s>>>(A, out_rowptr, cols, vals, cap_nnz);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "rows_scatter");
}

}  // namespace xg

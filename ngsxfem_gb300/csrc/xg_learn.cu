// Learned cut quadrature for P2 level sets on tetrahedra.
//
// No counterpart in the reference: it replaces, for a cut tetrahedron with a
// P2 level set, the isoparametric workflow the reference needs before its
// straight cut rule (LevelSetMeshAdaptation, python/lsetcurv.py:281-356, then
// StraightCutIntegrationRule on the deformed element).
//
// Rule of an element with P2 nodal values v (10, element-local order):
//   Q(f) = straight cut rule of the P1 interpolant on the NEG part (FP64)
//        + sum_i w_i(x) f(p_i),  i < 24,
// p_i a fixed point set in the reference tet and w = MLP(x), x = v / max|v|,
// an MLP 10 -> 256 -> 256 -> 24 with SiLU activations whose output y gives the
// weights w = R^-1 y, V = U R the thin QR of V[a][i] = p_i^a.  The network is
// trained on the moment defect d = m_iso - m_p1 (35 monomials of degree <= 4):
// the loss of a sample is sum_a ((U y - d)_a / s)^2 with s = max_a |m_iso,a|
// (floored), averaged over the batch.
//
// Precision: FP32 master parameters (Adam), BF16 copies used by every product
// of the forward and backward passes, FP32 accumulation; moments and the
// straight cut part in FP64.  All products are tiled FP32 FMA kernels
// (shared-memory tiles of 64 x 64, 4 x 4 outputs per thread); the split-K
// weight gradients are reduced in a fixed order (deterministic).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "xg_internal.h"

namespace xg {

int tet_moments_launch(const double* d_vals, int64_t n, int order, int deform, double* d_out, int32_t* d_nonconv,
                       cudaStream_t s, const int32_t* d_list, const int32_t* d_count);  // xg_iso.cu
// tensor-core inference (xg_mlp_tc.cu)
extern const int kTcPackedBytes;
int mlp_tc_pack(const float* d_params, int64_t off_w1, int64_t off_w2, int64_t off_w3, void* d_packed,
                cudaStream_t s);
int mlp_tc_forward(const float* d_x, int64_t B, const void* d_packed, const float* d_b1, const float* d_b2,
                   const float* d_b3, float* d_y, int* d_err, cudaStream_t s);

namespace {

constexpr int kIn = 10, kHid = 256, kOut = 24, kMom = 35;
constexpr int64_t kOffW1 = 0;
constexpr int64_t kOffB1 = kOffW1 + kIn * kHid;
constexpr int64_t kOffW2 = kOffB1 + kHid;
constexpr int64_t kOffB2 = kOffW2 + kHid * kHid;
constexpr int64_t kOffW3 = kOffB2 + kHid;
constexpr int64_t kOffB3 = kOffW3 + kHid * kOut;
constexpr int64_t kNumParams = kOffB3 + kOut;
// fixed output scale: the moment correction is kOutScale * U y, so that the
// network's outputs are of order one for defects of a few per cent of the
// element measure
constexpr float kOutScale = 1.0f / 256.0f;

// U of the thin QR V = U R of the Vandermonde matrix V[a][i] = p_i^a: the
// network output y gives the weights w = R^-1 y at the points and the moment
// correction V w = U y (a well-conditioned output layer)
__constant__ float c_V[kMom * kOut];   // U (FP32, loss)
__constant__ double c_Vd[kMom * kOut];  // U (FP64, rule)

// ---- fixed point set: orbits s31(0.075), s31(0.16), s211(0.025, 0.36), s31(0.32) in
// barycentric coordinates, each orbit's distinct permutations in lexicographic
// order; point = (lambda_0, lambda_1, lambda_2)
void point_set(double (*pts)[3]) {
  std::vector<std::vector<double>> out;
  auto orbit = [&](std::vector<double> b) {
    std::sort(b.begin(), b.end());
    std::vector<std::vector<double>> o;
    do o.push_back(b);
    while (std::next_permutation(b.begin(), b.end()));
    for (auto& x : o) out.push_back(x);
  };
  orbit({1 - 3 * 0.075, 0.075, 0.075, 0.075});
  orbit({1 - 3 * 0.16, 0.16, 0.16, 0.16});
  orbit({0.025, 0.025, 0.36, 1 - 2 * 0.025 - 0.36});
  orbit({1 - 3 * 0.32, 0.32, 0.32, 0.32});
  for (int i = 0; i < kOut; i++)
    for (int k = 0; k < 3; k++) pts[i][k] = out[i][k];
}

void vandermonde(double* V) {
  double p[kOut][3];
  point_set(p);
  int a = 0;
  for (int t = 0; t <= 4; t++)
    for (int ex = t; ex >= 0; ex--)
      for (int ey = t - ex; ey >= 0; ey--, a++) {
        const int ez = t - ex - ey;
        for (int i = 0; i < kOut; i++)
          V[a * kOut + i] = std::pow(p[i][0], ex) * std::pow(p[i][1], ey) * std::pow(p[i][2], ez);
      }
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// ---- kernels ------------------------------------------------------------------
__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ q, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    q[i] = __float2bfloat16_rn(p[i]);
}

template <typename T>
__device__ __forceinline__ float ld(const T* p, int64_t i);
template <>
__device__ __forceinline__ float ld<float>(const float* p, int64_t i) {
  return p[i];
}
template <>
__device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16* p, int64_t i) {
  return __bfloat162float(p[i]);
}

// C = op(A) op(B) over k in [z*kchunk, min(K, (z+1)*kchunk)), written to
// C + z*M*N (ldc = N) when splitting; op(A) is M x K, op(B) is K x N.
// TA: A stored K x M (lda = M); TB: B stored N x K (ldb = K).
constexpr int kBM = 64, kBN = 64, kBK = 16;
template <bool TA, bool TB, typename TBt>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, int kchunk, const float* __restrict__ A,
                                               const TBt* __restrict__ B, float* __restrict__ C) {
  __shared__ float As[kBK][kBM + 4];
  __shared__ float Bs[kBK][kBN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  float acc[4][4] = {};
  for (int k0 = kb; k0 < ke; k0 += kBK) {
    for (int t = threadIdx.x; t < kBK * kBM; t += 256) {
      const int kk = TA ? t / kBM : t % kBK, mm = TA ? t % kBM : t / kBK;
      const int gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < ke) v = TA ? A[(int64_t)gk * M + gm] : A[(int64_t)gm * K + gk];
      As[kk][mm] = v;
    }
    for (int t = threadIdx.x; t < kBK * kBN; t += 256) {
      const int kk = TB ? t % kBK : t / kBN, nn = TB ? t / kBK : t % kBN;
      const int gn = n0 + nn, gk = k0 + kk;
      float v = 0.f;
      if (gn < N && gk < ke) v = TB ? ld(B, (int64_t)gn * K + gk) : ld(B, (int64_t)gk * N + gn);
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  float* Cz = C + (int64_t)blockIdx.z * M * N;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
      if (gm < M && gn < N) Cz[(int64_t)gm * N + gn] = acc[i][j];
    }
}

// out[i] = sum_z part[z][i], z in order (deterministic split-K reduction)
__global__ void k_sum_parts(const float* __restrict__ part, int nz, int64_t n, float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < nz; z++) s += part[(int64_t)z * n + i];
    out[i] = s;
  }
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float sg = 1.f / (1.f + __expf(-z));
  return sg * (1.f + z * (1.f - sg));
}

// Z += bias (in place), H = silu(Z) (H may be null: bias only)
__global__ void k_bias_act(float* __restrict__ Z, const float* __restrict__ bias, int64_t rows, int cols,
                           float* __restrict__ H) {
  const int64_t n = rows * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float z = Z[i] + bias[i % cols];
    Z[i] = z;
    if (H) H[i] = silu(z);
  }
}

__global__ void k_act_grad(float* __restrict__ dH, const float* __restrict__ Z, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dH[i] *= dsilu(Z[i]);
}

// column sums of a rows x cols matrix: one thread per column, rows in order
__global__ void k_colsum(const float* __restrict__ X, int64_t rows, int cols, float* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int64_t r = 0; r < rows; r++) s += X[r * cols + c];
  out[c] = s;
}

// per-sample loss and dY: pred = kOutScale U y, r = (pred - t) / s,
// loss_i = |r|^2, dY = (2 / B) kOutScale U^T r / s
__global__ void k_moment_loss(const float* __restrict__ Y, const float* __restrict__ T, const float* __restrict__ S,
                              int64_t B, float* __restrict__ dY, float* __restrict__ loss_i) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B; i += (int64_t)gridDim.x * blockDim.x) {
    float y[kOut], r[kMom];
    for (int j = 0; j < kOut; j++) y[j] = Y[i * kOut + j];
    const float inv = 1.f / S[i];
    float l = 0.f;
    for (int a = 0; a < kMom; a++) {
      float p = 0.f;
      for (int j = 0; j < kOut; j++) p = fmaf(c_V[a * kOut + j], y[j], p);
      r[a] = (kOutScale * p - T[i * kMom + a]) * inv;
      l = fmaf(r[a], r[a], l);
    }
    loss_i[i] = l;
    const float g = 2.f / (float)B * inv * kOutScale;
    for (int j = 0; j < kOut; j++) {
      float s = 0.f;
      for (int a = 0; a < kMom; a++) s = fmaf(c_V[a * kOut + j], r[a], s);
      dY[i * kOut + j] = g * s;
    }
  }
}

// mean of n values, one block, fixed order
__global__ void k_mean(const float* __restrict__ x, int64_t n, float* __restrict__ out) {
  __shared__ float sm[256];
  float s = 0.f;
  for (int64_t i = threadIdx.x; i < n; i += 256) s += x[i];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sm[0] / (float)n;
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// features: u = v / max|v|, then the four vertex values of u and the six
// edge-midpoint deviations u_e - (u_a + u_b) / 2 (a linear map of the
// normalised nodal values that separates the linear part from the curvature)
__global__ void k_features(const double* __restrict__ v, int64_t n, float* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double m = 0.0;
    for (int k = 0; k < kIn; k++) m = fmax(m, fabs(v[i * kIn + k]));
    const double inv = m > 0.0 ? 1.0 / m : 0.0;
    double u[kIn];
    for (int k = 0; k < kIn; k++) u[k] = v[i * kIn + k] * inv;
    const int ea[6] = {0, 0, 0, 1, 1, 2}, eb[6] = {1, 2, 3, 2, 3, 3};
    for (int k = 0; k < 4; k++) x[i * kIn + k] = (float)u[k];
    for (int e = 0; e < 6; e++) x[i * kIn + 4 + e] = (float)(u[4 + e] - 0.5 * (u[ea[e]] + u[eb[e]]));
  }
}

// fallback list: elements in the relevant band whose curvature indicator
// max_e |u_e - (u_a + u_b) / 2| exceeds kappa_max
__global__ void k_fallback_list(const float* __restrict__ x, const double* __restrict__ vals, int64_t n,
                                double kappa_max, int32_t* __restrict__ list, int32_t* __restrict__ count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float k = 0.f;
    for (int e = 0; e < 6; e++) k = fmaxf(k, fabsf(x[i * kIn + 4 + e]));
    bool hn = false, hp = false;
    for (int c = 0; c < 4; c++) {
      double p = vals[i * kIn + c];
      if (fabs(p) < 1e-14) p = 1e-14;
      hn |= p < 0.0;
      hp |= p > 0.0;
    }
    if (hn && hp && (double)k > kappa_max) list[atomicAdd(count, 1)] = (int32_t)i;
  }
}

// out[i] += kOutScale U y[i] (FP64) for the elements with a cut P1 interpolant
__global__ void k_add_correction(const float* __restrict__ Y, const double* __restrict__ vals, int64_t n,
                                 double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    bool hn = false, hp = false;
    for (int k = 0; k < 4; k++) {
      double p = vals[i * kIn + k];
      if (fabs(p) < 1e-14) p = 1e-14;
      hn |= p < 0.0;
      hp |= p > 0.0;
    }
    if (!(hn && hp)) continue;  // outside the relevant band the plain rule is the isoparametric one
    double y[kOut];
    for (int j = 0; j < kOut; j++) y[j] = (double)Y[i * kOut + j];
    for (int a = 0; a < kMom; a++) {
      double s = 0.0;
      for (int j = 0; j < kOut; j++) s += c_Vd[a * kOut + j] * y[j];
      out[i * kMom + a] += (double)kOutScale * s;
    }
  }
}

unsigned grid1(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8)); }

}  // namespace
}  // namespace xg

using namespace xg;

struct xg_mlp {
  float* p = nullptr;           // master parameters (FP32)
  __nv_bfloat16* pb = nullptr;  // BF16 copy used by the products
  float* m = nullptr;           // Adam moments
  float* v = nullptr;
  float* g = nullptr;           // gradient (flat, like p)
  // activations / workspace, sized for cap rows
  int64_t cap = 0;
  float *x = nullptr, *z1 = nullptr, *h1 = nullptr, *z2 = nullptr, *h2 = nullptr, *y = nullptr, *dy = nullptr;
  float *dh1 = nullptr, *dh2 = nullptr, *li = nullptr, *part = nullptr;
  int32_t* list = nullptr;  // fallback elements
  int32_t* count = nullptr;
  void* tcw = nullptr;  // BF16 weight images of the tensor-core inference kernel
  int* err = nullptr;   // device status of the tensor-core kernel
};

namespace {

constexpr int kSplit = 32;
constexpr int64_t kMaxRows = 4194240;  // 65535 row tiles of 64

void mlp_free_ws(xg_mlp* m) {
  for (float* q : {m->x, m->z1, m->h1, m->z2, m->h2, m->y, m->dy, m->dh1, m->dh2, m->li, m->part}) cudaFree(q);
  cudaFree(m->list);
  cudaFree(m->count);
  m->x = m->z1 = m->h1 = m->z2 = m->h2 = m->y = m->dy = m->dh1 = m->dh2 = m->li = m->part = nullptr;
  m->list = m->count = nullptr;
  m->cap = 0;
}

int mlp_reserve(xg_mlp* m, int64_t rows) {
  if (rows <= m->cap) return XG_OK;
  mlp_free_ws(m);
  auto A = [](float** p, int64_t n) { return cudaMalloc((void**)p, sizeof(float) * std::max<int64_t>(n, 1)); };
  cudaError_t e = A(&m->x, rows * kIn);
  if (!e) e = A(&m->z1, rows * kHid);
  if (!e) e = A(&m->h1, rows * kHid);
  if (!e) e = A(&m->z2, rows * kHid);
  if (!e) e = A(&m->h2, rows * kHid);
  if (!e) e = A(&m->y, rows * kOut);
  if (!e) e = A(&m->dy, rows * kOut);
  if (!e) e = A(&m->dh1, rows * kHid);
  if (!e) e = A(&m->dh2, rows * kHid);
  if (!e) e = A(&m->li, rows);
  if (!e) e = A(&m->part, (int64_t)kSplit * kHid * kHid);
  if (!e) e = cudaMalloc((void**)&m->list, sizeof(int32_t) * std::max<int64_t>(rows, 1));
  if (!e) e = cudaMalloc((void**)&m->count, sizeof(int32_t));
  if (e) {
    mlp_free_ws(m);
    return cuda_fail(e, "xg_mlp workspace");
  }
  m->cap = rows;
  return XG_OK;
}

// thin QR of the Vandermonde matrix by modified Gram-Schmidt over its columns
// in order (positive diagonal of R): V = U R, U with orthonormal columns
void orthonormal_basis(double* U) {
  vandermonde(U);
  for (int j = 0; j < kOut; j++) {
    for (int i = 0; i < j; i++) {
      double d = 0.0;
      for (int a = 0; a < kMom; a++) d += U[a * kOut + i] * U[a * kOut + j];
      for (int a = 0; a < kMom; a++) U[a * kOut + j] -= d * U[a * kOut + i];
    }
    double nrm = 0.0;
    for (int a = 0; a < kMom; a++) nrm += U[a * kOut + j] * U[a * kOut + j];
    nrm = std::sqrt(nrm);
    for (int a = 0; a < kMom; a++) U[a * kOut + j] /= nrm;
  }
}

int upload_V() {
  static bool done = false;
  if (done) return XG_OK;
  double V[kMom * kOut];
  orthonormal_basis(V);
  float Vf[kMom * kOut];
  for (int i = 0; i < kMom * kOut; i++) Vf[i] = (float)V[i];
  XG_CUDA(cudaMemcpyToSymbol(c_V, Vf, sizeof(Vf)));
  XG_CUDA(cudaMemcpyToSymbol(c_Vd, V, sizeof(V)));
  done = true;
  return XG_OK;
}

template <bool TA, bool TB, typename TBt>
int gemm(int M, int N, int K, const float* A, const TBt* B, float* C, int split, float* part, cudaStream_t s) {
  dim3 grid((N + kBN - 1) / kBN, (M + kBM - 1) / kBM, split);
  const int kchunk = ((K + split - 1) / split + kBK - 1) / kBK * kBK;
  k_gemm<TA, TB, TBt><<<grid, 256, 0, s>>>(M, N, K, kchunk, A, B, split > 1 ? part : C);
  if (split > 1) k_sum_parts<<<grid1((int64_t)M * N), 256, 0, s>>>(part, split, (int64_t)M * N, C);
  XG_CUDA(cudaGetLastError());
  return XG_OK;
}

// forward of rows x (features already in m->x)
int forward(xg_mlp* m, int64_t B, cudaStream_t s) {
  int st;
  const int b = (int)B;
  if ((st = gemm<false, false>(b, kHid, kIn, m->x, m->pb + kOffW1, m->z1, 1, nullptr, s))) return st;
  k_bias_act<<<grid1(B * kHid), 256, 0, s>>>(m->z1, m->p + kOffB1, B, kHid, m->h1);
  if ((st = gemm<false, false>(b, kHid, kHid, m->h1, m->pb + kOffW2, m->z2, 1, nullptr, s))) return st;
  k_bias_act<<<grid1(B * kHid), 256, 0, s>>>(m->z2, m->p + kOffB2, B, kHid, m->h2);
  if ((st = gemm<false, false>(b, kOut, kHid, m->h2, m->pb + kOffW3, m->y, 1, nullptr, s))) return st;
  k_bias_act<<<grid1(B * kOut), 256, 0, s>>>(m->y, m->p + kOffB3, B, kOut, nullptr);
  XG_CUDA(cudaGetLastError());
  return XG_OK;
}

// backward from m->dy: gradient into g (flat, like the parameters)
int backward(xg_mlp* m, int64_t B, float* g, cudaStream_t s) {
  int st;
  const int b = (int)B;
  const int split = B >= 4096 ? kSplit : 1;
  // layer 3
  if ((st = gemm<true, false>(kHid, kOut, b, m->h2, m->dy, g + kOffW3, split, m->part, s))) return st;
  k_colsum<<<1, 256, 0, s>>>(m->dy, B, kOut, g + kOffB3);
  if ((st = gemm<false, true>(b, kHid, kOut, m->dy, m->pb + kOffW3, m->dh2, 1, nullptr, s))) return st;
  k_act_grad<<<grid1(B * kHid), 256, 0, s>>>(m->dh2, m->z2, B * kHid);
  // layer 2
  if ((st = gemm<true, false>(kHid, kHid, b, m->h1, m->dh2, g + kOffW2, split, m->part, s))) return st;
  k_colsum<<<1, 256, 0, s>>>(m->dh2, B, kHid, g + kOffB2);
  if ((st = gemm<false, true>(b, kHid, kHid, m->dh2, m->pb + kOffW2, m->dh1, 1, nullptr, s))) return st;
  k_act_grad<<<grid1(B * kHid), 256, 0, s>>>(m->dh1, m->z1, B * kHid);
  // layer 1
  if ((st = gemm<true, false>(kIn, kHid, b, m->x, m->dh1, g + kOffW1, split, m->part, s))) return st;
  k_colsum<<<1, 256, 0, s>>>(m->dh1, B, kHid, g + kOffB1);
  XG_CUDA(cudaGetLastError());
  return XG_OK;
}

}  // namespace

extern "C" {

int xg_mlp_param_count(int64_t* out) {
  if (!out) return XG_ERR_ARG;
  *out = kNumParams;
  return XG_OK;
}

int xg_learned_points(double* h_pts) {
  if (!h_pts) return XG_ERR_ARG;
  double p[kOut][3];
  point_set(p);
  std::memcpy(h_pts, p, sizeof(p));
  return XG_OK;
}

int xg_mlp_create(uint64_t seed, xg_mlp** out) {
  if (!out) return XG_ERR_ARG;
  *out = nullptr;
  int st = upload_V();
  if (st) return st;
  auto* m = new xg_mlp();
  // Glorot-uniform weights from a splitmix64 stream, zero biases; the output
  // layer scaled by 0.1 so that the initial correction is small
  std::vector<float> h(kNumParams, 0.f);
  uint64_t s = seed;
  auto fill = [&](int64_t off, int fin, int fout, float scale) {
    const float a = scale * std::sqrt(6.f / (float)(fin + fout));
    for (int64_t i = 0; i < (int64_t)fin * fout; i++) {
      const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
      h[off + i] = (float)((2.0 * u - 1.0) * a);
    }
  };
  fill(kOffW1, kIn, kHid, 1.f);
  fill(kOffW2, kHid, kHid, 1.f);
  fill(kOffW3, kHid, kOut, 0.1f);
  cudaError_t e = cudaMalloc((void**)&m->p, kNumParams * 4);
  if (!e) e = cudaMalloc((void**)&m->pb, kNumParams * 2);
  if (!e) e = cudaMalloc(&m->tcw, kTcPackedBytes);
  if (!e) e = cudaMalloc((void**)&m->err, sizeof(int));
  if (!e) e = cudaMemset(m->err, 0, sizeof(int));
  if (!e) e = cudaMalloc((void**)&m->m, kNumParams * 4);
  if (!e) e = cudaMalloc((void**)&m->v, kNumParams * 4);
  if (!e) e = cudaMalloc((void**)&m->g, kNumParams * 4);
  if (!e) e = cudaMemcpy(m->p, h.data(), kNumParams * 4, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemset(m->m, 0, kNumParams * 4);
  if (!e) e = cudaMemset(m->v, 0, kNumParams * 4);
  if (e) {
    cudaFree(m->p);
    cudaFree(m->pb);
    cudaFree(m->tcw);
    cudaFree(m->err);
    cudaFree(m->m);
    cudaFree(m->v);
    cudaFree(m->g);
    delete m;
    return cuda_fail(e, "xg_mlp_create");
  }
  k_to_bf16<<<grid1(kNumParams), 256>>>(m->p, m->pb, kNumParams);
  if ((st = mlp_tc_pack(m->p, kOffW1, kOffW2, kOffW3, m->tcw, nullptr))) {
    xg_mlp_destroy(m);
    return st;
  }
  *out = m;
  return XG_OK;
}

int xg_mlp_destroy(xg_mlp* m) {
  if (!m) return XG_OK;
  mlp_free_ws(m);
  cudaFree(m->p);
  cudaFree(m->pb);
  cudaFree(m->tcw);
  cudaFree(m->err);
  cudaFree(m->m);
  cudaFree(m->v);
  cudaFree(m->g);
  delete m;
  return XG_OK;
}

int xg_mlp_get_params(const xg_mlp* m, float* d_out, void* stream) {
  if (!m || !d_out) return XG_ERR_ARG;
  XG_CUDA(cudaMemcpyAsync(d_out, m->p, kNumParams * 4, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return XG_OK;
}

int xg_mlp_set_params(xg_mlp* m, const float* d_in, void* stream) {
  if (!m || !d_in) return XG_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  XG_CUDA(cudaMemcpyAsync(m->p, d_in, kNumParams * 4, cudaMemcpyDeviceToDevice, s));
  k_to_bf16<<<grid1(kNumParams), 256, 0, s>>>(m->p, m->pb, kNumParams);
  XG_CUDA(cudaGetLastError());
  return mlp_tc_pack(m->p, kOffW1, kOffW2, kOffW3, m->tcw, s);
}

int xg_mlp_forward(xg_mlp* m, const float* d_x, int64_t B, float* d_y, void* stream) {
  if (!m || !d_x || !d_y || B < 0 || B > kMaxRows) return XG_ERR_ARG;
  if (B == 0) return XG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int st = mlp_reserve(m, B);
  if (st) return st;
  XG_CUDA(cudaMemcpyAsync(m->x, d_x, B * kIn * 4, cudaMemcpyDeviceToDevice, s));
  if ((st = forward(m, B, s))) return st;
  XG_CUDA(cudaMemcpyAsync(d_y, m->y, B * kOut * 4, cudaMemcpyDeviceToDevice, s));
  return XG_OK;
}

int xg_mlp_loss_grad(xg_mlp* m, const float* d_x, const float* d_target, const float* d_scale, int64_t B,
                     float* d_loss, float* d_grad, void* stream) {
  if (!m || !d_x || !d_target || !d_scale || B <= 0 || B > kMaxRows) return XG_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int st = mlp_reserve(m, B);
  if (st) return st;
  XG_CUDA(cudaMemcpyAsync(m->x, d_x, B * kIn * 4, cudaMemcpyDeviceToDevice, s));
  if ((st = forward(m, B, s))) return st;
  k_moment_loss<<<grid1(B), 256, 0, s>>>(m->y, d_target, d_scale, B, m->dy, m->li);
  if (d_loss) k_mean<<<1, 256, 0, s>>>(m->li, B, d_loss);
  if ((st = backward(m, B, d_grad ? d_grad : m->g, s))) return st;
  XG_CUDA(cudaGetLastError());
  return XG_OK;
}

int xg_mlp_adam_step(xg_mlp* m, const float* d_grad, float lr, int64_t t, void* stream) {
  if (!m || t < 1) return XG_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)t), c2 = 1.f - std::pow(b2, (float)t);
  k_adam<<<grid1(kNumParams), 256, 0, s>>>(m->p, d_grad ? d_grad : m->g, m->m, m->v, kNumParams, lr, b1, b2, 1e-8f,
                                           c1, c2);
  k_to_bf16<<<grid1(kNumParams), 256, 0, s>>>(m->p, m->pb, kNumParams);
  XG_CUDA(cudaGetLastError());
  return mlp_tc_pack(m->p, kOffW1, kOffW2, kOffW3, m->tcw, s);
}

int xg_mlp_forward_tc(xg_mlp* m, const float* d_x, int64_t B, float* d_y, void* stream) {
  if (!m || !d_x || !d_y || B < 0) return XG_ERR_ARG;
  return mlp_tc_forward(d_x, B, m->tcw, m->p + kOffB1, m->p + kOffB2, m->p + kOffB3, d_y, m->err,
                        (cudaStream_t)stream);
}

int xg_mlp_check(xg_mlp* m) {
  if (!m) return XG_ERR_ARG;
  int h = 0;
  XG_CUDA(cudaMemcpy(&h, m->err, sizeof(int), cudaMemcpyDeviceToHost));
  XG_CUDA(cudaMemset(m->err, 0, sizeof(int)));
  if (h) set_last_error(std::string("device error: ") + xg_status_string(h));
  return h;
}

int xg_learned_features(const double* d_vals10, int64_t n, float* d_x, void* stream) {
  if (!d_vals10 || !d_x || n < 0) return XG_ERR_ARG;
  if (n == 0) return XG_OK;
  k_features<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(d_vals10, n, d_x);
  XG_CUDA(cudaGetLastError());
  return XG_OK;
}

int xg_learned_moments_tet(xg_mlp* m, const double* d_vals10, int64_t n, double kappa_max, double* d_out35,
                           int32_t* d_nfallback, void* stream) {
  return xg_learned_moments_tet_ex(m, d_vals10, n, kappa_max, -1, d_out35, d_nfallback, stream);
}

int xg_learned_moments_tet_ex(xg_mlp* m, const double* d_vals10, int64_t n, double kappa_max, int plain_subdivlvl,
                              double* d_out35, int32_t* d_nfallback, void* stream) {
  if (!m || !d_vals10 || !d_out35 || n < 0 || n > kMaxRows || plain_subdivlvl > 6) return XG_ERR_ARG;
  if (n == 0) return XG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int st = mlp_reserve(m, n);
  if (st) return st;
  // straight cut part (exact for degree <= 4 on the P1 sub-tetrahedra: order 4)
  if ((st = tet_moments_launch(d_vals10, n, 4, 0, d_out35, nullptr, s, nullptr, nullptr))) return st;
  k_features<<<grid1(n), 256, 0, s>>>(d_vals10, n, m->x);
  // the network on the tensor cores (all three layers per 128-row tile)
  if ((st = mlp_tc_forward(m->x, n, m->tcw, m->p + kOffB1, m->p + kOffB2, m->p + kOffB3, m->y, m->err, s)))
    return st;
  k_add_correction<<<grid1(n), 256, 0, s>>>(m->y, d_vals10, n, d_out35);
  if (kappa_max >= 0.0) {
    // plain (isoparametric, order 8) rule on the elements the network does not take
    XG_CUDA(cudaMemsetAsync(m->count, 0, sizeof(int32_t), s));
    k_fallback_list<<<grid1(n), 256, 0, s>>>(m->x, d_vals10, n, kappa_max, m->list, m->count);
    if (plain_subdivlvl >= 0) {
      // the plain rule is the subdivision rule of that level
      if ((st = ensure_device_rules())) return st;
      if ((st = subdiv_moments_launch(d_vals10, n, plain_subdivlvl, d_out35, m->list, m->count, m->err, s)))
        return st;
    } else if ((st = tet_moments_launch(d_vals10, n, 8, 1, d_out35, nullptr, s, m->list, m->count))) {
      return st;
    }
    if (d_nfallback) XG_CUDA(cudaMemcpyAsync(d_nfallback, m->count, sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  } else if (d_nfallback) {
    XG_CUDA(cudaMemsetAsync(d_nfallback, 0, sizeof(int32_t), s));
  }
  XG_CUDA(cudaGetLastError());
  return XG_OK;
}

}  // extern "C"

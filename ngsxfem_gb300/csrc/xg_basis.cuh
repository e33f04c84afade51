// H1 shape functions of libxg on simplices (NGSolve's own H1 basis is not
// available; the project's basis is stated here and identical on the CPU side):
//   vertex a            : lambda_a
//   edge (s,e), order>=2: lambda_s * lambda_e
//   edge (s,e), order 3 : lambda_s * lambda_e * (lambda_s - lambda_e)
//   face (a,b,c) (3D) / cell (2D), order 3 : lambda_a * lambda_b * lambda_c
// s / e are the edge's end points with the smaller / larger global vertex
// number, which keeps the odd edge functions conforming.  Local order:
// vertices, edges (the dofs of one edge adjacent), faces.
#pragma once

namespace xg {

__host__ __device__ constexpr int ndof_el(int D, int K) {
  return D == 2 ? (K + 1) * (K + 2) / 2 : (K + 1) * (K + 2) * (K + 3) / 6;
}

__host__ __device__ __forceinline__ void local_edge(int D, int j, int& a, int& b) {
  // trig edges (0,1),(0,2),(1,2); tet edges (0,1),(0,2),(0,3),(1,2),(1,3),(2,3)
  if (D == 2) {
    a = j == 2 ? 1 : 0;
    b = j == 0 ? 1 : 2;
  } else {
    const int A[6] = {0, 0, 0, 1, 1, 2};
    const int B[6] = {1, 2, 3, 2, 3, 3};
    a = A[j];
    b = B[j];
  }
}

__host__ __device__ __forceinline__ void local_face(int j, int& a, int& b, int& c) {
  // tet faces (0,1,2),(0,1,3),(0,2,3),(1,2,3)
  a = j == 3 ? 1 : 0;
  b = j <= 1 ? 1 : 2;
  c = j == 0 ? 2 : 3;
}

// Descriptor of local function i: type | a<<4 | b<<8 | c<<12
// type 0 vertex, 1 edge quadratic, 2 edge cubic, 3 face/cell bubble.
template <int D, int K>
__host__ __device__ __forceinline__ int fn_desc(int i, const int* gv) {
  if (i <= D) return 0 | (i << 4);
  int r = i - (D + 1);
  const int nedge = D == 2 ? 3 : 6;
  if (K > 1 && r < nedge * (K - 1)) {
    constexpr int KM = K > 1 ? K - 1 : 1;
    int j = r / KM, m = r % KM;
    int a, b;
    local_edge(D, j, a, b);
    int s = gv[a] < gv[b] ? a : b, e = gv[a] < gv[b] ? b : a;
    return (1 + m) | (s << 4) | (e << 8);
  }
  r -= K > 1 ? nedge * (K - 1) : 0;
  int a = 0, b = 1, c = 2;
  if (D == 3) local_face(r, a, b, c);
  return 3 | (a << 4) | (b << 8) | (c << 12);
}

// value and physical gradient of function `desc` at barycentric lam, with
// physical barycentric gradients g[D+1][D]
template <int D, typename T>
__host__ __device__ __forceinline__ void eval_fn(int desc, const T* lam, const T (*g)[D], T& phi, T* grad) {
  const int type = desc & 15, a = (desc >> 4) & 15, b = (desc >> 8) & 15, c = (desc >> 12) & 15;
  if (type == 0) {
    phi = lam[a];
#pragma unroll
    for (int k = 0; k < D; k++) grad[k] = g[a][k];
  } else if (type == 1) {
    phi = lam[a] * lam[b];
#pragma unroll
    for (int k = 0; k < D; k++) grad[k] = lam[b] * g[a][k] + lam[a] * g[b][k];
  } else if (type == 2) {
    const T q = lam[a] * lam[b], t = lam[a] - lam[b];
    phi = q * t;
#pragma unroll
    for (int k = 0; k < D; k++) {
      T dq = lam[b] * g[a][k] + lam[a] * g[b][k];
      grad[k] = dq * t + q * (g[a][k] - g[b][k]);
    }
  } else {
    phi = lam[a] * lam[b] * lam[c];
#pragma unroll
    for (int k = 0; k < D; k++)
      grad[k] = lam[b] * lam[c] * g[a][k] + lam[a] * lam[c] * g[b][k] + lam[a] * lam[b] * g[c][k];
  }
}

template <int D, typename T>
__host__ __device__ __forceinline__ T eval_fn_value(int desc, const T* lam) {
  const int type = desc & 15, a = (desc >> 4) & 15, b = (desc >> 8) & 15, c = (desc >> 12) & 15;
  if (type == 0) return lam[a];
  if (type == 1) return lam[a] * lam[b];
  if (type == 2) return lam[a] * lam[b] * (lam[a] - lam[b]);
  return lam[a] * lam[b] * lam[c];
}

// Derivatives of order 0..J along a fixed direction of function `desc`, with
// del[i] the derivative of lambda_i along it: every function is a product of
// at most three affine factors (the cubic edge function lambda_a lambda_b
// (lambda_a - lambda_b)), so along x + t n it is a cubic in t whose j-th
// coefficient times j! is the j-th derivative.  out[j], j = 0..J.
template <int J, typename T>
__host__ __device__ __forceinline__ void eval_fn_dir(int desc, const T* lam, const T* del, T* out) {
  const int type = desc & 15, a = (desc >> 4) & 15, b = (desc >> 8) & 15, c = (desc >> 12) & 15;
  T v[3], d[3];
  int m;
  v[0] = lam[a];
  d[0] = del[a];
  if (type == 0) {
    m = 1;
  } else {
    v[1] = lam[b];
    d[1] = del[b];
    m = type == 1 ? 2 : 3;
    if (type == 2) {
      v[2] = lam[a] - lam[b];
      d[2] = del[a] - del[b];
    } else if (type == 3) {
      v[2] = lam[c];
      d[2] = del[c];
    }
  }
  T p0 = 1, p1 = 0, p2 = 0, p3 = 0;  // coefficients of t^0..t^3
  for (int i = 0; i < m; i++) {
    p3 = p3 * v[i] + p2 * d[i];
    p2 = p2 * v[i] + p1 * d[i];
    p1 = p1 * v[i] + p0 * d[i];
    p0 = p0 * v[i];
  }
  out[0] = p0;
  if (J >= 1) out[1] = p1;
  if (J >= 2) out[2] = (T)2 * p2;
  if (J >= 3) out[3] = (T)6 * p3;
}

// FP64 accumulation for the plain path; FP32 with Kahan compensation per
// entry for the mixed path.
template <typename T>
struct Acc;
template <>
struct Acc<double> {
  double s;
  __device__ __forceinline__ void init() { s = 0.0; }
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double get() const { return s; }
};
template <>
struct Acc<float> {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ float get() const { return s; }
};

}  // namespace xg

// Basis change between the two elements of a facet patch.
//
// The extension of an element's H1 function to its neighbour is the same
// polynomial, so its coefficients in the neighbour's basis are exact: they
// follow from the polynomial's values at the neighbour's nodes by the
// hierarchical structure of the basis (xg_basis.cuh), degree by degree:
//   vertex a            value at vertex a
//   edge (a<b), K = 2   4 p(mid) - 2 (p_a + p_b)
//   edge (a<b), K = 3   with q(t) = p - p_a t - p_b (1-t) at t = lambda_a = 1/3, 2/3:
//                       E1: 9/4 (q1 + q2),  E2: 27/4 (q2 - q1)
//   face (a,b,c), K = 3 27 (p(centroid) - (p_a+p_b+p_c)/3 - (E1_ab+E1_ac+E1_bc)/9)
// Coefficients are for the canonical orientation (edge functions oriented by
// local vertex number); the element's own edge orientation is a sign
// (fn_sign) applied by the caller.  Host and device.
#pragma once

#include "xg_basis.cuh"

namespace xg {

// polynomial degree of a function descriptor (fn_desc)
__host__ __device__ __forceinline__ int fn_degree(int desc) {
  const int type = desc & 15;
  return type == 0 ? 1 : (type == 1 ? 2 : 3);
}

// degree of canonical local function k
template <int D, int K>
__host__ __device__ __forceinline__ int canon_degree(int k) {
  if (k <= D) return 1;
  if (K == 2) return 2;
  const int nedge = D == 2 ? 3 : 6;
  const int r = k - (D + 1);
  if (r < 2 * nedge) return (r & 1) ? 3 : 2;
  return 3;
}

// local edge index of the vertex pair a < b (order of local_edge)
template <int D>
__host__ __device__ __forceinline__ int edge_of(int a, int b) {
  if (D == 2) return a == 0 ? b - 1 : 2;
  return a == 0 ? b - 1 : (a == 1 ? b + 1 : 5);
}

// Node n of the canonical node list (vertices; per edge the midpoint (K = 2)
// or the points lambda_a = 1/3, 2/3 (K = 3); face centroids (K = 3)), mapped
// by the barycentric matrix L (entry (i, b) at L[i * si + b * sb]):
// out = L lambda(node).
template <int D, int K, typename T>
__host__ __device__ __forceinline__ void node_image(int n, const T* L, int si, int sb, T* out) {
  constexpr int NE = D == 2 ? 3 : 6;
  if (n <= D) {
#pragma unroll
    for (int i = 0; i <= D; i++) out[i] = L[i * si + n * sb];
    return;
  }
  int r = n - (D + 1);
  if (K >= 2 && r < NE * (K - 1)) {
    const int j = K == 2 ? r : r >> 1;
    int a, b;
    local_edge(D, j, a, b);
    T wa, wb;
    if (K == 2) {
      wa = wb = (T)0.5;
    } else {
      wa = (r & 1) ? (T)(2.0 / 3.0) : (T)(1.0 / 3.0);
      wb = (r & 1) ? (T)(1.0 / 3.0) : (T)(2.0 / 3.0);
    }
#pragma unroll
    for (int i = 0; i <= D; i++) out[i] = wa * L[i * si + a * sb] + wb * L[i * si + b * sb];
    return;
  }
  r -= K >= 2 ? NE * (K - 1) : 0;
  int a = 0, b = 1, c = 2;
  if (D == 3) local_face(r, a, b, c);
#pragma unroll
  for (int i = 0; i <= D; i++) out[i] = (L[i * si + a * sb] + L[i * si + b * sb] + L[i * si + c * sb]) * (T)(1.0 / 3.0);
}

// Canonical hierarchical coefficients of a polynomial of degree deg from its
// values p at the canonical nodes; coefficients of functions of degree above
// deg are exactly 0.  col[k * stride] receives coefficient k.
template <int D, int K, typename T>
__host__ __device__ __forceinline__ void nodal_to_hier(const T* p, int deg, T* col, int stride) {
  constexpr int NE = D == 2 ? 3 : 6;
#pragma unroll
  for (int c = 0; c <= D; c++) col[c * stride] = p[c];
  if constexpr (K == 1) return;
  T alpha[NE];
#pragma unroll
  for (int j = 0; j < NE; j++) {
    int a, b;
    local_edge(D, j, a, b);
    if (K == 2) {
      const int n = D + 1 + j;
      alpha[j] = deg >= 2 ? (T)4 * p[n] - (T)2 * (p[a] + p[b]) : (T)0;
      col[n * stride] = alpha[j];
    } else {
      const int n1 = D + 1 + 2 * j, n2 = n1 + 1;
      const T q1 = p[n1] - (p[a] + (T)2 * p[b]) * (T)(1.0 / 3.0);
      const T q2 = p[n2] - ((T)2 * p[a] + p[b]) * (T)(1.0 / 3.0);
      alpha[j] = deg >= 2 ? (T)2.25 * (q1 + q2) : (T)0;
      col[n1 * stride] = alpha[j];
      col[n2 * stride] = deg >= 3 ? (T)6.75 * (q2 - q1) : (T)0;
    }
  }
  if (K == 3) {
    constexpr int NF = D == 2 ? 1 : 4;
#pragma unroll
    for (int f = 0; f < NF; f++) {
      int a = 0, b = 1, c = 2;
      if (D == 3) local_face(f, a, b, c);
      const int n = D + 1 + 2 * NE + f;
      const T e = alpha[edge_of<D>(a, b)] + alpha[edge_of<D>(a, c)] + alpha[edge_of<D>(b, c)];
      col[n * stride] =
          deg >= 3 ? (T)27 * (p[n] - (p[a] + p[b] + p[c]) * (T)(1.0 / 3.0) - e * (T)(1.0 / 9.0)) : (T)0;
    }
  }
}

}  // namespace xg

// Integer term tables of the cut-element moment kernels (host side).
//
// Every basis function of xg_basis.cuh is a polynomial in the barycentric
// coordinates lambda, so the integrands of the term menu are integer
// combinations of barycentric monomials with element constants in front:
//   MASS  phi_p phi_q,   LAP  sum_ab d_a phi_p d_b phi_q  (x G_ab),
//   PD    phi_p d_b phi_q  (x nu_b or beta_b),   DP  d_b phi_p phi_q  (x nu_b)
// (d_a = derivative by lambda_a).  moment_tables lists, per matrix entry and
// kind, the terms (aux index, monomial index, integer coefficient); the
// moment kernel supplies the monomials' integrals over the cut rule.
#pragma once

#include <array>
#include <cstdint>
#include <initializer_list>
#include <map>
#include <utility>
#include <vector>

#include "xg_basis.cuh"

namespace xg {

__host__ __device__ constexpr int tri_size(int n) { return n * (n + 1) / 2; }
__host__ __device__ inline int tri_index(int p, int q, int n) { return p * n - p * (p - 1) / 2 + (q - p); }

constexpr int kMaxMomDeg = 6;  // 2K for K <= 3

__host__ __device__ constexpr int pair_count(int d) { return (d + 1) * (d + 2) / 2; }
__host__ __device__ constexpr int mono_count(int nvar, int d) {
  // number of monomials of degree <= d in nvar variables: binom(d + nvar, nvar)
  return nvar == 3 ? (d + 1) * (d + 2) * (d + 3) / 6 : (d + 1) * (d + 2) * (d + 3) * (d + 4) / 24;
}

using Expo = std::array<int, 4>;
using Poly = std::map<Expo, long long>;

// graded enumeration of the monomials of nvar barycentric variables up to kMaxMomDeg
inline std::vector<Expo> monomials(int nvar) {
  std::vector<Expo> out;
  for (int d = 0; d <= kMaxMomDeg; d++)
    for (int e0 = d; e0 >= 0; e0--)
      for (int e1 = d - e0; e1 >= 0; e1--) {
        if (nvar == 3) {
          out.push_back({e0, e1, d - e0 - e1, 0});
        } else {
          for (int e2 = d - e0 - e1; e2 >= 0; e2--) out.push_back({e0, e1, e2, d - e0 - e1 - e2});
        }
      }
  return out;
}

inline int pair_index(int a, int b) { return (a + b) * (a + b + 1) / 2 + b; }

inline Poly basis_poly(int desc) {
  const int type = desc & 15, a = (desc >> 4) & 15, b = (desc >> 8) & 15, c = (desc >> 12) & 15;
  auto mono = [](std::initializer_list<int> vars) {
    Expo e = {0, 0, 0, 0};
    for (int v : vars) e[v]++;
    return e;
  };
  Poly P;
  if (type == 0) {
    P[mono({a})] = 1;
  } else if (type == 1) {
    P[mono({a, b})] = 1;
  } else if (type == 2) {
    P[mono({a, a, b})] += 1;
    P[mono({a, b, b})] -= 1;
  } else {
    P[mono({a, b, c})] = 1;
  }
  return P;
}

inline Poly poly_mul(const Poly& x, const Poly& y) {
  Poly r;
  for (const auto& [ex, cx] : x)
    for (const auto& [ey, cy] : y) {
      Expo e;
      for (int k = 0; k < 4; k++) e[k] = ex[k] + ey[k];
      r[e] += cx * cy;
    }
  return r;
}

inline Poly poly_diff(const Poly& x, int v) {
  Poly r;
  for (const auto& [e, c] : x)
    if (e[v] > 0) {
      Expo f = e;
      f[v]--;
      r[f] += c * e[v];
    }
  return r;
}

// Integer term tables for the canonical orientation (local vertex numbers as
// global numbers; cubic edge functions flip with fn_sign): per entry (p, q)
// and kind, the terms (aux, monomial, coefficient) of
//   MASS phi_p phi_q, LAP sum_ab d_a phi_p d_b phi_q, PD phi_p d_b phi_q, DP d_b phi_p phi_q.
template <int D, int K>
void moment_tables(bool sym, std::vector<int32_t> (&ptr)[4], std::vector<int32_t> (&ix)[4],
                   std::vector<double> (&cf)[4]) {
  constexpr int N = ndof_el(D, K);
  const int E = sym ? tri_size(N) : N * N;
  const std::vector<Expo> ms = monomials(D + 1);
  std::map<Expo, int> mindex;
  for (size_t m = 0; m < ms.size(); m++) mindex[ms[m]] = (int)m;
  int gv[4] = {0, 1, 2, 3};
  std::vector<Poly> phi(N);
  std::vector<std::array<Poly, 4>> dphi(N);
  for (int i = 0; i < N; i++) {
    phi[i] = basis_poly(fn_desc<D, K>(i, gv));
    for (int a = 0; a <= D; a++) dphi[i][a] = poly_diff(phi[i], a);
  }
  for (int k = 0; k < 4; k++) {
    ptr[k].assign(1, 0);
    ix[k].clear();
    cf[k].clear();
  }
  for (int k = 0; k < E; k++) {
    int p, q;
    if (sym) {
      p = 0;
      int rem = k;
      while (rem >= N - p) {
        rem -= N - p;
        p++;
      }
      q = p + rem;
    } else {
      p = k / N;
      q = k % N;
    }
    std::map<std::pair<int, int>, long long> t[4];
    for (const auto& [e, c] : poly_mul(phi[p], phi[q])) t[0][{0, mindex.at(e)}] += c;
    for (int a = 0; a <= D; a++)
      for (int b = 0; b <= D; b++)
        for (const auto& [e, c] : poly_mul(dphi[p][a], dphi[q][b]))
          t[1][{tri_index(std::min(a, b), std::max(a, b), D + 1), mindex.at(e)}] += c;
    for (int b = 0; b <= D; b++) {
      for (const auto& [e, c] : poly_mul(phi[p], dphi[q][b])) t[2][{b, mindex.at(e)}] += c;
      for (const auto& [e, c] : poly_mul(dphi[p][b], phi[q])) t[3][{b, mindex.at(e)}] += c;
    }
    for (int kind = 0; kind < 4; kind++) {
      for (const auto& [key, c] : t[kind])
        if (c != 0) {
          ix[kind].push_back(key.second | key.first << 16);
          cf[kind].push_back((double)c);
        }
      ptr[kind].push_back((int32_t)ix[kind].size());
    }
  }
}

}  // namespace xg

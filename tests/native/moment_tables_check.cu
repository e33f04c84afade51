// Host check of the integer term tables of the cut-element moment kernels
// (ngsxfem_gb300/csrc/xg_moments.cuh): at random barycentric points the terms
// of every entry reproduce the integrands evaluated from the basis directly
// (values and lambda-derivatives from eval_fn), for D = 2, 3, K = 1..3, packed
// and full entry orders.  Prints the worst relative error; exit status 1
// above 1e-12.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>

#include "xg_moments.cuh"

using namespace xg;

// value and derivatives d_a phi (a = 0..D) of canonical function i at lam
template <int D, int K>
static void fn_and_dlam(int i, const double* lam, double& phi, double* d) {
  int gv[4] = {0, 1, 2, 3};
  const int desc = fn_desc<D, K>(i, gv);
  double g[D + 1][D], grad[D];
  for (int a = 0; a <= D; a++)
    for (int k = 0; k < D; k++) g[a][k] = (a == k) ? 1.0 : 0.0;
  eval_fn<D, double>(desc, lam, g, phi, grad);
  for (int k = 0; k < D; k++) d[k] = grad[k];
  for (int a = 0; a <= D; a++)
    for (int k = 0; k < D; k++) g[a][k] = (a == D && k == 0) ? 1.0 : 0.0;
  eval_fn<D, double>(desc, lam, g, phi, grad);
  d[D] = grad[0];
}

template <int D, int K>
static double check(bool sym, std::mt19937_64& rng) {
  constexpr int N = ndof_el(D, K);
  std::vector<int32_t> ptr[4], ix[4];
  std::vector<double> cf[4];
  moment_tables<D, K>(sym, ptr, ix, cf);
  const std::vector<Expo> ms = monomials(D + 1);
  std::uniform_real_distribution<double> U(-1, 1);
  double G[D + 1][D + 1], w[D + 1];
  for (int a = 0; a <= D; a++) {
    w[a] = U(rng);
    for (int b = a; b <= D; b++) G[a][b] = G[b][a] = U(rng);
  }
  double worst = 0;
  for (int t = 0; t < 8; t++) {
    double lam[4] = {0, 0, 0, 0};
    for (int a = 0; a <= D; a++) lam[a] = U(rng);
    double mono[210];
    for (size_t m = 0; m < ms.size(); m++) {
      double v = 1;
      for (int a = 0; a <= D; a++)
        for (int e = 0; e < ms[m][a]; e++) v *= lam[a];
      mono[m] = v;
    }
    double phi[N], d[N][4];
    for (int i = 0; i < N; i++) fn_and_dlam<D, K>(i, lam, phi[i], d[i]);
    const int E = sym ? tri_size(N) : N * N;
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
      double ref[4] = {phi[p] * phi[q], 0, 0, 0};
      for (int a = 0; a <= D; a++) {
        for (int b = 0; b <= D; b++) ref[1] += G[a][b] * d[p][a] * d[q][b];
        ref[2] += w[a] * phi[p] * d[q][a];
        ref[3] += w[a] * d[p][a] * phi[q];
      }
      for (int kind = 0; kind < 4; kind++) {
        double got = 0;
        for (int u = ptr[kind][k]; u < ptr[kind][k + 1]; u++) {
          const int x = ix[kind][u], aux = x >> 16, m = x & 0xffff;
          double f = 1;
          if (kind == 1) {
            int a = 0;
            while (tri_index(a, D, D + 1) < aux) a++;  // packed (a <= b) -> (a, b)
            const int b = a + (aux - tri_index(a, a, D + 1));
            f = G[a][b];
          } else if (kind >= 2) {
            f = w[aux];
          }
          got += cf[kind][u] * f * mono[m];
        }
        worst = std::max(worst, std::fabs(got - ref[kind]) / (1 + std::fabs(ref[kind])));
      }
    }
  }
  return worst;
}

int main() {
  std::mt19937_64 rng(11);
  double w = 0;
  for (int r = 0; r < 20; r++)
    for (int sym = 0; sym < 2; sym++) {
      w = std::max(w, check<2, 1>(sym, rng));
      w = std::max(w, check<2, 2>(sym, rng));
      w = std::max(w, check<2, 3>(sym, rng));
      w = std::max(w, check<3, 1>(sym, rng));
      w = std::max(w, check<3, 2>(sym, rng));
      w = std::max(w, check<3, 3>(sym, rng));
    }
  std::printf("worst relative error %.3e\n", w);
  return w < 1e-12 ? 0 : 1;
}

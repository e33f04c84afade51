// Host check of the facet-patch basis change (ngsxfem_gb300/csrc/xg_patch.cuh):
// for random affine maps between two simplices and every function of the
// second element (random edge orientation), the canonical hierarchical
// coefficients from node values reproduce the function on the first element.
// Prints the worst relative error; exit status 1 above 1e-10.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>

#include "xg_patch.cuh"

using namespace xg;

template <int D, int K>
static double check(std::mt19937_64& g) {
  constexpr int N = ndof_el(D, K);
  std::uniform_real_distribution<double> U(-1, 1);
  double L[D + 1][D + 1];
  for (int b = 0; b <= D; b++) {
    double s = 0;
    for (int i = 0; i < D; i++) {
      L[i][b] = U(g);
      s += L[i][b];
    }
    L[D][b] = 1 - s;
  }
  int gv2[4] = {0, 1, 2, 3}, gc[4] = {0, 1, 2, 3};
  std::shuffle(gv2, gv2 + D + 1, g);
  double worst = 0;
  for (int j = 0; j < N; j++) {
    const int desc = fn_desc<D, K>(j, gv2);
    double p[N], col[N];
    for (int n = 0; n < N; n++) {
      double lam2[4];
      node_image<D, K, double>(n, &L[0][0], D + 1, 1, lam2);
      p[n] = eval_fn_value<D, double>(desc, lam2);
    }
    nodal_to_hier<D, K, double>(p, fn_degree(desc), col, 1);
    for (int t = 0; t < 20; t++) {
      double lam[4], s = 0, lam2[4] = {0, 0, 0, 0};
      for (int k = 0; k < D; k++) {
        lam[k] = U(g);
        s += lam[k];
      }
      lam[D] = 1 - s;
      for (int i = 0; i <= D; i++)
        for (int b = 0; b <= D; b++) lam2[i] += L[i][b] * lam[b];
      const double ref = eval_fn_value<D, double>(desc, lam2);
      double got = 0;
      for (int k = 0; k < N; k++) got += col[k] * eval_fn_value<D, double>(fn_desc<D, K>(k, gc), lam);
      worst = std::max(worst, std::fabs(got - ref) / (1 + std::fabs(ref)));
    }
  }
  return worst;
}

int main() {
  std::mt19937_64 g(5);
  double w = 0;
  for (int r = 0; r < 200; r++) {
    w = std::max(w, check<2, 1>(g));
    w = std::max(w, check<2, 2>(g));
    w = std::max(w, check<2, 3>(g));
    w = std::max(w, check<3, 1>(g));
    w = std::max(w, check<3, 2>(g));
    w = std::max(w, check<3, 3>(g));
  }
  std::printf("worst relative error %.3e\n", w);
  return w < 1e-10 ? 0 : 1;
}

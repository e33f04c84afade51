// Host build of the boundary linear-form element code (csrc/xg_lfbnd.cuh,
// the body of the GPU kernel k_lf_bnd) as a shared library: the test
// (tests/test_oracle_bnd.py) gathers its element vectors with the oracle
// space's dof numbering and compares the result with orc_linear_form.  The
// rule table is the oracle's (orc_base_rule), as in the other native checks.
#include <cstdio>
#include <vector>

#include "xg_lfbnd.cuh"

extern "C" int orc_base_rule(int d, int p, double* pts, double* wts, int maxpts);

namespace {

xg::RuleTable g_tab;
bool g_filled = false;

void fill_table() {
  if (g_filled) return;
  int n = 0;
  for (int d = 0; d < 4; d++)
    for (int p = 0; p <= xg::kMaxOrder; p++) {
      double pts[3 * 256], w[256];
      const int c = orc_base_rule(d, p, pts, w, 256);
      g_tab.off[d][p] = n;
      g_tab.cnt[d][p] = c;
      for (int i = 0; i < c; i++) {
        for (int k = 0; k < 3; k++) g_tab.x[n + i][k] = pts[3 * i + k];
        g_tab.w[n + i] = w[i];
      }
      n += c;
    }
  g_filled = true;
}

template <int D, int K>
int run(int64_t nbnd, const double* xv, const int* gv, const double* xb, const double* lb, const xg_lterm* terms,
        int nterms, double* out) {
  constexpr int N = xg::ndof_el(D, K);
  for (int64_t b = 0; b < nbnd; b++) {
    double v[D + 1][3], w[D][3];
    for (int i = 0; i <= D; i++)
      for (int c = 0; c < 3; c++) v[i][c] = xv[(b * (D + 1) + i) * 3 + c];
    for (int i = 0; i < D; i++)
      for (int c = 0; c < 3; c++) w[i][c] = xb[(b * D + i) * 3 + c];
    const int st = xg::lfb::element_vector<D, K>(&g_tab, v, gv + b * (D + 1), w, lb + b * D, terms, nterms, b,
                                                 out + b * N);
    if (st) return st;
  }
  return 0;
}

}  // namespace

// per BND element b: owner vertices xv[b][D+1][3] with ids gv[b][D+1],
// boundary vertices xb[b][D][3] with level-set values lb[b][D]; out[b][N]
extern "C" int lfb_element_vectors(int D, int K, int64_t nbnd, const double* xv, const int* gv, const double* xb,
                                   const double* lb, const xg_lterm* terms, int nterms, double* out) {
  fill_table();
  if (D == 2 && K == 1) return run<2, 1>(nbnd, xv, gv, xb, lb, terms, nterms, out);
  if (D == 2 && K == 2) return run<2, 2>(nbnd, xv, gv, xb, lb, terms, nterms, out);
  if (D == 2 && K == 3) return run<2, 3>(nbnd, xv, gv, xb, lb, terms, nterms, out);
  if (D == 3 && K == 1) return run<3, 1>(nbnd, xv, gv, xb, lb, terms, nterms, out);
  if (D == 3 && K == 2) return run<3, 2>(nbnd, xv, gv, xb, lb, terms, nterms, out);
  if (D == 3 && K == 3) return run<3, 3>(nbnd, xv, gv, xb, lb, terms, nterms, out);
  return -1;
}

// Host check of the subdivision rules of csrc/xg_subdiv.cuh (the code the GPU
// kernels run) against the oracle's restatement of CutIntegrationRule with
// subdivlvl (orc_subdiv_rule, oracle/xg_oracle.cpp).  Both read the oracle's
// base rules; the oracle cuts in reference coordinates and maps, the device
// code cuts the physical simplex, so points and weights agree to rounding
// (1e-12 relative), in the same order.  Cases: random triangles and
// tetrahedra, level sets of order 1..3 with random coefficients (through the
// element), NEG / POS / IF, levels 0..3, orders 0, 2, 4.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "xg_subdiv.cuh"

extern "C" {
int orc_base_rule(int d, int p, double* pts, double* wts, int maxpts);
struct orc_space;
orc_space* orc_space_create(int D, int nv, const double* coords, int ne, const int32_t* elv, int order);
void orc_space_destroy(orc_space*);
int orc_space_info(const orc_space*, int64_t* out);
int orc_space_el_dofs(const orc_space*, int32_t* out);
int orc_subdiv_rule(const orc_space* s, const double* lset_coefs, int e, int dt, int order, int subdivlvl,
                    double* pts, double* wts, int maxpts);
}

namespace xg {
static RuleTable g_tab;
const RuleTable& host_rules() { return g_tab; }
}  // namespace xg

static void fill_table() {
  int n = 0;
  for (int d = 0; d < 4; d++)
    for (int p = 0; p <= xg::kMaxOrder; p++) {
      double pts[3 * 256], w[256];
      const int c = orc_base_rule(d, p, pts, w, 256);
      xg::g_tab.off[d][p] = n;
      xg::g_tab.cnt[d][p] = c;
      for (int i = 0; i < c; i++) {
        for (int k = 0; k < 3; k++) xg::g_tab.x[n + i][k] = pts[3 * i + k];
        xg::g_tab.w[n + i] = w[i];
      }
      n += c;
    }
}

struct Collect {
  std::vector<double> p, w;
  void operator()(const double* x, double ww) {
    p.push_back(x[0]);
    p.push_back(x[1]);
    p.push_back(x[2]);
    w.push_back(ww);
  }
};

static int g_fail = 0, g_cases = 0, g_points = 0;

template <int D, int K>
static void check(std::mt19937_64& rng) {
  std::normal_distribution<double> nd(0.0, 1.0);
  std::uniform_real_distribution<double> ud(-0.3, 0.3);
  double coords[12];
  for (int v = 0; v <= D; v++)
    for (int c = 0; c < D; c++) coords[v * D + c] = (v > 0 && c == v - 1 ? 1.0 : 0.0) + ud(rng);
  int32_t elv[4] = {0, 1, 2, 3};
  orc_space* s = orc_space_create(D, D + 1, coords, 1, elv, K);
  int64_t info[5];
  orc_space_info(s, info);
  const int ndof = (int)info[0], n = xg::ndof_el(D, K);
  std::vector<int32_t> eld(n);
  orc_space_el_dofs(s, eld.data());
  std::vector<double> coef(ndof);
  for (int i = 0; i < ndof; i++) coef[i] = nd(rng) * (i <= D ? 1.0 : 0.5);
  xg::sd::Elem<D, K> el;
  const int gv[4] = {0, 1, 2, 3};
  for (int r = 0; r < 3; r++) {
    el.x0[r] = r < D ? coords[D * D + r] : 0.0;
    for (int c = 0; c < 3; c++) el.F[r][c] = (r < D && c < D) ? coords[c * D + r] - coords[D * D + r] : 0.0;
  }
  for (int i = 0; i < n; i++) {
    el.coef[i] = coef[eld[i]];
    el.desc[i] = xg::fn_desc<D, K>(i, gv);
  }
  static std::vector<double> op(3 * 100000), ow(100000);
  for (int dt = 0; dt < 3; dt++)
    for (int L = 0; L <= 3; L++)
      for (int order : {0, 2, 4}) {
        Collect c;
        const int st = xg::sd::element_rule<D, K>(&xg::g_tab, el, dt, order, L, c);
        const int on = orc_subdiv_rule(s, coef.data(), 0, dt, order, L, op.data(), ow.data(), 100000);
        g_cases++;
        bool ok = true;
        if (on < 0) {
          ok = st != 0;
        } else {
          ok = st == 0 && (int)c.w.size() == on;
          double scale = 1e-300;
          for (int q = 0; ok && q < on; q++) scale = std::fmax(scale, std::fabs(ow[q]));
          for (int q = 0; ok && q < on; q++) {
            if (std::fabs(c.w[q] - ow[q]) > 1e-12 * scale) ok = false;
            for (int r = 0; r < D; r++)
              if (std::fabs(c.p[3 * q + r] - op[3 * q + r]) > 1e-12) ok = false;
          }
          g_points += on;
        }
        if (!ok) {
          if (g_fail < 10)
            std::printf("mismatch D=%d K=%d dt=%d L=%d order=%d: %zu vs %d points (status %d)\n", D, K, dt, L, order,
                        c.w.size(), on, st);
          g_fail++;
        }
      }
  orc_space_destroy(s);
}

int main() {
  fill_table();
  std::mt19937_64 rng(20261204);
  for (int t = 0; t < 60; t++) {
    check<2, 1>(rng);
    check<2, 2>(rng);
    check<2, 3>(rng);
    check<3, 1>(rng);
    check<3, 2>(rng);
    check<3, 3>(rng);
  }
  std::printf("%d cases, %d points, %d mismatches\n", g_cases, g_points, g_fail);
  return g_fail ? 1 : 0;
}

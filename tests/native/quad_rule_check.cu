// Host check of the quadrilateral / hexahedron cut rules of csrc/xg_quadcut.cuh
// (the code the rule and Integrate kernels run) against the oracle's
// restatement of LevelsetCutQuadrilateral (oracle/xg_oracle_quad.cpp).
// Both read the oracle's base rules, so points and weights must agree to the
// bit: the same count, the same order, the same status.  Cases: random vertex
// values, planar and axis-aligned cuts, vertices on the level set (after the
// +1e-14 perturbation), every order 0..8, NEG / POS / IF, the three swap
// policies, D = 2 and 3.
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "xg_quadcut.cuh"

extern "C" int orc_base_rule(int d, int p, double* pts, double* wts, int maxpts);
extern "C" int orc_quad_cut_rule(int D, const double* lset_vals, int dt, int order, int policy, double* pts,
                                 double* wts, int maxpts);

namespace xg {
// the rule table filled from the oracle's rules (the library's own table is
// built by xg_host.cpp and compared with the oracle's elsewhere)
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

static int g_fail = 0, g_cases = 0, g_points = 0, g_errors = 0;

static void check(int D, const double* v, int dt, int order, int pol) {
  Collect c;
  const int st = D == 2 ? xg::qc::tp_cut_rule<2>(&xg::g_tab, v, dt, order, pol, c)
                        : xg::qc::tp_cut_rule<3>(&xg::g_tab, v, dt, order, pol, c);
  static std::vector<double> op(3 * 20000), ow(20000);
  const int on = orc_quad_cut_rule(D, v, dt, order, pol, op.data(), ow.data(), 20000);
  g_cases++;
  // the oracle: count, -1 no rule, -(status)-1 error
  const int ost = on >= 0 ? 0 : (on == -1 ? -1 : -on - 1);
  bool ok = st == ost;
  if (ok && st == 0) {
    ok = (int)c.w.size() == on && std::memcmp(c.w.data(), ow.data(), sizeof(double) * on) == 0 &&
         std::memcmp(c.p.data(), op.data(), sizeof(double) * 3 * on) == 0;
    g_points += on;
  }
  if (st > 0) g_errors++;
  if (!ok) {
    if (g_fail < 10) {
      std::printf("MISMATCH D=%d dt=%d order=%d pol=%d status %d/%d count %zu/%d vals", D, dt, order, pol, st, ost,
                  c.w.size(), on);
      for (int i = 0; i < (D == 2 ? 4 : 8); i++) std::printf(" %.17g", v[i]);
      std::printf("\n");
    }
    g_fail++;
  }
}

static void all(int D, const double* v) {
  for (int order = 0; order <= 8; order++)
    for (int dt = 0; dt < 3; dt++)
      for (int pol = 0; pol < 3; pol++) check(D, v, dt, order, pol);
}

static double perturb(double d) { return std::fabs(d) < 1e-14 ? 1e-14 : d; }

int main() {
  fill_table();
  std::mt19937_64 rng(20261204);
  std::normal_distribution<double> nd(0.0, 1.0);
  std::uniform_real_distribution<double> ud(-1.0, 1.0);
  const double cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  for (int D = 2; D <= 3; D++) {
    const int nv = D == 2 ? 4 : 8;
    double v[8];
    for (int t = 0; t < 300; t++) {  // random multilinear level sets
      for (int i = 0; i < nv; i++) v[i] = nd(rng);
      all(D, v);
    }
    for (int t = 0; t < 200; t++) {  // planar level sets a + b.x
      const double a = ud(rng), b[3] = {ud(rng), ud(rng), ud(rng)};
      for (int i = 0; i < nv; i++) v[i] = perturb(a + b[0] * cx[i] + b[1] * cy[i] + (D == 3 ? b[2] * cz[i] : 0.0));
      all(D, v);
    }
    for (int t = 0; t < 100; t++) {  // axis-aligned and vertex-touching cuts
      const int ax = t % D;
      const double s = (t / D) % 5 == 0 ? 0.5 : ud(rng) * 0.5 + 0.5;
      for (int i = 0; i < nv; i++) {
        const double c = ax == 0 ? cx[i] : (ax == 1 ? cy[i] : cz[i]);
        v[i] = perturb((c - s) * (t % 2 ? 1.0 : -1.0) + (t % 3 == 0 ? 1e-3 * cy[i] : 0.0));
      }
      all(D, v);
    }
  }
  std::printf("%d cases, %d points, %d error statuses, %d mismatches\n", g_cases, g_points, g_errors, g_fail);
  return g_fail ? 1 : 0;
}

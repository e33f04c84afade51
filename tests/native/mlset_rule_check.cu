// Host check of the multi-level-set rules of csrc/xg_mlset.cuh (the code the
// GPU kernels run) against the oracle's restatement of
// StraightCutsIntegrationRule / CreateMultiLevelsetCutIntegrationRule
// (oracle/xg_oracle_mlset.cpp).  Both read the oracle's base rules: points,
// weights, counts and statuses must agree to the bit.  Cases: random
// triangles and tetrahedra, 1..5 random linear level sets, level sets through
// element vertices, random unions of domain tuples with NEG / POS / IF
// entries (codimension 0..3), orders 0..5.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "xg_mlset.cuh"

extern "C" int orc_base_rule(int d, int p, double* pts, double* wts, int maxpts);
extern "C" double orc_bnd_element_integral(int D, const double* xv, const double* l, int dt, int order, int ex,
                                           int ey, int ez, int* status);
extern "C" int orc_mlset_cut_rule(int D, const double* elc, int M, const double* lsets, int ntup, const int* dts,
                                  int order, double* pts, double* wts, int maxpts);

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

static int g_fail = 0, g_cases = 0, g_points = 0, g_errors = 0, g_norule = 0;

template <int D>
static void check(const double (*xv)[3], int M, const double (*lv)[D + 1], const std::vector<int>& dts, int order) {
  xg::ml::MlDesc md;
  md.M = M;
  md.ntup = (int)dts.size() / M;
  for (size_t i = 0; i < dts.size(); i++) md.dt[i] = (int8_t)dts[i];
  xg::ml::AGeo g;
  xg::ml::make_ageo<D>(xv, g);
  Collect c;
  int npts = 0;
  const int st = xg::ml::element_rule<D>(&xg::g_tab, g, md.M, md.ntup, md.dt, lv, order, c, &npts);
  double elc[12], lsets[8 * 4];
  for (int v = 0; v <= D; v++)
    for (int i = 0; i < D; i++) elc[v * D + i] = xv[v][i];
  for (int m = 0; m < M; m++)
    for (int v = 0; v <= D; v++) lsets[m * (D + 1) + v] = lv[m][v];
  static std::vector<double> op(3 * 40000), ow(40000);
  const int on = orc_mlset_cut_rule(D, elc, M, lsets, md.ntup, dts.data(), order, op.data(), ow.data(), 40000);
  g_cases++;
  bool ok;
  if (on < -1) {
    ok = st == -on - 1;
    g_errors++;
  } else if (on == -1) {
    ok = st == 0 && npts == 0;
    g_norule++;
  } else {
    ok = st == 0 && npts == on && (int)c.w.size() == on &&
         std::memcmp(c.w.data(), ow.data(), sizeof(double) * on) == 0 &&
         std::memcmp(c.p.data(), op.data(), sizeof(double) * 3 * on) == 0;
    g_points += on;
  }
  if (!ok) {
    if (g_fail < 10)
      std::printf("MISMATCH D=%d M=%d ntup=%d order=%d status %d oracle %d count %zu\n", D, M, md.ntup, order, st, on,
                  c.w.size());
    g_fail++;
  }
}

template <int D>
static void run(std::mt19937_64& rng, int ncase) {
  std::normal_distribution<double> nd(0.0, 1.0);
  std::uniform_int_distribution<int> um(1, 5), ut(1, 4), udt(0, 2), uord(0, 5);
  for (int t = 0; t < ncase; t++) {
    double xv[4][3] = {};
    for (int v = 0; v <= D; v++)
      for (int i = 0; i < D; i++) xv[v][i] = (v < D && v == i ? 1.0 : 0.0) + 0.3 * nd(rng);
    const int M = um(rng);
    double lv[8][D + 1];
    for (int m = 0; m < M; m++) {
      for (int v = 0; v <= D; v++) lv[m][v] = nd(rng);
      if (t % 5 == 0) lv[m][m % (D + 1)] = 1e-14;  // a vertex on the level set (perturbed)
    }
    const int nt = ut(rng);
    std::vector<int> dts;
    for (int k = 0; k < nt * M; k++) dts.push_back(udt(rng));
    if (t % 3 == 0)  // a volume tuple with the element's own signs, so uncut parts occur
      for (int m = 0; m < M; m++) dts[m] = lv[m][0] < 0 ? XG_NEG : XG_POS;
    check<D>(xv, M, lv, dts, uord(rng));
  }
}

// boundary elements: the share of random segments in 2D and triangles in 3D
template <int D>
static void run_bnd(std::mt19937_64& rng, int ncase) {
  std::normal_distribution<double> nd(0.0, 1.0);
  std::uniform_int_distribution<int> udt(0, 2), uord(0, 5), uex(0, 2);
  for (int t = 0; t < ncase; t++) {
    double xv[3][3] = {}, l[3];
    for (int v = 0; v < D; v++) {
      for (int i = 0; i < D; i++) xv[v][i] = nd(rng);
      l[v] = nd(rng);
    }
    const int dt = udt(rng), order = uord(rng), ex = uex(rng), ey = uex(rng), ez = uex(rng);
    double got = 0.0;
    auto emit = [&](const double* x, double w, double meas) {
      double fv = 1.0;
      for (int k = 0; k < ex; k++) fv *= x[0];
      double fy = 1.0;
      for (int k = 0; k < ey; k++) fy *= x[1];
      double fz = 1.0;
      if (D == 3)
        for (int k = 0; k < ez; k++) fz *= x[2];
      got += w * meas * (fv * fy * fz);
    };
    const int st = xg::ml::bnd_rule<D>(&xg::g_tab, xv, l, dt, order, emit);
    int ost = 0;
    const double ref = orc_bnd_element_integral(D, &xv[0][0], l, dt, order, ex, ey, ez, &ost);
    g_cases++;
    const bool ok = st == ost && (st || std::fabs(got - ref) <= 1e-13 * std::max(1.0, std::fabs(ref)));
    if (!ok) {
      if (g_fail < 10) std::printf("BND MISMATCH D=%d dt=%d order=%d: %g vs %g (status %d/%d)\n", D, dt, order, got, ref, st, ost);
      g_fail++;
    }
  }
}

int main() {
  fill_table();
  std::mt19937_64 rng(20261204);
  run<2>(rng, 20000);
  run<3>(rng, 20000);
  run_bnd<2>(rng, 5000);
  run_bnd<3>(rng, 5000);
  std::printf("%d cases, %d points, %d no-rule, %d error statuses, %d mismatches\n", g_cases, g_points, g_norule,
              g_errors, g_fail);
  return g_fail ? 1 : 0;
}

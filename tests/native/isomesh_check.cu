// Host check of the mesh-level isoparametric integration of
// csrc/xg_isomesh.cuh (the code the GPU kernels run, here on the host with
// the same three steps: per-element contributions, per-edge averages in
// element order, mapped rules) against the oracle's
// orc_iso_integrate_mesh (oracle/xg_oracle_iso.cpp, pinned on the reference's
// curved-circle test).  Both read the oracle's base rules.  Bar: 1e-12
// relative (the two cut rules take different but equivalent operation orders
// for the interface factor; the sums run in different orders).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "xg_isomesh.cuh"

extern "C" int orc_base_rule(int d, int p, double* pts, double* wts, int maxpts);
extern "C" double orc_iso_integrate_mesh(int D, int nv, const double* coords, int ne, const int32_t* elv,
                                         const double* p2vals, int dt, int order, double threshold, int deform,
                                         int* nonconv);

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

struct Mesh {
  int D, nv, ne;
  std::vector<double> xyz;   // nv x D
  std::vector<int32_t> elv;  // ne x (D+1)
};

static Mesh structured(int D, int n, double lo, double hi) {
  Mesh m;
  m.D = D;
  const int np = n + 1;
  m.nv = D == 2 ? np * np : np * np * np;
  for (int k = 0; k < (D == 3 ? np : 1); k++)
    for (int j = 0; j < np; j++)
      for (int i = 0; i < np; i++) {
        m.xyz.push_back(lo + (hi - lo) * i / n);
        m.xyz.push_back(lo + (hi - lo) * j / n);
        if (D == 3) m.xyz.push_back(lo + (hi - lo) * k / n);
      }
  auto id = [&](int i, int j, int k) { return i + np * (j + np * k); };
  for (int k = 0; k < (D == 3 ? n : 1); k++)
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        if (D == 2) {
          const int a = id(i, j, 0), b = id(i + 1, j, 0), c = id(i + 1, j + 1, 0), d = id(i, j + 1, 0);
          const int t[2][3] = {{a, b, c}, {a, c, d}};
          for (auto& tt : t) m.elv.insert(m.elv.end(), tt, tt + 3);
        } else {
          const int base = id(i, j, k), v111 = id(i + 1, j + 1, k + 1);
          const int step[3] = {1, np, np * np};
          const int perm[6][2] = {{0, 1}, {0, 2}, {1, 0}, {1, 2}, {2, 0}, {2, 1}};
          for (auto& p : perm) {
            const int t[4] = {base, base + step[p[0]], base + step[p[0]] + step[p[1]], v111};
            m.elv.insert(m.elv.end(), t, t + 4);
          }
        }
      }
  m.ne = (int)m.elv.size() / (D + 1);
  return m;
}

template <int D>
static double run(const Mesh& m, const std::vector<double>& p2, int dt, int order, double threshold, int deform) {
  constexpr int NE = D == 2 ? 3 : 6, NN = (D + 1) * (D + 2) / 2;
  // edges: unique (min, max) vertex pairs in lexicographic order
  std::vector<uint64_t> keys((size_t)m.ne * NE);
  for (int e = 0; e < m.ne; e++)
    for (int j = 0; j < NE; j++) {
      int a, b;
      xg::iso::edge_ends<D>(j, a, b);
      uint64_t va = (uint32_t)m.elv[e * (D + 1) + a], vb = (uint32_t)m.elv[e * (D + 1) + b];
      if (va > vb) std::swap(va, vb);
      keys[(size_t)e * NE + j] = (va << 32) | vb;
    }
  std::vector<uint64_t> uk(keys);
  std::sort(uk.begin(), uk.end());
  uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
  std::vector<int> eid(keys.size());
  for (size_t i = 0; i < keys.size(); i++) eid[i] = (int)(std::lower_bound(uk.begin(), uk.end(), keys[i]) - uk.begin());
  auto verts = [&](int e, double (*xv)[3]) {
    for (int v = 0; v <= D; v++)
      for (int c = 0; c < 3; c++) xv[v][c] = c < D ? m.xyz[(size_t)m.elv[e * (D + 1) + v] * D + c] : 0.0;
  };
  // step 1 and 2: contributions, averages in element order
  std::vector<double> gdef(uk.size() * 3, 0.0), cnt(uk.size(), 0.0);
  int nonconv = 0;
  if (deform)
    for (int e = 0; e < m.ne; e++) {
      double xv[4][3], contrib[6][3];
      verts(e, xv);
      bool band = false;
      if (!xg::iso::element_contrib<D>(&xg::g_tab, xv, &p2[(size_t)e * NN], threshold, contrib, &band, &nonconv))
        return NAN;
      if (!band) continue;
      for (int j = 0; j < NE; j++) {
        const int g = eid[(size_t)e * NE + j];
        for (int r = 0; r < D; r++) gdef[(size_t)g * 3 + r] += contrib[j][r];
        cnt[g] += 1.0;
      }
    }
  for (size_t g = 0; g < uk.size(); g++)
    if (cnt[g] > 0)
      for (int r = 0; r < 3; r++) gdef[g * 3 + r] /= cnt[g];
  // step 3
  double total = 0.0;
  for (int e = 0; e < m.ne; e++) {
    double xv[4][3], gl[6][3];
    verts(e, xv);
    for (int j = 0; j < NE; j++)
      for (int r = 0; r < 3; r++) gl[j][r] = gdef[(size_t)eid[(size_t)e * NE + j] * 3 + r];
    auto emit = [&](const double*, double w) { total += w; };
    if (xg::iso::element_rule<D>(&xg::g_tab, xv, &p2[(size_t)e * NN], gl, dt, order, emit)) return NAN;
  }
  return total;
}

template <int D>
static std::vector<double> p2_values(const Mesh& m, double (*f)(const double*)) {
  constexpr int NE = D == 2 ? 3 : 6;
  std::vector<double> out;
  for (int e = 0; e < m.ne; e++) {
    double xv[4][3] = {};
    for (int v = 0; v <= D; v++)
      for (int c = 0; c < D; c++) xv[v][c] = m.xyz[(size_t)m.elv[e * (D + 1) + v] * D + c];
    for (int v = 0; v <= D; v++) out.push_back(f(xv[v]));
    for (int j = 0; j < NE; j++) {
      int a, b;
      xg::iso::edge_ends<D>(j, a, b);
      double mid[3];
      for (int c = 0; c < 3; c++) mid[c] = 0.5 * (xv[a][c] + xv[b][c]);
      out.push_back(f(mid));
    }
  }
  return out;
}

static double circle(const double* x) { return std::sqrt(x[0] * x[0] + x[1] * x[1]) - 0.5; }
static double sphere(const double* x) {
  return std::sqrt((x[0] - .5) * (x[0] - .5) + (x[1] - .5) * (x[1] - .5) + (x[2] - .5) * (x[2] - .5)) - 0.3;
}

int main() {
  fill_table();
  int fails = 0, cases = 0;
  double worst = 0;
  for (int D = 2; D <= 3; D++) {
    const Mesh m = D == 2 ? structured(2, 12, -1.0, 1.0) : structured(3, 5, 0.0, 1.0);
    const std::vector<double> p2 = D == 2 ? p2_values<2>(m, circle) : p2_values<3>(m, sphere);
    for (int dt = 0; dt < 3; dt++)
      for (int order : {2, 4})
        for (double thr : {-1.0, 0.2})
          for (int deform : {0, 1}) {
            int nc = 0;
            const double ref =
                orc_iso_integrate_mesh(D, m.nv, m.xyz.data(), m.ne, m.elv.data(), p2.data(), dt, order, thr, deform, &nc);
            const double got = D == 2 ? run<2>(m, p2, dt, order, thr, deform) : run<3>(m, p2, dt, order, thr, deform);
            const double rel = std::fabs(got - ref) / std::max(1.0, std::fabs(ref));
            worst = std::max(worst, rel);
            cases++;
            if (!(rel <= 1e-12)) {
              fails++;
              std::printf("MISMATCH D=%d dt=%d order=%d thr=%g deform=%d: %.17g vs %.17g\n", D, dt, order, thr, deform,
                          got, ref);
            }
          }
  }
  std::printf("%d cases, worst relative difference %.3g, %d mismatches\n", cases, worst, fails);
  return fails ? 1 : 0;
}

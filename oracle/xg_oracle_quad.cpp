// Oracle: CPU restatement of ngsxfem's straight-cut rules on quadrilaterals
// and hexahedra.  TEST INFRASTRUCTURE ONLY (see xg_oracle.h): only tests/,
// the smoke check and the CPU legs of bench.py load it.  Built with
// -ffp-contract=off so that x86 and Arm hosts give identical bits.
//
// Restated from ngsxfem cutint/straightcutrule.cpp (object structure kept:
// a level-set wrapper, quadrilateral boxes, a recursive cut-quadrilateral):
//   :11-24    CheckIfStraightCut (with epsilon)
//   :41-64    SimpleX::CalcIFPolytopEUsingLset (general simplex points)
//   :66-77    SimpleX::GetVolume, Quadrilateral::GetVolume
//   :80-128   GetPlainIntegrationRule (simplex, quadrilateral)
//   :131-204  LevelsetCutSimplex::Decompose / GetIntegrationRule
//   :206-249  LevelsetCutQuadrilateral::HasTopologyChangeAlongXi / Decompose
//   :250-301  GetTensorProductAlongXiIntegrationRule (c = 0.999 bound)
//   :303-350  GetIntegrationRuleOn{XY,XZ,YZ}PermutatedQuad
//   :352-405  GetSufficientCritsQBound (3D), GetExactCritsQBound2D
//   :407-457  GetDimensionSwap
//   :459-501  GetIntegrationRuleAlongXi, GetFallbackIntegrationRule, GetIntegrationRule
//   :503-556  LevelsetWrapper (multilinear coefficients, value, gradient,
//             update_initial_coefs)
//   :558-578  TransformQuadUntrafoToIRInterface (bilinear / trilinear map)
//   :582-677  StraightCutIntegrationRule, quadrilateral branch
//   cutint/cutintegral.cpp:126-212  Integrate
// pow(x, 2) of the reference is written x * x.
// NGSolve pieces not in the reference tree are this project's definitions:
// the quadrilateral / hexahedron base rule is the tensor product of the
// segment rule (x outermost, z innermost); the element map is the bilinear
// (trilinear) interpolation of the vertices in the order
// (0,0),(1,0),(1,1),(0,1) [, the same at z = 1].
#include <algorithm>
#include <atomic>
#include <cmath>
#include <set>
#include <thread>
#include <vector>

#include "xg_oracle.h"

namespace {

enum { NEG = 0, POS = 1, IF = 2 };
enum { Q_FIRST_ALLOWED = 0, Q_FIND_OPTIMAL = 1, Q_ALWAYS_NONE = 2 };
enum { SW_ID, SW_X_Y, SW_X_Z, SW_Y_Z, SW_NONE };

// error codes thrown as exceptions by the reference
enum { E_PLAIN_CUT = 4, E_BAD_DECOMP = 5, E_NONFINITE = 7, E_IF_BOUND = 9 };
struct QErr {
  int code;
};

struct V3 {
  double x[3];
};
V3 v3(double a, double b, double c) { return V3{{a, b, c}}; }

struct Rule1 {
  std::vector<double> p, w;  // 3 coordinates per point
};
// base rules of the product's family (orc_base_rule): d = 0 point, 1 segment,
// 2 trig, 3 tet
Rule1 base(int d, int order) {
  Rule1 r;
  std::vector<double> p(3 * 512), w(512);
  const int n = orc_base_rule(d, order, p.data(), w.data(), 512);
  r.p.assign(p.begin(), p.begin() + 3 * n);
  r.w.assign(w.begin(), w.begin() + n);
  return r;
}

struct IR {
  std::vector<V3> p;
  std::vector<double> w;
  void add(const V3& a, double b) {
    p.push_back(a);
    w.push_back(b);
  }
};

int check_cut(const std::vector<double>& v, double eps = 0.0) {
  bool haspos = false, hasneg = false;
  for (double d : v) {
    if (!haspos && (d > eps)) haspos = true;
    if (!hasneg && (d < -eps)) hasneg = true;
    if (haspos && hasneg) break;
  }
  if ((hasneg && haspos) || (!hasneg && !haspos)) return IF;
  return hasneg ? NEG : POS;
}

// ---- LevelsetWrapper (straightcutrule.cpp:503-556) -------------------------------
struct Lset {
  double c[2][2][2];
  std::vector<double> initial_coefs;
  Lset(const std::vector<double>& vals, int et /* 1 segm, 4 quad, 8 hex */) {
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) c[i][j][k] = 0.;
    if (et == 1) {
      c[0][0][0] = vals[1];
      c[1][0][0] = vals[0] - vals[1];
    } else if (et == 4) {
      c[0][0][0] = vals[0];
      c[1][0][0] = vals[1] - c[0][0][0];
      c[0][1][0] = vals[3] - c[0][0][0];
      c[1][1][0] = vals[2] - c[1][0][0] - c[0][1][0] - c[0][0][0];
    } else {
      c[0][0][0] = vals[0];
      c[1][0][0] = vals[1] - vals[0];
      c[0][1][0] = vals[3] - vals[0];
      c[0][0][1] = vals[4] - vals[0];
      c[1][1][0] = vals[2] - c[1][0][0] - c[0][1][0] - c[0][0][0];
      c[1][0][1] = vals[5] - c[1][0][0] - c[0][0][1] - c[0][0][0];
      c[0][1][1] = vals[7] - c[0][1][0] - c[0][0][1] - c[0][0][0];
      c[1][1][1] = vals[6] - c[1][1][0] - c[1][0][1] - c[0][1][1] - c[1][0][0] - c[0][1][0] - c[0][0][1] -
                   c[0][0][0];
    }
    initial_coefs = vals;
  }
  double operator()(const V3& p) const {
    double v = 0;
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++)
          v += c[i][j][k] * std::pow(p.x[0], i) * std::pow(p.x[1], j) * std::pow(p.x[2], k);
    return v;
  }
  V3 grad(const V3& p) const {
    V3 g;
    g.x[0] = c[1][0][0] + c[1][1][0] * p.x[1] + c[1][0][1] * p.x[2] + c[1][1][1] * p.x[1] * p.x[2];
    g.x[1] = c[0][1][0] + c[1][1][0] * p.x[0] + c[0][1][1] * p.x[2] + c[1][1][1] * p.x[0] * p.x[2];
    g.x[2] = c[0][0][1] + c[0][1][1] * p.x[1] + c[1][0][1] * p.x[0] + c[1][1][1] * p.x[0] * p.x[1];
    return g;
  }
  void update_initial_coefs(const std::vector<V3>& pts) {
    initial_coefs.resize(pts.size());
    for (size_t i = 0; i < pts.size(); i++) {
      const double d = (*this)(pts[i]);
      initial_coefs[i] = std::fabs(d) > 1e-14 ? d : 1e-14;
    }
  }
};

double norm3(const V3& a) { return std::sqrt(a.x[0] * a.x[0] + a.x[1] * a.x[1] + a.x[2] * a.x[2]); }
V3 sub3(const V3& a, const V3& b) { return v3(a.x[0] - b.x[0], a.x[1] - b.x[1], a.x[2] - b.x[2]); }

// ---- simplices with general points (straightcutrule.cpp:41-204) ----------------------
// D = points - 1; volume as in SimpleX::GetVolume
double simplex_volume(const std::vector<V3>& p) {
  const int D = (int)p.size() - 1;
  if (D == 0) return 1;
  if (D == 1) return norm3(sub3(p[1], p[0]));
  if (D == 2) {
    const V3 a = sub3(p[2], p[0]), b = sub3(p[1], p[0]);
    return norm3(v3(a.x[1] * b.x[2] - a.x[2] * b.x[1], a.x[2] * b.x[0] - a.x[0] * b.x[2],
                    a.x[0] * b.x[1] - a.x[1] * b.x[0]));
  }
  const V3 a = sub3(p[3], p[0]), b = sub3(p[2], p[0]), c = sub3(p[1], p[0]);
  const double det = a.x[0] * (b.x[1] * c.x[2] - b.x[2] * c.x[1]) + a.x[1] * (b.x[2] * c.x[0] - b.x[0] * c.x[2]) +
                     a.x[2] * (b.x[0] * c.x[1] - b.x[1] * c.x[0]);
  return std::fabs(det);
}

void simplex_plain_rule(const std::vector<V3>& p, int order, IR& ir) {
  const double trafofac = simplex_volume(p);
  const Rule1 r = base((int)p.size() - 1, order);
  for (size_t q = 0; q < r.w.size(); q++) {
    const double* ip = &r.p[3 * q];
    double originweight = 1.0;
    for (size_t m = 0; m + 1 < p.size(); ++m) originweight -= ip[m];
    V3 pt;
    for (int k = 0; k < 3; k++) pt.x[k] = originweight * p[0].x[k];
    for (size_t m = 0; m + 1 < p.size(); ++m)
      for (int k = 0; k < 3; k++) pt.x[k] += ip[m] * p[m + 1].x[k];
    ir.add(pt, r.w[q] * trafofac);
  }
}

// CalcIFPolytopEUsingLset on a simplex with points p
std::vector<V3> calc_if_polytope(const std::vector<V3>& p, const std::vector<double>& l) {
  if (check_cut(l) != IF) throw QErr{E_PLAIN_CUT};
  std::vector<V3> out;
  if (p.size() == 2) {
    const double t = l[0] / (l[0] - l[1]);
    V3 r;
    for (int k = 0; k < 3; k++) r.x[k] = p[0].x[k] + t * (p[1].x[k] - p[0].x[k]);
    out.push_back(r);
    return out;
  }
  for (size_t i = 0; i < p.size(); i++)
    for (size_t j = i + 1; j < p.size(); j++)
      if ((l[i] >= 0) != (l[j] >= 0)) {
        const std::vector<V3> e = calc_if_polytope({p[i], p[j]}, {l[i], l[j]});
        out.push_back(e[0]);
      }
  return out;
}

// LevelsetCutSimplex::GetIntegrationRule: Decompose, then the plain rules
void cut_simplex_rule(const std::vector<V3>& s, const std::vector<double>& l, int dt, int order, IR& ir) {
  const int D = (int)s.size() - 1;
  const std::vector<V3> c = calc_if_polytope(s, l);
  std::vector<std::vector<V3>> dec;
  if (dt == IF) {
    if ((int)c.size() == D)
      dec.push_back(c);
    else if (c.size() == 4 && D == 3) {
      dec.push_back({c[0], c[1], c[3]});
      dec.push_back({c[0], c[2], c[3]});
    } else
      throw QErr{E_BAD_DECOMP};
  } else {
    std::vector<int> rel;
    for (int i = 0; i < D + 1; i++)
      if (((dt == POS) && (l[i] >= 0)) || ((dt == NEG) && (l[i] < 0))) rel.push_back(i);
    if (rel.size() == 1) {
      std::vector<V3> a(c);
      a.push_back(s[rel[0]]);
      dec.push_back(a);
    } else if (rel.size() == 2 && D == 2) {
      dec.push_back({s[rel[0]], s[rel[1]], c[1]});
      std::vector<V3> b(c);
      b.push_back(s[rel[0]]);
      dec.push_back(b);
    } else if (rel.size() == 2 && D == 3) {
      if (c.size() != 4) throw QErr{E_BAD_DECOMP};
      std::vector<V3> a(c);
      a[0] = s[rel[1]];
      dec.push_back(a);
      dec.push_back({s[rel[0]], s[rel[1]], c[1], c[2]});
      std::vector<V3> cc(c);
      cc[3] = s[rel[0]];
      dec.push_back(cc);
    } else if (rel.size() == 3 && D == 3) {
      if (c.size() != 3) throw QErr{E_BAD_DECOMP};
      std::vector<V3> a(c);
      a.push_back(s[rel[2]]);
      dec.push_back(a);
      dec.push_back({s[rel[0]], s[rel[1]], s[rel[2]], c[1]});
      std::vector<V3> cc(c);
      cc[2] = s[rel[0]];
      cc.push_back(s[rel[2]]);
      dec.push_back(cc);
    } else {
      throw QErr{E_BAD_DECOMP};
    }
  }
  for (auto& d : dec) {
    if ((int)d.size() != (dt == IF ? D : D + 1)) throw QErr{E_BAD_DECOMP};
    simplex_plain_rule(d, order, ir);
  }
}

// ---- Quadrilateral (straightcutrule.hpp:76-100, straightcutrule.cpp:73-128) -----------
struct Quad {
  int D;
  std::vector<V3> points;
  Quad(double x0, double x1, double y0, double y1) : D(2) {
    points = {v3(x0, y0, 0), v3(x1, y0, 0), v3(x1, y1, 0), v3(x0, y1, 0)};
  }
  Quad(double x0, double x1, double y0, double y1, double z0, double z1) : D(3) {
    points = {v3(x0, y0, z0), v3(x1, y0, z0), v3(x1, y1, z0), v3(x0, y1, z0),
              v3(x0, y0, z1), v3(x1, y0, z1), v3(x1, y1, z1), v3(x0, y1, z1)};
  }
  static Quad unit(int D) { return D == 2 ? Quad(0, 1, 0, 1) : Quad(0, 1, 0, 1, 0, 1); }
  std::vector<double> lset_vals(const Lset& l) const {
    std::vector<double> v;
    for (auto& p : points) v.push_back(l(p));
    return v;
  }
  double volume() const {
    if (D == 2) {
      const V3 a = sub3(points[3], points[0]), b = sub3(points[1], points[0]);
      return norm3(v3(a.x[1] * b.x[2] - a.x[2] * b.x[1], a.x[2] * b.x[0] - a.x[0] * b.x[2],
                      a.x[0] * b.x[1] - a.x[1] * b.x[0]));
    }
    const V3 a = sub3(points[4], points[0]), b = sub3(points[3], points[0]), c = sub3(points[1], points[0]);
    const double det = a.x[0] * (b.x[1] * c.x[2] - b.x[2] * c.x[1]) + a.x[1] * (b.x[2] * c.x[0] - b.x[0] * c.x[2]) +
                       a.x[2] * (b.x[0] * c.x[1] - b.x[1] * c.x[0]);
    return std::fabs(det);
  }
  // tensor-product base rule (x outermost) mapped by points[0] + A ip
  void plain_rule(int order, IR& ir) const {
    const double trafofac = volume();
    const Rule1 s = base(1, order);
    const int n = (int)s.w.size();
    double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    const int cols[3] = {1, 3, 4};
    for (int k = 0; k < D; k++)
      for (int r = 0; r < 3; r++) A[r][k] = points[cols[k]].x[r] - points[0].x[r];
    const int nz = D == 3 ? n : 1;
    for (int a = 0; a < n; a++)
      for (int b = 0; b < n; b++)
        for (int c = 0; c < nz; c++) {
          const double ip[3] = {s.p[3 * a], s.p[3 * b], D == 3 ? s.p[3 * c] : 0.0};
          const double w = D == 3 ? s.w[a] * s.w[b] * s.w[c] : s.w[a] * s.w[b];
          V3 pt;
          for (int r = 0; r < 3; r++) {
            double acc = A[r][0] * ip[0];
            acc += A[r][1] * ip[1];
            acc += A[r][2] * ip[2];
            pt.x[r] = points[0].x[r] + acc;
          }
          ir.add(pt, w * trafofac);
        }
  }
};

const double kC = 0.999;
const double kCBound = 1. / std::sqrt(1 - kC * kC);

// ---- LevelsetCutQuadrilateral (straightcutrule.cpp:206-501) ----------------------------
struct CutQuad {
  Lset lset;
  int dt;
  Quad q;
  int pol;
  bool consider_dim_swap;

  CutQuad(const Lset& l, int dt_, const Quad& q_, int pol_, bool swap = true)
      : lset(l), dt(dt_), q(q_), pol(pol_), consider_dim_swap(swap) {}

  std::vector<std::pair<int, int>> xi_edges() const {
    if (q.D == 2) return {{1, 2}, {0, 3}};
    return {{0, 4}, {1, 5}, {2, 6}, {3, 7}};
  }

  bool has_topology_change_along_xi() const {
    for (auto t : xi_edges()) {
      const std::vector<double> vals = {lset(q.points[t.second]), lset(q.points[t.first])};
      if (check_cut(vals) == IF) return true;
    }
    return false;
  }

  std::vector<CutQuad> decompose() const {
    std::set<double> xs{0, 1};
    for (auto t : xi_edges()) {
      const std::vector<double> vals = {lset(q.points[t.second]), lset(q.points[t.first])};
      if (check_cut(vals) == IF) {
        // the unit segment (1,0,0)-(0,0,0) of SimpleX(ET_SEGM)
        const std::vector<V3> p = calc_if_polytope({v3(1, 0, 0), v3(0, 0, 0)}, vals);
        if (!std::isnan(p[0].x[0])) xs.insert(p[0].x[0]);
      }
    }
    std::vector<double> v(xs.begin(), xs.end());
    std::vector<CutQuad> out;
    for (size_t i = 0; i + 1 < v.size(); i++) {
      const double xi0 = v[i], xi1 = v[i + 1];
      if (q.D == 2)
        out.emplace_back(lset, dt, Quad(q.points[0].x[0], q.points[2].x[0], xi0, xi1), pol);
      else
        out.emplace_back(lset, dt,
                         Quad(q.points[0].x[0], q.points[2].x[0], q.points[0].x[1], q.points[2].x[1], xi0, xi1),
                         pol);
    }
    return out;
  }

  void tensor_product_along_xi(IR& ir, int order) const {
    const int xi = q.D == 2 ? 1 : 2;
    const double xi0 = q.points[0].x[xi];
    const double xi1 = xi == 1 ? q.points[2].x[1] : q.points[4].x[2];
    const Rule1 r1 = base(1, order);
    for (size_t a = 0; a < r1.w.size(); a++) {
      const double xi_ast = xi0 + r1.p[3 * a] * (xi1 - xi0);
      IR sub;
      if (q.D == 2) {
        std::vector<double> lp(2);
        lp[1] = lset(v3(q.points[0].x[0], xi_ast, 0));
        lp[0] = lset(v3(q.points[2].x[0], xi_ast, 0));
        cut_simplex_rule({v3(1, 0, 0), v3(0, 0, 0)}, lp, dt, order, sub);
      } else {
        std::vector<double> lp(4);
        lp[0] = lset(v3(q.points[0].x[0], q.points[0].x[1], xi_ast));
        lp[1] = lset(v3(q.points[2].x[0], q.points[0].x[1], xi_ast));
        lp[2] = lset(v3(q.points[2].x[0], q.points[2].x[1], xi_ast));
        lp[3] = lset(v3(q.points[0].x[0], q.points[2].x[1], xi_ast));
        CutQuad child(Lset(lp, 4), dt, Quad::unit(2), pol);
        child.rule(sub, order);
      }
      for (size_t b = 0; b < sub.w.size(); b++) {
        V3 ip = v3(0, 0, 0);
        ip.x[xi] = xi_ast;
        ip.x[0] = q.points[0].x[0] + sub.p[b].x[0] * (q.points[2].x[0] - q.points[0].x[0]);
        if (q.D == 3) ip.x[1] = q.points[0].x[1] + sub.p[b].x[1] * (q.points[2].x[1] - q.points[0].x[1]);
        double fac = 1;
        if (dt == IF) {
          const V3 g = lset.grad(ip);
          if (q.D == 2)
            fac = norm3(g) / std::fabs(g.x[0]);
          else
            fac = norm3(g) / std::sqrt(g.x[0] * g.x[0] + g.x[1] * g.x[1]);
          if (std::isnan(fac) || fac > kCBound) throw QErr{E_IF_BOUND};
        }
        ir.add(ip, sub.w[b] * r1.w[a] * (xi1 - xi0) * fac);
      }
    }
  }

  // rule of the quadrilateral with coordinates permuted by perm (new
  // coordinate i = old coordinate perm[i]); the level set coefficients are
  // permuted alike and the points mapped back
  void permuted_rule(IR& ir, int order, const int* perm, bool along_xi) const {
    Lset lr = lset;
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) {
          int idx[3] = {i, j, k}, src[3];
          for (int m = 0; m < 3; m++) src[perm[m]] = idx[m];
          lr.c[i][j][k] = lset.c[src[0]][src[1]][src[2]];
        }
    // the permuted unit box is the unit box again (the reference swaps the
    // corner points back into the canonical order)
    CutQuad me(lr, dt, q, pol, false);
    IR rot;
    if (along_xi)
      me.rule_along_xi(rot, order);
    else
      me.rule(rot, order);
    for (size_t i = 0; i < rot.w.size(); i++) {
      V3 p;
      for (int m = 0; m < 3; m++) p.x[perm[m]] = rot.p[i].x[m];
      ir.add(p, rot.w[i]);
    }
  }

  std::vector<double> sufficient_crits_q_bound() const {
    double Vsq = 0;
    std::vector<V3> corners = {v3(0, 0, 0), v3(1, 0, 0), v3(0, 1, 0), v3(1, 1, 0),
                               v3(0, 0, 1), v3(1, 0, 1), v3(0, 1, 1), v3(1, 1, 1)};
    for (int d = 0; d < 3; d++) {
      double mx = 0;
      for (auto& p : corners) {
        const double gd = lset.grad(p).x[d];
        const double v = gd * gd;
        if (v > mx) mx = v;
      }
      Vsq += mx;
    }
    const double V = std::sqrt(Vsq);
    std::vector<double> qm{0, 0, 0};
    for (auto& p : corners)
      for (int d = 0; d < 3; d++) {
        const double gd = lset.grad(p).x[d];
        const double q_est = V * V / (V * V - gd * gd);
        if (q_est > qm[d]) qm[d] = q_est;
      }
    for (int d = 0; d < 3; d++) qm[d] = std::sqrt(1 - 1 / qm[d]);
    return qm;
  }

  std::vector<double> exact_crits_q_bound_2d() const {
    bool allow[2] = {true, true};
    double h_root = -lset.c[1][0][0] / lset.c[1][1][0];
    if ((h_root > 0) && (h_root < 1)) allow[1] = false;
    h_root = -lset.c[0][1][0] / lset.c[1][1][0];
    if ((h_root > 0) && (h_root < 1)) allow[0] = false;
    std::vector<double> qm{0, 0};
    for (const V3& p : {v3(0, 0, 0), v3(1, 0, 0), v3(1, 1, 0), v3(0, 1, 0)}) {
      const V3 g = lset.grad(p);
      const double q_y = std::fabs(g.x[1]) / norm3(g);
      const double q_x = std::fabs(g.x[0]) / norm3(g);
      if (q_y > qm[1]) qm[1] = q_y;
      if (q_x > qm[0]) qm[0] = q_x;
    }
    for (int i = 0; i < 2; i++)
      if (!allow[i]) qm[i] = 2;
    return qm;
  }

  int dimension_swap() const {
    if (pol == Q_ALWAYS_NONE) return SW_NONE;
    if (!consider_dim_swap) return SW_ID;
    if (q.D == 2) {
      const std::vector<double> e = exact_crits_q_bound_2d();
      if (pol == Q_FIRST_ALLOWED) {
        if (e[1] < kC) return SW_ID;
        if (e[0] < kC) return SW_X_Y;
        return SW_NONE;
      }
      if ((e[0] < kC) && (e[1] < kC)) return e[1] <= e[0] ? SW_ID : SW_X_Y;
      if (e[1] < kC) return SW_ID;
      if (e[0] < kC) return SW_X_Y;
      return SW_NONE;
    }
    const std::vector<double> s = sufficient_crits_q_bound();
    for (double d : s)
      if (std::isnan(d)) throw QErr{E_NONFINITE};
    if (pol == Q_FIRST_ALLOWED) {
      if (s[2] < kC) return SW_ID;
      if (s[1] < kC) return SW_Y_Z;
      if (s[0] < kC) return SW_X_Z;
      return SW_NONE;
    }
    // std::min_element with the comparison v1 <= v2: the last of equal minima
    int md = 0;
    for (int d = 1; d < 3; d++)
      if (s[d] <= s[md]) md = d;
    if (s[md] < kC) return md == 0 ? SW_X_Z : (md == 1 ? SW_Y_Z : SW_ID);
    return SW_NONE;
  }

  void rule_along_xi(IR& ir, int order) const {
    const int dt_quad = check_cut(q.lset_vals(lset));
    if (dt_quad == IF) {
      if (has_topology_change_along_xi()) {
        for (const CutQuad& s : decompose()) {
          const int d = check_cut(s.q.lset_vals(lset), 1e-15);
          if (d == IF)
            s.tensor_product_along_xi(ir, order);
          else if (d == dt)
            s.q.plain_rule(order, ir);
        }
      } else {
        tensor_product_along_xi(ir, order);
      }
    } else if (dt_quad == dt) {
      q.plain_rule(order, ir);
    }
  }

  void fallback_rule(IR& ir, int order) const {
    std::vector<std::vector<int>> subs;
    if (q.D == 2)
      subs = {{0, 1, 3}, {2, 1, 3}};
    else
      subs = {{3, 0, 1, 5}, {3, 1, 2, 5}, {3, 5, 2, 6}, {4, 5, 0, 3}, {4, 7, 5, 3}, {7, 6, 5, 3}};
    for (auto& idx : subs) {
      std::vector<V3> pl;
      for (int i : idx) pl.push_back(q.points[i]);
      Lset ls = lset;
      ls.update_initial_coefs(pl);
      const int d = check_cut(ls.initial_coefs);
      if ((d != IF) && (d == dt))
        simplex_plain_rule(pl, order, ir);
      else if (d == IF)
        cut_simplex_rule(pl, ls.initial_coefs, dt, order, ir);
    }
  }

  void rule(IR& ir, int order) const {
    const int sw = dimension_swap();
    static const int pxy[3] = {1, 0, 2}, pxz[3] = {2, 1, 0}, pyz[3] = {0, 2, 1};
    if (sw == SW_ID)
      rule_along_xi(ir, order);
    else if (sw == SW_X_Y)
      permuted_rule(ir, order, pxy, true);
    else if (sw == SW_Y_Z)
      permuted_rule(ir, order, pyz, false);
    else if (sw == SW_X_Z)
      permuted_rule(ir, order, pxz, false);
    else
      fallback_rule(ir, order);
  }
};

// StraightCutIntegrationRuleUntransformed (straightcutrule.cpp:814-879) for
// ET_QUAD / ET_HEX: -1 for "no rule", the point count, or -(error code) - 1
int quad_rule_untrafo(int D, const double* lv, int dt, int order, int pol, IR& ir) {
  const int nv = D == 2 ? 4 : 8;
  std::vector<double> vals(lv, lv + nv);
  const int dom = check_cut(vals);
  try {
    if (dom == IF) {
      Lset l(vals, nv);
      CutQuad cq(l, dt, Quad::unit(D), pol);
      cq.rule(ir, order);
      return (int)ir.w.size();
    }
  } catch (const QErr& e) {
    return -e.code - 1;
  }
  if (dom != dt) return -1;
  Quad::unit(D).plain_rule(order, ir);
  return (int)ir.w.size();
}

// bilinear / trilinear element map: x(xi) = sum_v N_v(xi) x_v, Jacobian J
void tp_map(int D, const double* xv /* [nv][3] */, const V3& xi, double* x, double J[3][3]) {
  const int nv = D == 2 ? 4 : 8;
  for (int i = 0; i < 3; i++) {
    x[i] = 0;
    for (int k = 0; k < 3; k++) J[i][k] = 0;
  }
  // vertex v sits at the corner (cx, cy, cz) of the unit box
  static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  for (int v = 0; v < nv; v++) {
    const double fx = cx[v] ? xi.x[0] : 1 - xi.x[0], gx = cx[v] ? 1.0 : -1.0;
    const double fy = cy[v] ? xi.x[1] : 1 - xi.x[1], gy = cy[v] ? 1.0 : -1.0;
    const double fz = D == 3 ? (cz[v] ? xi.x[2] : 1 - xi.x[2]) : 1.0, gz = cz[v] ? 1.0 : -1.0;
    const double N = fx * fy * fz;
    const double dN[3] = {gx * fy * fz, fx * gy * fz, fx * fy * gz};
    for (int i = 0; i < D; i++) {
      x[i] += N * xv[3 * v + i];
      for (int k = 0; k < D; k++) J[i][k] += xv[3 * v + i] * dN[k];
    }
  }
}

double det_inv(int D, double J[3][3], double Ji[3][3]) {
  if (D == 2) {
    const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double id = 1.0 / det;
    Ji[0][0] = J[1][1] * id;
    Ji[0][1] = -J[0][1] * id;
    Ji[1][0] = -J[1][0] * id;
    Ji[1][1] = J[0][0] * id;
    return det;
  }
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  const double id = 1.0 / det;
  Ji[0][0] = c00 * id;
  Ji[1][0] = c01 * id;
  Ji[2][0] = c02 * id;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  return det;
}

// |J^-T n_ref| with n_ref the normalised gradient of the multilinear level set at xi
// (TransformQuadUntrafoToIRInterface)
double if_weight_factor(int D, const Lset& l, const V3& xi, double Ji[3][3]) {
  const V3 g = l.grad(xi);
  const double nn = norm3(g);
  double n[3];
  for (int k = 0; k < 3; k++) n[k] = g.x[k] / nn;
  double np[3] = {0, 0, 0};
  for (int k = 0; k < D; k++) {
    double s = 0;
    for (int j = 0; j < D; j++) s += Ji[j][k] * n[j];
    np[k] = s;
  }
  return std::sqrt(np[0] * np[0] + np[1] * np[1] + np[2] * np[2]);
}

}  // namespace

extern "C" {

int orc_quad_cut_rule(int D, const double* lset_vals, int dt, int order, int policy, double* pts, double* wts,
                      int maxpts) {
  IR ir;
  const int n = quad_rule_untrafo(D, lset_vals, dt, order, policy, ir);
  if (n < 0) return n;
  if (n > maxpts) return -3 - 1;
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < 3; k++) pts[3 * i + k] = ir.p[i].x[k];
    wts[i] = ir.w[i];
  }
  return n;
}

// CutInformation::Update (xfem/cutinfo.cpp:61-132) on a quadrilateral /
// hexahedral mesh: per element the weights of the order-0 NEG and POS rules,
// ratio = NEG / (NEG + POS), domain IF / NEG / POS, bits[8][ceil(ne/64)] per
// combined domain type.  Returns 0 or the first error status.
int orc_quad_cutinfo(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* lset, int policy,
                     uint8_t* dom, double* ratio, uint64_t* bits) {
  (void)nv;
  (void)coords;
  const int nve = D == 2 ? 4 : 8;
  const int64_t nw = (ne + 63) / 64;
  for (int64_t i = 0; i < 8 * nw; i++) bits[i] = 0;
  int status = 0;
  for (int e = 0; e < ne; e++) {
    double lv[8];
    for (int v = 0; v < nve; v++) lv[v] = lset[elv[(size_t)e * nve + v]];
    double part[2] = {0.0, 0.0};  // [NEG, POS]
    for (int np : {POS, NEG}) {
      IR ir;
      const int n = quad_rule_untrafo(D, lv, np, 0, policy, ir);
      if (n < -1) {
        if (!status) status = -n - 1;
        continue;
      }
      for (double w : ir.w) part[np] += w;
    }
    ratio[e] = part[NEG] / (part[NEG] + part[POS]);
    const int d = part[NEG] > 0.0 ? (part[POS] > 0.0 ? IF : NEG) : POS;
    dom[e] = (uint8_t)d;
    const int rows[3][4] = {{1, 3, 5, 7}, {2, 3, 6, 7}, {4, 5, 6, 7}};  // NEG, POS, IF
    for (int r : rows[d]) bits[r * nw + (e >> 6)] |= 1ull << (e & 63);
  }
  return status;
}

int orc_quad_straight_cut_rule(int D, const double* xv, const double* lset_vals, int dt, int order, int policy,
                               double* pts, double* wts, int maxpts) {
  const int n = orc_quad_cut_rule(D, lset_vals, dt, order, policy, pts, wts, maxpts);
  if (n == 0) return -1;  // an empty cut rule is "no rule" (straightcutrule.cpp:627-628)
  if (n < 0 || dt != IF) return n;
  const int nv = D == 2 ? 4 : 8;
  Lset l(std::vector<double>(lset_vals, lset_vals + nv), nv);
  for (int i = 0; i < n; i++) {
    const V3 xi = v3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    double x[3], J[3][3], Ji[3][3];
    tp_map(D, xv, xi, x, J);
    det_inv(D, J, Ji);
    wts[i] = wts[i] * if_weight_factor(D, l, xi, Ji);
  }
  return n;
}

// Integrate(x^ex y^ey z^ez * dCut(lset, dt, order, quad_dir_policy)) over the
// elements [e0, e1) of a quadrilateral / hexahedral mesh: coords [nv][D],
// elements [ne][2^D], lset at the vertices.  *status = first error code.
static double quad_integrate_range(int D, const double* coords, const int32_t* elv, const double* lset, int dt,
                                   int order, int policy, int ex, int ey, int ez, int e0, int e1, int* status) {
  const int nve = D == 2 ? 4 : 8;
  double sum = 0;
  for (int e = e0; e < e1; e++) {
    double xv[8 * 3] = {0}, lv[8];
    for (int v = 0; v < nve; v++) {
      const int id = elv[(size_t)e * nve + v];
      lv[v] = lset[id];
      for (int i = 0; i < D; i++) xv[3 * v + i] = coords[(size_t)id * D + i];
    }
    IR ir;
    const int n = quad_rule_untrafo(D, lv, dt, order, policy, ir);
    if (n < -1) {
      if (*status == 0) *status = -n - 1;
      continue;
    }
    if (n <= 0) continue;
    Lset l(std::vector<double>(lv, lv + nve), nve);
    const bool cut = check_cut(std::vector<double>(lv, lv + nve)) == IF;
    for (int q = 0; q < n; q++) {
      double x[3], J[3][3], Ji[3][3];
      tp_map(D, xv, ir.p[q], x, J);
      const double det = det_inv(D, J, Ji);
      double w = ir.w[q];
      if (cut && dt == IF) w = w * if_weight_factor(D, l, ir.p[q], Ji);
      const double fv = std::pow(x[0], ex) * std::pow(x[1], ey) * (D == 3 ? std::pow(x[2], ez) : 1.0);
      sum += w * std::fabs(det) * fv;
    }
  }
  return sum;
}

orc_csr* orc_quad_assemble(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* lset,
                           const orc_term* terms, int nterms, int policy, int nthreads, int* status) {
  const int nve = D == 2 ? 4 : 8;
  static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  std::vector<int32_t> slot(ne, -1);
  std::vector<double> elm;
  int st = 0, nact = 0;
  for (int e = 0; e < ne; e++) {
    double xv[8 * 3] = {0}, lv[8];
    for (int v = 0; v < nve; v++) {
      const int id = elv[(size_t)e * nve + v];
      lv[v] = lset[id];
      for (int i = 0; i < D; i++) xv[3 * v + i] = coords[(size_t)id * D + i];
    }
    const std::vector<double> lvec(lv, lv + nve);
    const int dom = check_cut(lvec);
    auto on = [&](const orc_term& T) {
      if (T.defined_on && !((T.defined_on[e >> 6] >> (e & 63)) & 1u)) return false;
      return dom == IF || dom == T.domain;
    };
    bool any = false;
    for (int t = 0; t < nterms; t++) any |= on(terms[t]);
    if (!any) continue;
    slot[e] = nact++;
    elm.resize((size_t)nact * nve * nve, 0.0);
    double* A = &elm[(size_t)slot[e] * nve * nve];
    Lset l(lvec, nve);
    for (int t = 0; t < nterms; t++) {
      const orc_term& T = terms[t];
      if (!on(T)) continue;
      IR ir;
      const int n = quad_rule_untrafo(D, lv, T.domain, T.order >= 0 ? T.order : 2, policy, ir);
      if (n < -1) {
        if (!st) st = -n - 1;
        continue;
      }
      for (int q = 0; q < n; q++) {
        double x[3], J[3][3], Ji[3][3];
        tp_map(D, xv, ir.p[q], x, J);
        const double det = det_inv(D, J, Ji), adet = std::fabs(det);
        double w = ir.w[q] * adet;
        if (dom == IF && T.domain == IF) w *= if_weight_factor(D, l, ir.p[q], Ji);
        double c = T.coef;
        if (T.hpow != 0) c *= std::pow(std::pow(adet, 1.0 / D), (double)T.hpow);
        // Q1 shapes and physical gradients (grad_x = J^-T grad_xi)
        double N[8], G[8][3];
        const double* p = ir.p[q].x;
        for (int v = 0; v < nve; v++) {
          const double fx = cx[v] ? p[0] : 1 - p[0], gx = cx[v] ? 1.0 : -1.0;
          const double fy = cy[v] ? p[1] : 1 - p[1], gy = cy[v] ? 1.0 : -1.0;
          const double fz = D == 3 ? (cz[v] ? p[2] : 1 - p[2]) : 1.0, gz = cz[v] ? 1.0 : -1.0;
          N[v] = fx * fy * fz;
          const double dN[3] = {gx * fy * fz, fx * gy * fz, fx * fy * gz};
          for (int k = 0; k < 3; k++) {
            double acc = 0.0;
            if (k < D)
              for (int j = 0; j < D; j++) acc += Ji[j][k] * dN[j];
            G[v][k] = acc;
          }
        }
        double nrm[3] = {0, 0, 0};
        if (T.kind == ORC_TERM_NGRADU_V || T.kind == ORC_TERM_U_NGRADV) {
          const V3 g = l.grad(ir.p[q]);
          double nn = 0.0;
          for (int k = 0; k < D; k++) {
            double acc = 0.0;
            for (int j = 0; j < D; j++) acc += Ji[j][k] * g.x[j];
            nrm[k] = acc;
            nn += acc * acc;
          }
          nn = std::sqrt(nn);
          for (int k = 0; k < D; k++) nrm[k] /= nn;
        }
        const double* bb = T.kind == ORC_TERM_CONV ? T.b : nrm;
        for (int a = 0; a < nve; a++)      // test
          for (int b = 0; b < nve; b++) {  // trial
            double v;
            switch (T.kind) {
              case ORC_TERM_MASS: v = N[a] * N[b]; break;
              case ORC_TERM_LAPLACE: v = G[a][0] * G[b][0] + G[a][1] * G[b][1] + G[a][2] * G[b][2]; break;
              case ORC_TERM_U_NGRADV: v = N[b] * (bb[0] * G[a][0] + bb[1] * G[a][1] + bb[2] * G[a][2]); break;
              default: v = (bb[0] * G[b][0] + bb[1] * G[b][1] + bb[2] * G[b][2]) * N[a]; break;
            }
            A[a * nve + b] += w * c * v;
          }
      }
    }
  }
  if (status) *status = st;
  return orc_csr_from_elements(nv, nve, ne, elv, slot.data(), elm.data(), nact, nthreads);
}

double orc_quad_integrate(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* lset,
                          int dt, int order, int policy, int ex, int ey, int ez, int* status) {
  (void)nv;
  int st = 0;
  const double v = quad_integrate_range(D, coords, elv, lset, dt, order, policy, ex, ey, ez, 0, ne, &st);
  if (status) *status = st;
  return v;
}

// the same with nthreads host threads taking chunks of 256 elements; the
// chunk sums are added in chunk order (the result does not depend on the
// thread count)
double orc_quad_integrate_mt(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* lset,
                             int dt, int order, int policy, int ex, int ey, int ez, int nthreads, int* status) {
  (void)nv;
  if (nthreads < 1) nthreads = 1;
  const int chunk = 256, nch = (ne + chunk - 1) / chunk;
  std::vector<double> part(nch, 0.0);
  std::vector<int> st(nch, 0);
  std::atomic<int> next(0);
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; t++)
    th.emplace_back([&]() {
      for (int c = next.fetch_add(1); c < nch; c = next.fetch_add(1)) {
        const int e0 = c * chunk, e1 = e0 + chunk < ne ? e0 + chunk : ne;
        part[c] = quad_integrate_range(D, coords, elv, lset, dt, order, policy, ex, ey, ez, e0, e1, &st[c]);
      }
    });
  for (auto& t : th) t.join();
  double sum = 0;
  int first = 0;
  for (int c = 0; c < nch; c++) {
    sum += part[c];
    if (!first) first = st[c];
  }
  if (status) *status = first;
  return sum;
}

}  // extern "C"

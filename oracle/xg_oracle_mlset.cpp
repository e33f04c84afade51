// Oracle: CPU restatement of ngsxfem's multi-level-set straight-cut rules on
// simplices.  TEST INFRASTRUCTURE ONLY (see xg_oracle.h).  Built with
// -ffp-contract=off.
//
// Restated (object structure kept: a list of simplices refined level set by
// level set, breadth first):
//   cutint/straightcutrule.cpp:679-812   StraightCutsIntegrationRule
//   cutint/straightcutrule.cpp:41-64, 131-204  CalcIFPolytopEUsingLset,
//                                         LevelsetCutSimplex::Decompose on
//                                         simplices of any dimension and position
//   cutint/straightcutrule.cpp:503-556   LevelsetWrapper on ET_TRIG / ET_TET,
//                                         update_initial_coefs
//   cutint/straightcutrule.cpp:558-578   TransformQuadUntrafoToIRInterface
//   cutint/mlsetintegration.cpp:6-180    CreateMultiLevelsetCutIntegrationRule
//                                         (compatibility, condensing, parts)
//   cutint/cutintegral.cpp:126-212       Integrate
// The element geometry is affine: x = x_D + F xi with F(:,k) = x_k - x_D.
#include <algorithm>
#include <cmath>
#include <vector>

#include "xg_oracle.h"

namespace {

enum { NEG = 0, POS = 1, IF = 2 };
enum { E_CAPACITY = 3, E_PLAIN_CUT = 4, E_BAD_DECOMP = 5, E_UNSUPPORTED = 6 };
struct MErr {
  int code;
};

struct V3 {
  double x[3];
};
using Simplex = std::vector<V3>;

struct Rule1 {
  std::vector<double> p, w;
};
Rule1 base(int d, int order) {
  Rule1 r;
  std::vector<double> p(3 * 512), w(512);
  const int n = orc_base_rule(d, order, p.data(), w.data(), 512);
  r.p.assign(p.begin(), p.begin() + 3 * n);
  r.w.assign(w.begin(), w.begin() + n);
  return r;
}

int check_cut(const std::vector<double>& v) {
  bool haspos = false, hasneg = false;
  for (double d : v) {
    if (!haspos && d > 0) haspos = true;
    if (!hasneg && d < 0) hasneg = true;
    if (haspos && hasneg) break;
  }
  if ((hasneg && haspos) || (!hasneg && !haspos)) return IF;
  return hasneg ? NEG : POS;
}

// LevelsetWrapper of the element's linear level set (ET_TRIG / ET_TET vertex
// values; c000 = v_D, c100 = v_0 - v_D, c010 = v_1 - v_D, c001 = v_2 - v_D)
struct Lset {
  double c[2][2][2];
  std::vector<double> initial_coefs;
  Lset(int D, const double* v) {
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) c[i][j][k] = 0.;
    if (D == 2) {
      c[0][0][0] = v[2];
      c[1][0][0] = v[0] - v[2];
      c[0][1][0] = v[1] - v[2];
    } else {
      c[0][0][0] = v[3];
      c[1][0][0] = v[0] - v[3];
      c[0][1][0] = v[1] - v[3];
      c[0][0][1] = v[2] - v[3];
    }
    initial_coefs.assign(v, v + D + 1);
  }
  double operator()(const V3& p) const {
    double s = 0;
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++)
        for (int k = 0; k < 2; k++) {
          double t = c[i][j][k];
          if (i) t = t * p.x[0];
          if (j) t = t * p.x[1];
          if (k) t = t * p.x[2];
          s += t;
        }
    return s;
  }
  void update_initial_coefs(const Simplex& pts) {
    initial_coefs.resize(pts.size());
    for (size_t i = 0; i < pts.size(); i++) {
      const double d = (*this)(pts[i]);
      initial_coefs[i] = std::fabs(d) > 1e-14 ? d : 1e-14;
    }
  }
  // constant reference gradient and its unit normal
  void normal(double* n) const {
    const double g[3] = {c[1][0][0], c[0][1][0], c[0][0][1]};
    const double nn = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    for (int k = 0; k < 3; k++) n[k] = g[k] / nn;
  }
};

double norm3(const double* a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

double simplex_volume(const Simplex& p) {
  const int D = (int)p.size() - 1;
  if (D == 0) return 1;
  double a[3], b[3], c[3];
  if (D == 1) {
    for (int k = 0; k < 3; k++) a[k] = p[1].x[k] - p[0].x[k];
    return norm3(a);
  }
  if (D == 2) {
    for (int k = 0; k < 3; k++) {
      a[k] = p[2].x[k] - p[0].x[k];
      b[k] = p[1].x[k] - p[0].x[k];
    }
    const double cr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    return norm3(cr);
  }
  for (int k = 0; k < 3; k++) {
    a[k] = p[3].x[k] - p[0].x[k];
    b[k] = p[2].x[k] - p[0].x[k];
    c[k] = p[1].x[k] - p[0].x[k];
  }
  return std::fabs(a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) +
                   a[2] * (b[0] * c[1] - b[1] * c[0]));
}

// CalcIFPolytopEUsingLset on a simplex of any dimension (points p, values l)
std::vector<V3> cut_points(const Simplex& p, const std::vector<double>& l) {
  if (check_cut(l) != IF) throw MErr{E_PLAIN_CUT};
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
      if ((l[i] >= 0) != (l[j] >= 0)) out.push_back(cut_points({p[i], p[j]}, {l[i], l[j]})[0]);
  return out;
}

// LevelsetCutSimplex::Decompose of simplex s (dimension s.size()-1) by the
// values l (the level set's initial_coefs on s)
std::vector<Simplex> decompose(const Simplex& s, const std::vector<double>& l, int dt) {
  const int D = (int)s.size() - 1;
  const std::vector<V3> c = cut_points(s, l);
  std::vector<Simplex> out;
  if (dt == IF) {
    if ((int)c.size() == D)
      out.push_back(c);
    else if (c.size() == 4 && D == 3) {
      out.push_back({c[0], c[1], c[3]});
      out.push_back({c[0], c[2], c[3]});
    } else
      throw MErr{E_BAD_DECOMP};
    return out;
  }
  std::vector<int> rel;
  for (int i = 0; i < D + 1; i++)
    if (((dt == POS) && (l[i] >= 0)) || ((dt == NEG) && (l[i] < 0))) rel.push_back(i);
  if (rel.size() == 1) {
    Simplex a(c);
    a.push_back(s[rel[0]]);
    out.push_back(a);
  } else if (rel.size() == 2 && D == 2) {
    out.push_back({s[rel[0]], s[rel[1]], c[1]});
    Simplex b(c);
    b.push_back(s[rel[0]]);
    out.push_back(b);
  } else if (rel.size() == 2 && D == 3) {
    if (c.size() != 4) throw MErr{E_BAD_DECOMP};
    Simplex a(c);
    a[0] = s[rel[1]];
    out.push_back(a);
    out.push_back({s[rel[0]], s[rel[1]], c[1], c[2]});
    Simplex cc(c);
    cc[3] = s[rel[0]];
    out.push_back(cc);
  } else if (rel.size() == 3 && D == 3) {
    if (c.size() != 3) throw MErr{E_BAD_DECOMP};
    Simplex a(c);
    a.push_back(s[rel[2]]);
    out.push_back(a);
    out.push_back({s[rel[0]], s[rel[1]], s[rel[2]], c[1]});
    Simplex cc(c);
    cc[2] = s[rel[0]];
    cc.push_back(s[rel[2]]);
    out.push_back(cc);
  } else {
    throw MErr{E_BAD_DECOMP};
  }
  return out;
}

void plain_rule(const Simplex& p, int order, std::vector<V3>& pts, std::vector<double>& wts) {
  const double trafofac = simplex_volume(p);
  const Rule1 r = base((int)p.size() - 1, order);
  for (size_t q = 0; q < r.w.size(); q++) {
    const double* ip = &r.p[3 * q];
    double ow = 1.0;
    for (size_t m = 0; m + 1 < p.size(); ++m) ow -= ip[m];
    V3 pt;
    for (int k = 0; k < 3; k++) pt.x[k] = ow * p[0].x[k];
    for (size_t m = 0; m + 1 < p.size(); ++m)
      for (int k = 0; k < 3; k++) pt.x[k] += ip[m] * p[m + 1].x[k];
    pts.push_back(pt);
    wts.push_back(r.w[q] * trafofac);
  }
}

struct Geo {
  int D;
  double F[3][3], Finv[3][3], det;
};

Geo make_geo(int D, const double* elc /* (D+1) x D */) {
  Geo g;
  g.D = D;
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) g.F[i][k] = g.Finv[i][k] = 0;
  for (int k = 0; k < D; k++)
    for (int i = 0; i < D; i++) g.F[i][k] = elc[k * D + i] - elc[D * D + i];
  if (D == 2) {
    const double a = g.F[0][0], b = g.F[0][1], c = g.F[1][0], d = g.F[1][1];
    g.det = a * d - b * c;
    const double id = 1.0 / g.det;
    g.Finv[0][0] = d * id;
    g.Finv[0][1] = -b * id;
    g.Finv[1][0] = -c * id;
    g.Finv[1][1] = a * id;
  } else {
    const double(*F)[3] = g.F;
    const double c00 = F[1][1] * F[2][2] - F[1][2] * F[2][1];
    const double c01 = F[1][2] * F[2][0] - F[1][0] * F[2][2];
    const double c02 = F[1][0] * F[2][1] - F[1][1] * F[2][0];
    g.det = F[0][0] * c00 + F[0][1] * c01 + F[0][2] * c02;
    const double id = 1.0 / g.det;
    g.Finv[0][0] = c00 * id;
    g.Finv[1][0] = c01 * id;
    g.Finv[2][0] = c02 * id;
    g.Finv[0][1] = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) * id;
    g.Finv[1][1] = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) * id;
    g.Finv[2][1] = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) * id;
    g.Finv[0][2] = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) * id;
    g.Finv[1][2] = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) * id;
    g.Finv[2][2] = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) * id;
  }
  return g;
}

// StraightCutsIntegrationRule: the element is cut by every level set given
// (values lv[i][0..D]); returns false for "no rule" (an empty rule)
bool straight_cuts_rule(const Geo& g, const std::vector<const double*>& lv, const std::vector<int>& dts, int order,
                        std::vector<V3>& pts, std::vector<double>& wts) {
  const int D = g.D, M = (int)lv.size();
  Simplex ref;
  for (int i = 0; i <= D; i++) {
    V3 v = {{0, 0, 0}};
    if (i < D) v.x[i] = 1.0;
    ref.push_back(v);
  }
  std::vector<Simplex> last = decompose(ref, std::vector<double>(lv[0], lv[0] + D + 1), dts[0]);
  for (int i = 1; i < M; i++) {
    Lset l(D, lv[i]);
    std::vector<Simplex> cur;
    for (const Simplex& s : last) {
      Lset ls = l;
      ls.update_initial_coefs(s);
      const int d = check_cut(ls.initial_coefs);
      if (d == IF) {
        for (const Simplex& t : decompose(s, ls.initial_coefs, dts[i])) cur.push_back(t);
      } else if (d == dts[i]) {
        cur.push_back(s);
      }
    }
    last = cur;
  }
  const size_t first = wts.size();
  for (const Simplex& s : last) plain_rule(s, order, pts, wts);
  if (wts.size() == first) return false;
  std::vector<int> ifs;
  for (int i = 0; i < M; i++)
    if (dts[i] == IF) ifs.push_back(i);
  if (ifs.size() == 1) {
    double n[3];
    Lset(D, lv[ifs[0]]).normal(n);
    double np[3] = {0, 0, 0};
    for (int k = 0; k < D; k++) {
      double s = 0;
      for (int j = 0; j < D; j++) s += g.Finv[j][k] * n[j];
      np[k] = s;
    }
    const double fac = norm3(np);
    for (size_t q = first; q < wts.size(); q++) wts[q] = wts[q] * fac;
  } else if (ifs.size() == 2) {
    if (D == 2) {
      for (size_t q = first; q < wts.size(); q++) wts[q] = wts[q] / std::fabs(g.det);
    } else {
      double n0[3], n1[3];
      Lset(D, lv[ifs[0]]).normal(n0);
      Lset(D, lv[ifs[1]]).normal(n1);
      const double cr[3] = {n0[1] * n1[2] - n0[2] * n1[1], n0[2] * n1[0] - n0[0] * n1[2],
                            n0[0] * n1[1] - n0[1] * n1[0]};
      const double cp_fac = 1. / norm3(cr);
      double nv[3];
      for (int i = 0; i < 3; i++) nv[i] = cp_fac * (g.F[i][0] * cr[0] + g.F[i][1] * cr[1] + g.F[i][2] * cr[2]);
      const double fac = norm3(nv);
      for (size_t q = first; q < wts.size(); q++) wts[q] = wts[q] * fac / std::fabs(g.det);
    }
  } else if (ifs.size() == 3) {
    if (D != 3) throw MErr{E_UNSUPPORTED};
    for (size_t q = first; q < wts.size(); q++) wts[q] = wts[q] / std::fabs(g.det);
  } else if (ifs.size() > 3) {
    throw MErr{E_UNSUPPORTED};
  }
  return true;
}

// CreateMultiLevelsetCutIntegrationRule for one element: the parts of every
// domain tuple (dts[t * M + i]) concatenated; lv[i] = values of level set i
// at the element's vertices.  Returns false if no part has points.
bool mlset_element_rule(const Geo& g, int M, const std::vector<const double*>& lv, int ntup, const int* dts,
                        int order, std::vector<V3>& pts, std::vector<double>& wts) {
  const int D = g.D;
  std::vector<int> ldt(M);
  for (int i = 0; i < M; i++) ldt[i] = check_cut(std::vector<double>(lv[i], lv[i] + D + 1));
  bool any = false;
  for (int t = 0; t < ntup; t++) {
    const int* dt = dts + (size_t)t * M;
    bool compatible = true, cut = false;
    for (int i = 0; i < M; i++) {
      if (ldt[i] != IF && ldt[i] != dt[i])
        compatible = false;
      else if (ldt[i] == IF)
        cut = true;
    }
    if (!compatible) continue;
    if (!cut) {
      const Rule1 r = base(D, order);
      for (size_t q = 0; q < r.w.size(); q++) {
        pts.push_back(V3{{r.p[3 * q], r.p[3 * q + 1], r.p[3 * q + 2]}});
        wts.push_back(r.w[q]);
      }
      any = true;
      continue;
    }
    std::vector<const double*> cl;
    std::vector<int> cdt;
    for (int i = 0; i < M; i++)
      if (ldt[i] == IF || ldt[i] != dt[i]) {
        cl.push_back(lv[i]);
        cdt.push_back(dt[i]);
      }
    any |= straight_cuts_rule(g, cl, cdt, order, pts, wts);
  }
  return any;
}

}  // namespace

extern "C" {

int orc_mlset_cut_rule(int D, const double* elc, int M, const double* lsets, int ntup, const int* dts, int order,
                       double* pts, double* wts, int maxpts) {
  const Geo g = make_geo(D, elc);
  std::vector<const double*> lv;
  for (int i = 0; i < M; i++) lv.push_back(lsets + (size_t)i * (D + 1));
  std::vector<V3> p;
  std::vector<double> w;
  try {
    if (!mlset_element_rule(g, M, lv, ntup, dts, order, p, w)) return -1;
  } catch (const MErr& e) {
    return -e.code - 1;
  }
  if ((int)w.size() > maxpts) return -E_CAPACITY - 1;
  for (size_t i = 0; i < w.size(); i++) {
    for (int k = 0; k < 3; k++) pts[3 * i + k] = p[i].x[k];
    wts[i] = w[i];
  }
  return (int)w.size();
}

// MultiLevelsetCutInformation (xfem/cutinfo.cpp:306-419): mode 0
// (GetElementsOfDomainType) marks the elements whose level-set domain types
// equal one of the tuples; mode 1 (GetElementsWithContribution) those whose
// rule of the region (order 0) has a positive weight sum.  bits: ceil(ne/64)
// words.  Returns 0 or the first error status.
int orc_mlset_mark(int D, int nv, const double* coords, int ne, const int32_t* elv, int M, const double* lsets,
                   int ntup, const int* dts, int mode, uint64_t* bits) {
  if (M < 1 || M > 8) return E_UNSUPPORTED;
  int status = 0;
  for (int w = 0; w < (ne + 63) / 64; w++) bits[w] = 0;
  for (int e = 0; e < ne; e++) {
    double elc[12], lvals[8 * 4];
    for (int v = 0; v <= D; v++) {
      const int id = elv[(size_t)e * (D + 1) + v];
      for (int i = 0; i < D; i++) elc[v * D + i] = coords[(size_t)id * D + i];
      for (int m = 0; m < M; m++) lvals[m * (D + 1) + v] = lsets[(size_t)m * nv + id];
    }
    bool mark = false;
    if (mode == 0) {
      int ldt[8];
      for (int m = 0; m < M; m++) ldt[m] = check_cut(std::vector<double>(lvals + m * (D + 1), lvals + (m + 1) * (D + 1)));
      for (int t = 0; t < ntup && !mark; t++) {
        bool match = true;
        for (int m = 0; m < M; m++) match &= dts[t * M + m] == ldt[m];
        mark = match;
      }
    } else {
      const Geo g = make_geo(D, elc);
      std::vector<const double*> lv;
      for (int m = 0; m < M; m++) lv.push_back(lvals + m * (D + 1));
      std::vector<V3> p;
      std::vector<double> w;
      try {
        if (mlset_element_rule(g, M, lv, ntup, dts, 0, p, w)) {
          double part = 0;
          for (double x : w) part += x;
          mark = part > 0;
        }
      } catch (const MErr& err) {
        if (!status) status = err.code;
      }
    }
    if (mark) bits[e >> 6] |= 1ull << (e & 63);
  }
  return status;
}

double orc_mlset_integrate(int D, int nv, const double* coords, int ne, const int32_t* elv, int M,
                           const double* lsets, int ntup, const int* dts, int order, int ex, int ey, int ez,
                           int* status) {
  double sum = 0;
  if (status) *status = 0;
  if (M < 1 || M > 8) {
    if (status) *status = E_UNSUPPORTED;
    return 0.0;
  }
  for (int e = 0; e < ne; e++) {
    double elc[12], lvals[8 * 4];
    for (int v = 0; v <= D; v++) {
      const int id = elv[(size_t)e * (D + 1) + v];
      for (int i = 0; i < D; i++) elc[v * D + i] = coords[(size_t)id * D + i];
      for (int m = 0; m < M; m++) lvals[m * (D + 1) + v] = lsets[(size_t)m * nv + id];
    }
    const Geo g = make_geo(D, elc);
    std::vector<const double*> lv;
    for (int m = 0; m < M; m++) lv.push_back(lvals + m * (D + 1));
    std::vector<V3> p;
    std::vector<double> w;
    try {
      if (!mlset_element_rule(g, M, lv, ntup, dts, order, p, w)) continue;
    } catch (const MErr& err) {
      if (status && *status == 0) *status = err.code;
      continue;
    }
    const double meas = std::fabs(g.det);
    for (size_t q = 0; q < w.size(); q++) {
      double x[3] = {0, 0, 0};
      for (int i = 0; i < D; i++) {
        double s = elc[D * D + i];
        for (int k = 0; k < D; k++) s += g.F[i][k] * p[q].x[k];
        x[i] = s;
      }
      const double fv = std::pow(x[0], ex) * std::pow(x[1], ey) * (D == 3 ? std::pow(x[2], ez) : 1.0);
      sum += w[q] * meas * fv;
    }
  }
  return sum;
}

}  // extern "C"

// ---- boundary cut integration (dCut(lset, dt, vb=BND)) -------------------------------
// StraightCutIntegrationRule on a boundary element (cutint/straightcutrule.cpp:
// 582-677 with the ET_SEGM-in-2D point measure of :641-651) and Integrate over
// the boundary elements (cutint/cutintegral.cpp:126-212).  Boundary elements:
// the element facets that belong to one element, vertices ascending; the
// reference simplex of dimension D-1 maps by x = x_last + F xi.
namespace {

// the rule of one boundary element in physical points xs (3 per point) and
// weights ws = w * measure
void bnd_element_rule(int D, const double (*xv)[3], const double* l, int dt, int order, std::vector<double>& xs,
                      std::vector<double>& ws) {
  xs.clear();
  ws.clear();
  const int d = D - 1;  // dimension of the boundary element
  // F (3 x d): columns x_k - x_d; measure: length (d = 1) or |F1 x F2| (d = 2)
  double F[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  for (int k = 0; k < d; k++)
    for (int r = 0; r < 3; r++) F[r][k] = xv[k][r] - xv[d][r];
  double meas;
  if (d == 1) {
    const double a[3] = {F[0][0], F[1][0], F[2][0]};
    meas = norm3(a);
  } else {
    const double cr[3] = {F[1][0] * F[2][1] - F[2][0] * F[1][1], F[2][0] * F[0][1] - F[0][0] * F[2][1],
                          F[0][0] * F[1][1] - F[1][0] * F[0][1]};
    meas = norm3(cr);
  }
  std::vector<double> lv(l, l + d + 1);
  const int dom = check_cut(lv);
  std::vector<V3> pts;
  std::vector<double> wts;
  if (dom != IF) {
    if (dom != dt) return;
    const Rule1 r = base(d, order);
    for (size_t q = 0; q < r.w.size(); q++) {
      pts.push_back(V3{{r.p[3 * q], r.p[3 * q + 1], r.p[3 * q + 2]}});
      wts.push_back(r.w[q]);
    }
  } else {
    if (dt == IF && d != 1) throw MErr{E_UNSUPPORTED};
    Simplex ref;
    for (int i = 0; i <= d; i++) {
      V3 v = {{0, 0, 0}};
      if (i < d) v.x[i] = 1.0;
      ref.push_back(v);
    }
    for (const Simplex& s : decompose(ref, lv, dt)) plain_rule(s, order, pts, wts);
    if (dt == IF)  // point measure: weight / measure, so that weight * measure = 1
      for (double& w : wts) w = w / meas;
  }
  for (size_t q = 0; q < wts.size(); q++) {
    for (int r = 0; r < 3; r++) {
      double s = xv[d][r];
      for (int k = 0; k < d; k++) s += F[r][k] * pts[q].x[k];
      xs.push_back(s);
    }
    ws.push_back(wts[q] * meas);
  }
}

double bnd_element_integral(int D, const double (*xv)[3], const double* l, int dt, int order, int ex, int ey, int ez) {
  std::vector<double> xs, ws;
  bnd_element_rule(D, xv, l, dt, order, xs, ws);
  double sum = 0;
  for (size_t q = 0; q < ws.size(); q++) {
    const double* x = &xs[3 * q];
    const double fv = std::pow(x[0], ex) * std::pow(x[1], ey) * (D == 3 ? std::pow(x[2], ez) : 1.0);
    sum += ws[q] * fv;
  }
  return sum;
}

}  // namespace

// the rule of one boundary element: physical points (3 per point) and weights
// w * measure; returns the number of points, -1 when more than cap, or
// -(error code)
extern "C" int orc_bnd_element_rule(int D, const double* xv, const double* l, int dt, int order, double* xs, double* ws,
                                    int cap) {
  double v[3][3];
  for (int i = 0; i < D; i++)
    for (int r = 0; r < 3; r++) v[i][r] = xv[3 * i + r];
  std::vector<double> px, pw;
  try {
    bnd_element_rule(D, v, l, dt, order, px, pw);
  } catch (const MErr& err) {
    return -err.code;
  }
  if ((int)pw.size() > cap) return -1;
  std::copy(px.begin(), px.end(), xs);
  std::copy(pw.begin(), pw.end(), ws);
  return (int)pw.size();
}

// one boundary element (vertices xv[D][3], values l[D]); *status on an error
extern "C" double orc_bnd_element_integral(int D, const double* xv, const double* l, int dt, int order, int ex, int ey,
                                           int ez, int* status) {
  double v[3][3];
  for (int i = 0; i < D; i++)
    for (int r = 0; r < 3; r++) v[i][r] = xv[3 * i + r];
  *status = 0;
  try {
    return bnd_element_integral(D, v, l, dt, order, ex, ey, ez);
  } catch (const MErr& err) {
    *status = err.code;
  }
  return 0.0;
}

extern "C" double orc_integrate_bnd(int D, int nv, const double* coords, int ne, const int32_t* elv,
                                    const double* lset, int dt, int order, int ex, int ey, int ez,
                                    const uint8_t* defined_on, int* status) {
  (void)nv;
  if (status) *status = 0;
  // facets (sorted vertex triples / pairs) and their element counts
  std::vector<std::vector<int>> facets;
  for (int e = 0; e < ne; e++)
    for (int skip = 0; skip <= D; skip++) {
      std::vector<int> f;
      for (int v = 0; v <= D; v++)
        if (v != skip) f.push_back(elv[(size_t)e * (D + 1) + v]);
      std::sort(f.begin(), f.end());
      facets.push_back(f);
    }
  std::sort(facets.begin(), facets.end());
  double sum = 0;
  int64_t b = 0;  // BND element number: boundary facets in lexicographic order
  for (size_t i = 0; i < facets.size();) {
    size_t j = i;
    while (j < facets.size() && facets[j] == facets[i]) j++;
    if (j - i == 1 && (!defined_on || defined_on[b])) {
      double xv[3][3] = {}, l[3];
      for (int v = 0; v < D; v++) {
        const int id = facets[i][v];
        l[v] = lset[id];
        for (int r = 0; r < D; r++) xv[v][r] = coords[(size_t)id * D + r];
      }
      try {
        sum += bnd_element_integral(D, xv, l, dt, order, ex, ey, ez);
      } catch (const MErr& err) {
        if (status && *status == 0) *status = err.code;
      }
    }
    if (j - i == 1) b++;
    i = j;
  }
  return sum;
}

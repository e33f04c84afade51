// Host side of libxg: status reporting, the quadrature rule family, mesh
// topology (the ngcomp::MeshAccess tables the reference reads) and H1 dof
// tables.  None of this runs per assembly step.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "xg_internal.h"
#include "xg_topology.h"

namespace xg {

static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }
int cuda_fail(cudaError_t e, const char* what) {
  set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  return XG_ERR_CUDA;
}

// ---- Gauss-Jacobi nodes by Newton's method with deflation ------------------------
// P_n^{(a,0)} by the three-term recurrence; weights 2^{a+1} / ((1-x^2) P_n'(x)^2).
static void jacobi_eval(int n, double a, double x, double* p, double* dp) {
  const double b = 0.0;
  // P_1 = ((a - b) + (a + b + 2) x) / 2, written so that x = 0 stays exact
  double p0 = 1.0, p1 = 0.5 * (a - b) + 0.5 * (a + b + 2.0) * x;
  if (n == 0) { *p = 1.0; *dp = 0.0; return; }
  // derivative: d/dx P_n^{(a,b)} = (n+a+b+1)/2 * P_{n-1}^{(a+1,b+1)}
  auto pval = [](int m, double aa, double bb, double xx) {
    double q0 = 1.0, q1 = 0.5 * (aa - bb) + 0.5 * (aa + bb + 2.0) * xx;
    if (m == 0) return q0;
    for (int k = 2; k <= m; k++) {
      double c = 2.0 * k + aa + bb;
      double a1 = 2.0 * k * (k + aa + bb) * (c - 2.0);
      double a2 = (c - 1.0) * (aa * aa - bb * bb);
      double a3 = (c - 2.0) * (c - 1.0) * c;
      double a4 = 2.0 * (k + aa - 1.0) * (k + bb - 1.0) * c;
      double q2 = ((a2 + a3 * xx) * q1 - a4 * q0) / a1;
      q0 = q1;
      q1 = q2;
    }
    return q1;
  };
  for (int k = 2; k <= n; k++) {
    double c = 2.0 * k + a + b;
    double a1 = 2.0 * k * (k + a + b) * (c - 2.0);
    double a2 = (c - 1.0) * (a * a - b * b);
    double a3 = (c - 2.0) * (c - 1.0) * c;
    double a4 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * c;
    double p2 = ((a2 + a3 * x) * p1 - a4 * p0) / a1;
    p0 = p1;
    p1 = p2;
  }
  *p = p1;
  *dp = 0.5 * (n + a + b + 1.0) * pval(n - 1, a + 1.0, b + 1.0, x);
}

static void gauss_jacobi01(int n, int alpha, std::vector<double>& x01, std::vector<double>& w01) {
  std::vector<double> x(n);
  const double a = alpha;
  for (int k = 0; k < n; k++) {
    double z = -std::cos(M_PI * (k + 0.75) / (n + 0.5));  // ascending initial guesses
    if (alpha == 0 && n % 2 == 1 && k == n / 2) z = 0.0;   // middle Gauss-Legendre node
    for (int it = 0; it < 100; it++) {
      double p, dp;
      jacobi_eval(n, a, z, &p, &dp);
      double defl = 0.0;
      for (int j = 0; j < k; j++) defl += 1.0 / (z - x[j]);
      double dz = p / (dp - p * defl);
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    x[k] = z;
  }
  std::sort(x.begin(), x.end());
  x01.resize(n);
  w01.resize(n);
  for (int k = 0; k < n; k++) {
    double p, dp;
    jacobi_eval(n, a, x[k], &p, &dp);
    double w = std::ldexp(1.0, alpha + 1) / ((1.0 - x[k] * x[k]) * dp * dp);
    x01[k] = 0.5 * (1.0 + x[k]);
    w01[k] = w * std::ldexp(1.0, -alpha - 1);
  }
}

static RuleTable build_rules() {
  RuleTable t;
  std::memset(&t, 0, sizeof(t));
  int n = 0;
  auto add = [&](double a, double b, double c, double w) {
    t.x[n][0] = a; t.x[n][1] = b; t.x[n][2] = c; t.w[n] = w; n++;
  };
  // fully symmetric orbits; parameters solved from the moment equations
  // (oracle/derive_symmetric_rules.py)
  auto sym21 = [&](double a, double w) {
    const double b = 1.0 - 2.0 * a;
    add(a, a, 0, w); add(a, b, 0, w); add(b, a, 0, w);
  };
  auto sym31 = [&](double a, double w) {
    const double b = 1.0 - 3.0 * a;
    add(a, a, a, w); add(a, a, b, w); add(a, b, a, w); add(b, a, a, w);
  };
  auto sym22 = [&](double c, double w) {
    const double d2 = 0.5 - c;
    add(c, c, d2, w); add(c, d2, c, w); add(c, d2, d2, w); add(d2, c, c, w); add(d2, c, d2, w); add(d2, d2, c, w);
  };
  for (int d = 0; d <= 3; d++)
    for (int p = 0; p <= kMaxOrder; p++) {
      t.off[d][p] = n;
      int m = p / 2 + 1;
      if (d == 0) {
        add(0, 0, 0, 1.0);
      } else if (d == 1) {
        std::vector<double> x, w;
        gauss_jacobi01(m, 0, x, w);
        for (int i = 0; i < m; i++) add(x[i], 0, 0, w[i]);
      } else if (d == 2) {
        if (p <= 1) add(1.0 / 3, 1.0 / 3, 0, 0.5);
        else if (p == 2) {
          add(1.0 / 6, 1.0 / 6, 0, 1.0 / 6);
          add(2.0 / 3, 1.0 / 6, 0, 1.0 / 6);
          add(1.0 / 6, 2.0 / 3, 0, 1.0 / 6);
        } else if (p == 4) {
          sym21(0.4459484909159648863183293, 0.1116907948390057328475035);
          sym21(0.09157621350977074345957146, 0.05497587182766093381916316);
        } else if (p == 5) {
          add(1.0 / 3, 1.0 / 3, 0, 0.1125);
          sym21(0.4701420641051150897704412, 0.06619707639425309036882469);
          sym21(0.1012865073234563388009874, 0.06296959027241357629784197);
        } else {
          std::vector<double> xu, wu, xv, wv;
          gauss_jacobi01(m, 1, xu, wu);
          gauss_jacobi01(m, 0, xv, wv);
          for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++) add(xu[i], xv[j] * (1 - xu[i]), 0, wu[i] * wv[j]);
        }
      } else {
        if (p <= 1) add(0.25, 0.25, 0.25, 1.0 / 6);
        else if (p == 2) {
          double a = (5.0 + 3.0 * std::sqrt(5.0)) / 20.0, b = (5.0 - std::sqrt(5.0)) / 20.0;
          add(a, b, b, 1.0 / 24);
          add(b, a, b, 1.0 / 24);
          add(b, b, a, 1.0 / 24);
          add(b, b, b, 1.0 / 24);
        } else if (p == 4 || p == 5) {
          sym31(0.09273525031089122640232391, 0.01224884051939365825728503);
          sym31(0.3108859192633006097973457, 0.01878132095300264179986428);
          sym22(0.4544962958743503505081195, 0.007091003462846911073011571);
        } else {
          std::vector<double> xu, wu, xv, wv, xw, ww;
          gauss_jacobi01(m, 2, xu, wu);
          gauss_jacobi01(m, 1, xv, wv);
          gauss_jacobi01(m, 0, xw, ww);
          for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++)
              for (int k = 0; k < m; k++) {
                double u = xu[i], v = xv[j], s = xw[k];
                add(u, (1 - u) * v, (1 - u) * (1 - v) * s, wu[i] * wv[j] * ww[k]);
              }
        }
      }
      t.cnt[d][p] = n - t.off[d][p];
    }
  if (n > kRuleCap) std::abort();
  return t;
}

const RuleTable& host_rules() {
  static RuleTable t = build_rules();
  return t;
}

}  // namespace xg

using namespace xg;

namespace {
template <class T>
int upload(T** d, const std::vector<T>& h) {
  if (h.empty()) { *d = nullptr; return XG_OK; }
  XG_CUDA(cudaMalloc((void**)d, sizeof(T) * h.size()));
  XG_CUDA(cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  return XG_OK;
}
// AoS (n x m) -> SoA (m x n)
template <class T>
std::vector<T> to_soa(const std::vector<T>& a, size_t n, int m) {
  std::vector<T> s(a.size());
  for (size_t i = 0; i < n; i++)
    for (int j = 0; j < m; j++) s[(size_t)j * n + i] = a[i * m + j];
  return s;
}
}  // namespace

extern "C" {

const char* xg_status_string(int s) {
  switch (s) {
    case XG_OK: return "ok";
    case XG_ERR_ARG: return "invalid argument";
    case XG_ERR_CUDA: return "CUDA error";
    case XG_ERR_CAPACITY: return "capacity exceeded";
    case XG_ERR_PLAIN_CUT: return "cut requested on an uncut (sub-)simplex";
    case XG_ERR_BAD_DECOMP: return "unsupported cut topology";
    case XG_ERR_UNSUPPORTED: return "unsupported element, order or term";
    case XG_ERR_NONFINITE: return "non-finite weight or matrix entry";
    case XG_ERR_NO_DEVICE: return "no usable CUDA device";
    case XG_ERR_IF_BOUND: return "quadrilateral interface scaling factor above its bound";
    case XG_ERR_TIMEOUT: return "a bounded device wait timed out";
  }
  return "unknown status";
}

const char* xg_last_error(void) { return g_last_error.c_str(); }

int xg_device_ok(int* ok) {
  *ok = 0;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    set_last_error(e != cudaSuccess ? cudaGetErrorString(e) : "no device");
    return XG_ERR_NO_DEVICE;
  }
  int dev = 0;
  XG_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  XG_CUDA(cudaGetDeviceProperties(&prop, dev));
  *ok = (prop.major == 10 && prop.minor == 3) ? 1 : 0;
  if (!*ok) {
    set_last_error("device is sm_" + std::to_string(prop.major) + std::to_string(prop.minor) +
                   ", library is built for sm_103a only");
    return XG_ERR_NO_DEVICE;
  }
  return XG_OK;
}

int xg_base_rule_size(int d, int p) {
  if (d < 0 || d > 3) return -1;
  return host_rules().cnt[d][clamp_order(p)];
}

int xg_base_rule(int d, int p, double* h_pts, double* h_wts, int max_pts) {
  if (d < 0 || d > 3 || !h_pts || !h_wts) return -1;
  const RuleTable& t = host_rules();
  const int q = clamp_order(p), off = t.off[d][q], cnt = t.cnt[d][q];
  if (cnt > max_pts) return -1;
  for (int i = 0; i < cnt; i++) {
    for (int c = 0; c < 3; c++) h_pts[3 * i + c] = t.x[off + i][c];
    h_wts[i] = t.w[off + i];
  }
  return cnt;
}

int xg_mesh_create(int dim, int32_t nv, const double* h_coords, int32_t ne, const int32_t* h_elv, xg_mesh** out) {
  if (!out || (dim != 2 && dim != 3) || nv <= 0 || ne <= 0 || !h_coords || !h_elv) {
    set_last_error("xg_mesh_create: bad arguments");
    return XG_ERR_ARG;
  }
  if (ne >= (1 << 26)) {
    set_last_error("xg_mesh_create: more than 2^26 elements");
    return XG_ERR_CAPACITY;
  }
  *out = nullptr;
  auto* m = new xg_mesh();
  m->dim = dim; m->nv = nv; m->ne = ne;
  cudaGetDevice(&m->device);
  const int nvl = dim + 1;
  m->h_elv.assign(h_elv, h_elv + (size_t)ne * nvl);
  for (size_t i = 0; i < m->h_elv.size(); i++)
    if (m->h_elv[i] < 0 || m->h_elv[i] >= nv) {
      delete m;
      set_last_error("xg_mesh_create: vertex index out of range");
      return XG_ERR_ARG;
    }
  // edges and faces numbered in lexicographic order of their vertex tuples
  const int nel = dim == 2 ? 3 : 6;
  m->nedges = number_edges(dim, ne, h_elv, m->h_el_edges);
  if (dim == 3) m->nfaces = number_faces(ne, h_elv, m->h_el_faces);
  m->nfacets = dim == 2 ? m->nedges : m->nfaces;
  const std::vector<int32_t>& elf = dim == 2 ? m->h_el_edges : m->h_el_faces;
  const int nfl = dim + 1;
  m->h_facet_els.assign((size_t)m->nfacets * 2, -1);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < nfl; j++) {
      int f = elf[(size_t)e * (dim == 2 ? 3 : 4) + j];
      if (m->h_facet_els[2 * (size_t)f] < 0) m->h_facet_els[2 * (size_t)f] = e;
      else if (m->h_facet_els[2 * (size_t)f + 1] < 0) m->h_facet_els[2 * (size_t)f + 1] = e;
      else {
        delete m;
        set_last_error("xg_mesh_create: facet shared by more than two elements");
        return XG_ERR_ARG;
      }
    }
  {
    std::vector<int> cnt(nv, 0);
    for (size_t i = 0; i < m->h_elv.size(); i++) cnt[m->h_elv[i]]++;
    m->max_vertex_elems = *std::max_element(cnt.begin(), cnt.end());
  }
  // BND elements: boundary facets in facet order, vertices in ascending order
  std::vector<int32_t> bnd_v;
  {
    const int stride = dim == 2 ? 3 : 4;
    for (int64_t f = 0; f < m->nfacets; f++)
      if (m->h_facet_els[2 * (size_t)f + 1] < 0) m->h_bnd_facets.push_back((int32_t)f);
    m->nbnd = (int64_t)m->h_bnd_facets.size();
    bnd_v.resize((size_t)dim * m->nbnd);
    for (int64_t b = 0; b < m->nbnd; b++) {
      const int f = m->h_bnd_facets[b], e = m->h_facet_els[2 * (size_t)f];
      int lf = 0;
      while (elf[(size_t)e * stride + lf] != f) lf++;
      int v[3];
      for (int q = 0; q < dim; q++) v[q] = h_elv[(size_t)e * nvl + (dim == 2 ? TRI_EDGES[lf][q] : TET_FACES[lf][q])];
      std::sort(v, v + dim);
      for (int q = 0; q < dim; q++) bnd_v[(size_t)q * m->nbnd + b] = v[q];
    }
  }
  // upload (SoA)
  std::vector<double> xyz((size_t)dim * nv);
  for (int v = 0; v < nv; v++)
    for (int c = 0; c < dim; c++) xyz[(size_t)c * nv + v] = h_coords[(size_t)v * dim + c];
  int st = XG_OK;
  if ((st = upload(&m->d_xyz, xyz)) || (st = upload(&m->d_elv, to_soa(m->h_elv, ne, nvl))) ||
      (st = upload(&m->d_el_edges, to_soa(m->h_el_edges, ne, nel))) ||
      (dim == 3 && (st = upload(&m->d_el_faces, to_soa(m->h_el_faces, ne, 4)))) ||
      (st = upload(&m->d_facet_els, to_soa(m->h_facet_els, (size_t)m->nfacets, 2))) ||
      (st = upload(&m->d_bnd_v, bnd_v))) {
    xg_mesh_destroy(m);
    return st;
  }
  {
    std::vector<int32_t> efa((size_t)ne * nvl);
    const std::vector<int32_t>& src = dim == 2 ? m->h_el_edges : m->h_el_faces;
    const int stride = dim == 2 ? 3 : 4;
    for (int e = 0; e < ne; e++)
      for (int j = 0; j < nvl; j++) efa[(size_t)e * nvl + j] = src[(size_t)e * stride + j];
    st = upload(&m->d_el_facets_aos, efa);
    if (!st) {
      XG_CUDA(cudaMalloc((void**)&m->d_facet_els_aos, sizeof(int2) * (size_t)m->nfacets));
      XG_CUDA(cudaMemcpy(m->d_facet_els_aos, m->h_facet_els.data(), sizeof(int2) * (size_t)m->nfacets,
                         cudaMemcpyHostToDevice));
    }
  }
  if (st) {
    xg_mesh_destroy(m);
    return st;
  }
  m->d_el_facets = dim == 2 ? m->d_el_edges : m->d_el_faces;
  if (cudaMalloc((void**)&m->d_err, sizeof(int)) != cudaSuccess || cudaMemset(m->d_err, 0, sizeof(int)) != cudaSuccess ||
      cudaMalloc((void**)&m->d_cutlist, sizeof(int32_t) * ((size_t)std::max<int64_t>(m->ne, m->nbnd) + 1)) !=
          cudaSuccess) {
    xg_mesh_destroy(m);
    set_last_error("xg_mesh_create: cudaMalloc failed");
    return XG_ERR_CUDA;
  }
  if ((st = ensure_device_rules())) {
    xg_mesh_destroy(m);
    return st;
  }
  *out = m;
  return XG_OK;
}

int xg_mesh_create_tensor(int dim, int32_t nv, const double* h_coords, int32_t ne, const int32_t* h_elv,
                          xg_mesh** out) {
  if (!out || (dim != 2 && dim != 3) || nv <= 0 || ne <= 0 || !h_coords || !h_elv) {
    set_last_error("xg_mesh_create_tensor: bad arguments");
    return XG_ERR_ARG;
  }
  *out = nullptr;
  const int nvl = 1 << dim;
  for (size_t i = 0; i < (size_t)ne * nvl; i++)
    if (h_elv[i] < 0 || h_elv[i] >= nv) {
      set_last_error("xg_mesh_create_tensor: vertex index out of range");
      return XG_ERR_ARG;
    }
  auto* m = new xg_mesh();
  m->dim = dim; m->nv = nv; m->ne = ne; m->tensor = 1;
  cudaGetDevice(&m->device);
  m->h_elv.assign(h_elv, h_elv + (size_t)ne * nvl);
  std::vector<double> xyz((size_t)dim * nv);
  for (int v = 0; v < nv; v++)
    for (int c = 0; c < dim; c++) xyz[(size_t)c * nv + v] = h_coords[(size_t)v * dim + c];
  int st = XG_OK;
  if ((st = upload(&m->d_xyz, xyz)) || (st = upload(&m->d_elv, to_soa(m->h_elv, ne, nvl)))) {
    xg_mesh_destroy(m);
    return st;
  }
  if (cudaMalloc((void**)&m->d_err, sizeof(int)) != cudaSuccess || cudaMemset(m->d_err, 0, sizeof(int)) != cudaSuccess) {
    xg_mesh_destroy(m);
    set_last_error("xg_mesh_create_tensor: cudaMalloc failed");
    return XG_ERR_CUDA;
  }
  if ((st = ensure_device_rules())) {
    xg_mesh_destroy(m);
    return st;
  }
  *out = m;
  return XG_OK;
}

int xg_mesh_destroy(xg_mesh* m) {
  if (!m) return XG_OK;
  cudaFree(m->d_xyz);
  cudaFree(m->d_elv);
  cudaFree(m->d_el_edges);
  cudaFree(m->d_el_faces);
  cudaFree(m->d_facet_els);
  cudaFree(m->d_bnd_v);
  cudaFree(m->d_el_facets_aos);
  cudaFree(m->d_facet_els_aos);
  cudaFree(m->d_err);
  cudaFree(m->d_cutlist);
  cudaFree(m->d_edge_ptr);
  cudaFree(m->d_edge_inc);
  cudaFree(m->d_iso);
  cudaFree(m->d_scratch);
  delete m;
  return XG_OK;
}

int xg_mesh_info(const xg_mesh* m, int64_t* o) {
  if (!m || !o) return XG_ERR_ARG;
  o[0] = m->dim; o[1] = m->nv; o[2] = m->ne; o[3] = m->nedges; o[4] = m->nfaces; o[5] = m->nfacets;
  return XG_OK;
}

int xg_mesh_boundary(const xg_mesh* m, int64_t* h_nbnd, int32_t* h_facets) {
  if (!m || !h_nbnd) return XG_ERR_ARG;
  *h_nbnd = m->nbnd;
  if (h_facets) std::copy(m->h_bnd_facets.begin(), m->h_bnd_facets.end(), h_facets);
  return XG_OK;
}

int xg_mesh_facet_elements(const xg_mesh* m, int32_t* h_out) {
  if (!m || !h_out) return XG_ERR_ARG;
  std::memcpy(h_out, m->h_facet_els.data(), sizeof(int32_t) * m->h_facet_els.size());
  return XG_OK;
}

int xg_space_create(xg_mesh* m, int order, xg_space** out) {
  if (!m || !out || order < 1 || order > 3) {
    set_last_error("xg_space_create: order must be 1..3");
    return XG_ERR_ARG;
  }
  if (m->tensor) {
    set_last_error("xg_space_create: H1 spaces are built on simplex meshes only");
    return XG_ERR_UNSUPPORTED;
  }
  *out = nullptr;
  auto* s = new xg_space();
  const int D = m->dim, k = order, ne = m->ne, nvl = D + 1;
  s->mesh = m;
  s->order = k;
  s->nd = D == 2 ? (k + 1) * (k + 2) / 2 : (k + 1) * (k + 2) * (k + 3) / 6;
  s->nds = s->nd;
  const int nd = s->nd, nel = D == 2 ? 3 : 6;
  const int64_t nbub = (k == 3) ? (D == 3 ? m->nfaces : ne) : 0;
  s->ndof = m->nv + m->nedges * (k - 1) + nbub;
  s->ndof_s = s->ndof;
  if (s->ndof >= ((int64_t)1 << 31)) {
    delete s;
    set_last_error("xg_space_create: more than 2^31 dofs");
    return XG_ERR_CAPACITY;
  }
  s->h_el_dofs.resize((size_t)ne * nd);
  for (int e = 0; e < ne; e++) {
    int32_t* d = &s->h_el_dofs[(size_t)e * nd];
    int n = 0;
    for (int i = 0; i < nvl; i++) d[n++] = m->h_elv[(size_t)e * nvl + i];
    if (k >= 2)
      for (int j = 0; j < nel; j++)
        for (int q = 0; q < k - 1; q++) d[n++] = (int32_t)(m->nv + (int64_t)m->h_el_edges[(size_t)e * nel + j] * (k - 1) + q);
    if (k == 3) {
      if (D == 3)
        for (int j = 0; j < 4; j++) d[n++] = (int32_t)(m->nv + m->nedges * 2 + m->h_el_faces[(size_t)e * 4 + j]);
      else
        d[n++] = (int32_t)(m->nv + m->nedges * 2 + e);
    }
  }
  std::vector<int32_t> ptr(s->ndof + 1, 0);
  for (size_t i = 0; i < s->h_el_dofs.size(); i++) ptr[s->h_el_dofs[i] + 1]++;
  int mx = 0;
  for (int64_t i = 0; i < s->ndof; i++) {
    mx = std::max(mx, ptr[i + 1]);
    ptr[i + 1] += ptr[i];
  }
  s->max_adj = mx;
  std::vector<int32_t> adj(s->h_el_dofs.size());
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
  for (int e = 0; e < ne; e++)
    for (int i = 0; i < nd; i++) adj[fill[s->h_el_dofs[(size_t)e * nd + i]]++] = e * 32 + i;
  int st;
  if ((st = upload(&s->d_el_dofs, to_soa(s->h_el_dofs, ne, nd))) || (st = upload(&s->d_el_dofs_aos, s->h_el_dofs)) ||
      (st = upload(&s->d_dof_adj_ptr, ptr)) ||
      (st = upload(&s->d_dof_adj, adj))) {
    xg_space_destroy(s);
    return st;
  }
  *out = s;
  return XG_OK;
}

int xg_space_create_l2(xg_mesh* m, int order, xg_space** out) {
  if (!m || !out || order < 1 || order > 3) {
    set_last_error("xg_space_create_l2: order must be 1..3");
    return XG_ERR_ARG;
  }
  if (m->tensor) {
    set_last_error("xg_space_create_l2: L2 spaces are built on simplex meshes only");
    return XG_ERR_UNSUPPORTED;
  }
  *out = nullptr;
  auto* s = new xg_space();
  const int D = m->dim, ne = m->ne;
  s->mesh = m;
  s->order = order;
  s->nd = D == 2 ? (order + 1) * (order + 2) / 2 : (order + 1) * (order + 2) * (order + 3) / 6;
  s->nds = s->nd;
  const int nd = s->nd;
  s->ndof = (int64_t)ne * nd;
  s->ndof_s = s->ndof;
  if (s->ndof >= ((int64_t)1 << 31)) {
    delete s;
    set_last_error("xg_space_create_l2: more than 2^31 dofs");
    return XG_ERR_CAPACITY;
  }
  s->h_el_dofs.resize((size_t)s->ndof);
  std::vector<int32_t> ptr(s->ndof + 1), adj((size_t)s->ndof);
  for (int64_t i = 0; i < s->ndof; i++) {
    s->h_el_dofs[i] = (int32_t)i;
    ptr[i + 1] = (int32_t)(i + 1);
    adj[i] = (int32_t)((i / nd) * 32 + i % nd);
  }
  s->max_adj = 1;
  int st;
  if ((st = upload(&s->d_el_dofs, to_soa(s->h_el_dofs, ne, nd))) || (st = upload(&s->d_el_dofs_aos, s->h_el_dofs)) ||
      (st = upload(&s->d_dof_adj_ptr, ptr)) || (st = upload(&s->d_dof_adj, adj))) {
    xg_space_destroy(s);
    return st;
  }
  *out = s;
  return XG_OK;
}

int xg_space_create_st(xg_mesh* m, int order, int order_time, xg_space** out) {
  if (!m || !out || order < 1 || order > 3 || order_time < 0 || order_time > 2) {
    set_last_error("xg_space_create_st: space order 1..3, time order 0..2");
    return XG_ERR_ARG;
  }
  if (m->tensor) {
    set_last_error("xg_space_create_st: space-time spaces are built on simplex meshes only");
    return XG_ERR_UNSUPPORTED;
  }
  *out = nullptr;
  xg_space* sp = nullptr;
  int st = xg_space_create(m, order, &sp);
  if (st) return st;
  const int nds = sp->nd, nt = order_time + 1, N = nds * nt, ne = m->ne;
  const int64_t ndof_s = sp->ndof;
  if (N > 32 || ndof_s * nt >= ((int64_t)1 << 31)) {
    xg_space_destroy(sp);
    set_last_error("xg_space_create_st: too many space-time dofs per element or in total");
    return XG_ERR_CAPACITY;
  }
  std::vector<int32_t> spatial = sp->h_el_dofs;
  cudaFree(sp->d_el_dofs);
  cudaFree(sp->d_el_dofs_aos);
  cudaFree(sp->d_dof_adj_ptr);
  cudaFree(sp->d_dof_adj);
  sp->d_el_dofs = sp->d_el_dofs_aos = sp->d_dof_adj_ptr = sp->d_dof_adj = nullptr;
  sp->kt = order_time;
  sp->nds = nds;
  sp->ndof_s = ndof_s;
  sp->nd = N;
  sp->ndof = ndof_s * nt;
  sp->h_el_dofs.resize((size_t)ne * N);
  for (int e = 0; e < ne; e++)
    for (int it = 0; it < nt; it++)
      for (int j = 0; j < nds; j++)
        sp->h_el_dofs[(size_t)e * N + it * nds + j] = (int32_t)(it * ndof_s + spatial[(size_t)e * nds + j]);
  std::vector<int32_t> ptr(sp->ndof + 1, 0);
  for (size_t i = 0; i < sp->h_el_dofs.size(); i++) ptr[sp->h_el_dofs[i] + 1]++;
  int mx = 0;
  for (int64_t i = 0; i < sp->ndof; i++) {
    mx = std::max(mx, ptr[i + 1]);
    ptr[i + 1] += ptr[i];
  }
  sp->max_adj = mx;
  std::vector<int32_t> adj(sp->h_el_dofs.size());
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
  for (int e = 0; e < ne; e++)
    for (int i = 0; i < N; i++) adj[fill[sp->h_el_dofs[(size_t)e * N + i]]++] = e * 32 + i;
  if ((st = upload(&sp->d_el_dofs, to_soa(sp->h_el_dofs, ne, N))) || (st = upload(&sp->d_el_dofs_aos, sp->h_el_dofs)) ||
      (st = upload(&sp->d_dof_adj_ptr, ptr)) || (st = upload(&sp->d_dof_adj, adj))) {
    xg_space_destroy(sp);
    return st;
  }
  *out = sp;
  return XG_OK;
}

int xg_space_destroy(xg_space* s) {
  if (!s) return XG_OK;
  cudaFree(s->d_el_dofs);
  cudaFree(s->d_el_dofs_aos);
  cudaFree(s->d_dof_adj_ptr);
  cudaFree(s->d_dof_adj);
  delete s;
  return XG_OK;
}

int xg_space_info(const xg_space* s, int64_t* o) {
  if (!s || !o) return XG_ERR_ARG;
  o[0] = s->ndof; o[1] = s->nd; o[2] = s->order;
  return XG_OK;
}

int xg_space_info_st(const xg_space* s, int64_t* o) {
  if (!s || !o) return XG_ERR_ARG;
  o[0] = s->ndof; o[1] = s->nd; o[2] = s->order; o[3] = s->kt; o[4] = s->ndof_s; o[5] = s->nds;
  return XG_OK;
}

int xg_space_element_dofs(const xg_space* s, int32_t* h_out) {
  if (!s || !h_out) return XG_ERR_ARG;
  std::memcpy(h_out, s->h_el_dofs.data(), sizeof(int32_t) * s->h_el_dofs.size());
  return XG_OK;
}

}  // extern "C"

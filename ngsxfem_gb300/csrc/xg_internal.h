// Internal declarations shared by the host objects and the kernels of libxg.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/xg.h"

struct xg_mesh;

namespace xg {

// ---- quadrature rule family (host-built, device __constant__) ------------------
// segment order p: Gauss-Legendre with p/2+1 points on [0,1]
// trig: p<=1 centroid; p==2 3-point (1/6,1/6,2/3); p==4 6-point and p==5
//       7-point fully symmetric rules; otherwise collapsed Gauss-Jacobi
//       conical product, p/2+1 points per direction
// tet : p<=1 centroid; p==2 4-point (a,b,b,b), a=(5+3sqrt5)/20; p==4,5
//       14-point fully symmetric rule; otherwise conical product, p/2+1
//       points per direction
constexpr int kMaxOrder = 8;
constexpr int kRuleCap = 512;  // total points of all tables

struct RuleTable {
  int off[4][kMaxOrder + 1];
  int cnt[4][kMaxOrder + 1];
  double x[kRuleCap][3];
  double w[kRuleCap];
};
const RuleTable& host_rules();
int ensure_device_rules();  // uploads the table to the current device (once per device)

#ifdef __CUDACC__
__host__ __device__
#endif
inline int clamp_order(int p) { return p < 0 ? 0 : (p > kMaxOrder ? kMaxOrder : p); }

// ---- device error word -----------------------------------------------------------
// first error wins (atomicCAS from 0)
#ifdef __CUDACC__
__device__ __forceinline__ void set_err(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// mesh size h = |det F|^(1/D) and h^hp for the integer powers of the
// coefficients (cbrt / sqrt and repeated products instead of two pow calls)
template <int D>
__device__ __forceinline__ double mesh_h(double meas) {
  return D == 3 ? cbrt(meas) : (D == 2 ? sqrt(meas) : meas);
}
__device__ __forceinline__ double int_pow(double h, int hp) {
  double r = 1.0;
  for (int k = 0; k < (hp < 0 ? -hp : hp); k++) r *= h;
  return hp < 0 ? 1.0 / r : r;
}

// finiteness and sign flips on the bit pattern (integer pipe; the FP64 pipe of
// GB300 is narrow and also issues comparisons and negations)
__device__ __forceinline__ bool finite_bits(double v) {
  return ((__double_as_longlong(v) >> 52) & 0x7ff) != 0x7ff;
}
__device__ __forceinline__ bool finite_bits(float v) { return ((__float_as_int(v) >> 23) & 0xff) != 0xff; }
__device__ __forceinline__ double neg_if(double v, bool c) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v) ^ ((unsigned long long)c << 63);
  return __longlong_as_double((long long)b);
}
__device__ __forceinline__ float neg_if(float v, bool c) {
  return __uint_as_float(__float_as_uint(v) ^ ((unsigned)c << 31));
}
#endif

// ---- errors ----------------------------------------------------------------------
void set_last_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
#define XG_CUDA(call)                                 \
  do {                                                \
    cudaError_t _e = (call);                          \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

// ---- term groups passed by value to the kernels -------------------------------
constexpr int kMaxGroups = 6;
constexpr int kMaxPatch = 4;

// volume terms with equal (domain, order, defined_on) share one quadrature rule
struct GroupDesc {
  int domain;
  int order;
  const uint64_t* defined_on;
  double c[5];    // coefficients of MASS, LAPLACE, NGRADU_V, U_NGRADV, CONV
  int hpow[5];
  int used;       // bitmask of kinds present
  double b[3];
};
struct PatchDesc {
  int order;
  const uint64_t* defined_on;
  double c;
  int hpow;
};
// skeleton terms (XG_TERM_SKEL_*) with equal (region, defined_on) share one
// facet rule; c / hpow per kind, index kind - XG_TERM_SKEL_JUMP
constexpr int kMaxSkel = 4;
constexpr int kSkelKinds = 6;
struct SkelDesc {
  int region;                  // XG_NEG / XG_POS: the facet cut to the domain; XG_WHOLE: all of it
  const uint64_t* defined_on;  // facet bits, NULL = every interior facet
  int used;                    // bit (kind - XG_TERM_SKEL_JUMP)
  double c[kSkelKinds];
  int hpow[kSkelKinds];
};
struct FormDesc {
  int ngroups;
  GroupDesc g[kMaxGroups];
  int npatch;
  PatchDesc p[kMaxPatch];
  int nskel;
  SkelDesc s[kMaxSkel];
};

// space-time volume terms with equal (domain, order, defined_on, tref,
// convection) share one space-time rule
struct StGroupDesc {
  int domain;
  int order;       // spatial rule order
  const uint64_t* defined_on;
  double tref;     // < 0: over the slab; >= 0: fixed reference time (spatial rule of the trace)
  double c[7];     // coefficients per kind (MASS, LAPLACE, -, -, CONV, -, DT_U_V)
  int hpow[7];
  int used;
  double b[3], bc[3], bs[3];  // convection b(t) = b + bc cos(omega t) + bs sin(omega t)
  double omega, t0, dt;       // t = t0 + dt * tau
};
struct StFormDesc {
  int ngroups;
  StGroupDesc g[kMaxGroups];
  int kt_l;        // time order of the level set
  int order_time;  // time rule order
};
struct StLaunch {
  int D, K, KT, precision;
  int ne, nv;
  const int32_t* elv;
  const double* xyz;
  const double* lset_st;
  StFormDesc desc;
  const int32_t* list;
  const int* count;
  const int* slot_base;  // element-matrix slot of list entry 0 (device), or null for 0
  void* elmat;
  int* err;
};
int launch_st_elmat(const StLaunch& a, cudaStream_t s);

// CutInfo updates with a caller-owned list of the cut elements ([ne + 1] ints;
// forms pass their own so that forms of one mesh may run concurrently)
int cutinfo_update_ws(xg_mesh* m, const double* d_lset, uint8_t* d_dom, double* d_ratio, uint64_t* d_bits,
                      int32_t* cutlist, void* stream);
int cutinfo_update_st_ws(xg_mesh* m, const double* d_lset_st, int kt_lset, uint8_t* d_dom, double* d_ratio,
                         uint64_t* d_bits, int32_t* cutlist, void* stream);

// quadrilateral / hexahedral meshes (xg_quad.cu)
int upload_rules_quad();
int upload_rules_quad_int();
int upload_rules_mlset();
int upload_rules_isomesh();
int upload_rules_skel();  // xg_skel.cu
int upload_rules_subdiv();  // xg_subdiv.cu
int upload_rules_mlform();  // xg_mlform.cu

// a bilinear-form term on a region of several level sets (device copy)
struct MlTermDev {
  int kind, order, hpow, normal_lset;
  int ntup, tup_off;           // the region: ntup tuples of M entries at tuples + tup_off
  double coef;
  double b[3];
  const uint64_t* defined_on;  // element bits, NULL = all
};
// the element matrices of such terms for the listed elements (xg_mlform.cu),
// written at the elements' row slots
struct MlFormLaunch {
  int dim, order, M;
  int ne, nv;
  const int32_t* elv;
  const double* xyz;
  const double* lsets;         // [M][nv]
  const MlTermDev* terms;
  int nterms;
  const int8_t* tuples;
  const int32_t* list;         // active elements
  const int* counts;           // [1]: their number
  const int32_t* rowslot;
  void* elmat;
  int fp64;
  int* err;
};
int mlform_launch(const MlFormLaunch& launch, cudaStream_t s);
// per-element NEG moments of P2 level sets on the reference tetrahedron by
// the subdivision rule (xg_subdiv.cu); with d_list, only the d_count listed
// elements
int subdiv_moments_launch(const double* d_vals10, int64_t n, int levels, double* d_out35, const int32_t* d_list,
                          const int32_t* d_count, int* d_err, cudaStream_t s);

// skeleton terms of a form (xg_skel.cu): the facet matrices of the active
// facet list, written into (accumulate = 0) or added to (1) famat, full rows
// of 2 nd per facet slot
struct SkelLaunch {
  int dim, order;
  int ne, nv;
  const int32_t* elv;   // [D+1][ne]
  const double* xyz;    // [3][nv]
  int64_t nf;
  const int32_t* fel;   // [2][nf]
  const double* lset;   // P1 vertex values
  const int32_t* l_fa;  // active facets
  const int* counts;    // [2]: number of active facets
  void* famat;
  int64_t cap_fa;
  int accumulate;
  int fp64;
  int* err;
};
int skel_launch(const SkelLaunch& a, const FormDesc& form, cudaStream_t s);

// boundary terms of bilinear forms (xg_form_set_bnd_terms; xg_bform.cu)
constexpr int kMaxBnd = 8;
struct BndTermDev {
  int domain, order, hpow;
  double coef;
  const uint64_t* defined_on;  // BND element bits; NULL = all
};
struct BndDesc {
  int n;
  BndTermDev t[kMaxBnd];
};
struct BndFormLaunch {
  int dim, order;
  int ne, nv;
  const int32_t* elv;    // [D+1][ne]
  const double* xyz;     // [D][nv]
  const double* lset;    // P1 vertex values
  int64_t nbnd;
  const int32_t* bnd_v;  // [D][nbnd]
  int n_own;             // elements owning a BND element, ascending
  const int32_t* own_el;
  const int32_t* own_ptr;  // [n_own + 1]
  const int32_t* own_bnd;  // their BND elements, ascending per owner
  BndDesc d;
  uint32_t* act_un;
  const uint32_t* act_cut;
  const int32_t* rowslot;  // [ne][nd] element row slots
  void* elmat;
  int fp64;
  int* err;
};
// volume terms with a coefficient field (xg_form_set_coef_terms; xg_cform.cu)
constexpr int kMaxCoef = 8;
struct CoefTermDev {
  int kind, domain, order, hpow;
  double coef, b[3];
  int e[3];
  int gf_order;            // 0: no coefficient field
  const int32_t* gf_dofs;  // [nd_gf][ne] element dofs of its space
  const double* gf;        // its coefficients
  const uint64_t* defined_on;
  const double* gdef;      // mesh deformation [nedges][3] (physical edge coefficients) or NULL
};
struct CoefDesc {
  int n;
  CoefTermDev t[kMaxCoef];
};
struct CoefFormLaunch {
  int dim, order;
  int ne, nv;
  const int32_t* elv;
  const double* xyz;
  const int32_t* el_edges; // [nedges per element][ne]
  const double* lset;      // P1 vertex values
  const uint8_t* dom;      // element domain types
  CoefDesc d;
  uint32_t* act_un;
  const uint32_t* act_cut;
  int64_t nw32;
  const int32_t* l_un;     // active elements: uncut list, then cut list
  const int32_t* l_cut;
  const int* counts;
  const int32_t* rowslot;
  void* elmat;
  int fp64;
  int* err;
};
// facet-patch terms on the deformed mesh (xg_form_set_deformation; xg_cform.cu)
struct PatchDefLaunch {
  int dim, order;
  int ne, nv;
  const int32_t* elv;
  const double* xyz;
  const int32_t* el_edges;
  const double* gdef;      // [nedges][3]
  int64_t nf;
  const int32_t* fel;      // [2][nf]
  const int32_t* l_fa;     // active facets
  const int* counts;       // [2]: their number
  int npatch;
  PatchDesc p[kMaxPatch];
  void* famat;             // [slot][2n][2n] full rows
  int64_t cap_fa;
  int fp64;
  int* err;
};
int patch_def_launch(const PatchDefLaunch& a, cudaStream_t s);
int coef_active_launch(const CoefFormLaunch& a, cudaStream_t s);
int coef_elmat_launch(const CoefFormLaunch& a, cudaStream_t s);
int upload_rules_cform();
int upload_rules_qform();  // xg_qform.cu
int bnd_active_launch(const BndFormLaunch& a, cudaStream_t s);
int bnd_elmat_launch(const BndFormLaunch& a, cudaStream_t s);
int upload_rules_bform();
int quad_rule_capacity(int dim, int dt, int order);
int quad_cut_rules(xg_mesh* m, const double* d_lset, const int32_t* d_elems, int32_t n, int dt, int order, int pol,
                   int32_t max_pts, int32_t* d_counts, double* d_pts, double* d_wts, void* stream);
int quad_integrate(xg_mesh* m, const double* d_lset, int dt, int order, int pol, int ex, int ey, int ez,
                   const uint64_t* d_defined_on, double* d_result, void* stream);
int quad_cutinfo(xg_mesh* m, const double* d_lset, uint8_t* d_dom, double* d_ratio, uint64_t* d_bits, void* stream);

}  // namespace xg

// ---- objects behind the opaque handles ------------------------------------------
struct xg_mesh {
  int dim = 0, nv = 0, ne = 0, device = 0;
  int tensor = 0;  // 1: quadrilaterals / hexahedra (2^dim vertices, no facet topology)
  int64_t nedges = 0, nfaces = 0, nfacets = 0;
  int max_vertex_elems = 0;  // max elements sharing a vertex
  // device (SoA)
  double* d_xyz = nullptr;       // [dim][nv]
  int32_t* d_elv = nullptr;      // [dim+1][ne] ([2^dim][ne] for tensor meshes)
  int32_t* d_el_edges = nullptr; // [3|6][ne]
  int32_t* d_el_faces = nullptr; // [4][ne] (3D)
  int32_t* d_el_facets = nullptr;// [dim+1][ne] (alias of edges / faces)
  int32_t* d_facet_els = nullptr;// [2][nfacets]
  int32_t* d_el_facets_aos = nullptr;  // [ne][dim+1] element-major
  int2* d_facet_els_aos = nullptr;     // [nfacets] (first, second element; -1 boundary)
  int64_t nbnd = 0;                    // BND elements: the boundary facets in facet order
  int32_t* d_bnd_v = nullptr;          // [dim][nbnd] their vertices, ascending
  int* d_err = nullptr;
  int32_t* d_cutlist = nullptr;  // [max(ne, nbnd) + 1]: count, then the cut elements of the last marking
  int32_t* d_edge_ptr = nullptr; // [nedges + 1] edge -> incident elements (isoparametric averaging)
  int32_t* d_edge_inc = nullptr; // element * 8 + local edge, elements ascending
  void* d_iso = nullptr;         // isoparametric workspace
  size_t iso_bytes = 0;
  // host
  std::vector<int32_t> h_elv;       // ne*(dim+1)
  std::vector<int32_t> h_el_edges;  // ne*nel_edges
  std::vector<int32_t> h_el_faces;  // ne*4
  std::vector<int32_t> h_facet_els; // nfacets*2
  std::vector<int32_t> h_bnd_facets; // nbnd
  // compaction scratch (sized for max(ne, nfacets))
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
};

struct xg_space {
  xg_mesh* mesh = nullptr;
  int order = 1, nd = 0;
  int64_t ndof = 0;
  int kt = -1;          // time order of a space-time space (-1: spatial space)
  int nds = 0;          // spatial dofs per element
  int64_t ndof_s = 0;   // spatial dofs
  int32_t* d_el_dofs = nullptr;     // [nd][ne]
  int32_t* d_el_dofs_aos = nullptr; // [ne][nd] element-major (scatter gathers)
  int32_t* d_dof_adj_ptr = nullptr; // [ndof+1]
  int32_t* d_dof_adj = nullptr;     // element*32 + local index, elements ascending
  int max_adj = 0;
  std::vector<int32_t> h_el_dofs;   // ne*nd
};

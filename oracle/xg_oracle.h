/*
 * Oracle for the cut-element hot path: a CPU restatement of ngsxfem's
 * straight-cut quadrature, CutInfo marking, facet marking, cut bilinear-form
 * and facet-patch (ghost-penalty) element matrices and their sparse assembly.
 *
 * THIS IS TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it, and only as the
 * checker or the timed CPU baseline.  The product (ngsxfem_gb300/) never links
 * or calls it.
 *
 * Parity status: the reference (ngsxfem) needs NGSolve, which cannot be built
 * or imported here, so point- and entry-level parity with the real reference
 * is unpinned.  The oracle is pinned against the closed-form known answers the
 * reference's own tests assert (areas, perimeters, monomial moments of planar
 * cuts, space-time planar cuts); see tests/test_oracle_known_answers.py.
 */
#ifndef XG_ORACLE_H
#define XG_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Domain types, same values as ngsxfem utils/ngsxstd.hpp:16-35.  ORC_WHOLE
 * (skeleton terms only): the whole facet, no level-set restriction. */
enum { ORC_NEG = 0, ORC_POS = 1, ORC_IF = 2, ORC_WHOLE = 3 };

/* Term kinds; identical numbering to the product's XG_TERM_*. */
enum {
  ORC_TERM_MASS = 0,       /* c * u * v                          */
  ORC_TERM_LAPLACE = 1,    /* c * grad u . grad v                */
  ORC_TERM_NGRADU_V = 2,   /* c * (n . grad u) * v, n = grad(lset)/|grad(lset)| */
  ORC_TERM_U_NGRADV = 3,   /* c * u * (n . grad v)               */
  ORC_TERM_CONV = 4,       /* c * (b . grad u) * v               */
  ORC_TERM_GHOST_MASS = 5, /* c * (u - u.Other()) * (v - v.Other()) on a facet patch */
  ORC_TERM_DT_U_V = 6,     /* space-time: c * v * d/dtau u (dtref) */
  /* skeleton terms on interior facets F (u / v: element 1 of the facet, u' / v':
   * element 2, n_F: unit normal of F pointing out of element 1), over F in the
   * domain (ORC_NEG / ORC_POS: the cut facet) or the whole facet (ORC_WHOLE) */
  ORC_TERM_SKEL_JUMP = 7,    /* c * (u - u') * (v - v')                               */
  ORC_TERM_SKEL_FLUX = 8,    /* c * ((grad u + grad u') . n_F) * (v - v')             */
  ORC_TERM_SKEL_FLUX_T = 9,  /* c * (u - u') * ((grad v + grad v') . n_F)             */
  ORC_TERM_SKEL_DN1 = 10,    /* c * [d_n u] [d_n v], [d^k_n w] = d^k_n w - d^k_n w'  */
  ORC_TERM_SKEL_DN2 = 11,    /* c * [d^2_n u] [d^2_n v]                              */
  ORC_TERM_SKEL_DN3 = 12,    /* c * [d^3_n u] [d^3_n v]                              */
  ORC_TERM_NGRADU_NGRADV = 13 /* c * (n . grad u) (n . grad v); coefficient terms (orc_cterm) */
};

typedef struct {
  int kind;
  int domain;      /* ORC_NEG / ORC_POS / ORC_IF (ignored for GHOST_MASS) */
  int order;       /* -1: default order (trial+test-difforders; 2*maxorder for patches) */
  int hpow;        /* coefficient multiplied by h^hpow, h = |det F|^(1/D) of the (first) element */
  double coef;
  double b[3];     /* convection field for ORC_TERM_CONV */
  const uint64_t* defined_on; /* element bits (volume terms) or facet bits (patch terms); NULL = all */
} orc_term;

/* --- single-element functions -------------------------------------------- */
int orc_check_if_straight_cut(const double* vals, int n, double eps);
void orc_interpolate_p1_perturb(double* vals, int n, double eps);
/* Base rule of the rule family for element dimension d (1 segment, 2 trig, 3 tet) and order p.
 * Returns number of points; pts has 3 doubles per point. */
int orc_base_rule(int d, int p, double* pts, double* wts, int maxpts);
/* Straight-cut rule on one simplex with physical vertex coords elc[(D+1)*D].
 * Returns number of points, -1 for "no rule" (nullptr), or < -1 on error. */
int orc_straight_cut_rule(int D, const double* elc, const double* lset, int dt, int order,
                          double* pts, double* wts, int maxpts);

/* --- mesh-level functions ------------------------------------------------- */
typedef struct orc_space orc_space;
/* coords: nv*D (AoS), elv: ne*(D+1). order: H1 order 1..3. */
orc_space* orc_space_create(int D, int nv, const double* coords, int ne, const int32_t* elv, int order);
void orc_space_destroy(orc_space*);
int orc_space_info(const orc_space*, int64_t* out /* [ndof, nedges, nfaces, nfacets, ndof_el] */);
int orc_space_el_dofs(const orc_space*, int32_t* out /* ne*ndof_el */);
int orc_space_facet_els(const orc_space*, int32_t* out /* nfacets*2 */);

/* CutInfo.Update: dom[ne] (NEG/POS/IF by volume fractions), cut_ratio[ne],
 * bits[8][nwords] element bitsets per COMBINED_DOMAIN_TYPE (64 elements per word). */
int orc_cutinfo(const orc_space*, const double* lset_vertex, uint8_t* dom, double* cut_ratio,
                uint64_t* bits, int nthreads);
/* BND elements: the boundary facets in facet order, vertices ascending (nbnd x D);
 * returns nbnd.  Either output may be NULL. */
int orc_boundary_elements(const orc_space*, int32_t* facets, int32_t* verts);
/* CutInfo.Update for BND elements: dom, cut_ratio, bits[8][nwords] over the BND elements. */
int orc_cutinfo_bnd(const orc_space*, const double* lset_vertex, uint8_t* dom, double* cut_ratio, uint64_t* bits);
/* CutInfo.Update node part: cut-neighbouring node bitsets (vertices, edges, faces
 * (3D), elements) and node domain types (vertices, edges, faces (3D), cells). */
int orc_cutinfo_nodes(const orc_space*, const uint8_t* dom, const double* cut_ratio, uint64_t* nb_v,
                      uint64_t* nb_e, uint64_t* nb_f, uint64_t* nb_el, uint8_t* dv, uint8_t* de, uint8_t* df,
                      uint8_t* dc);
int orc_facets_with_neighbor_types(const orc_space*, const uint64_t* a, const uint64_t* b,
                                   int bnd_a, int bnd_b, int use_and, uint64_t* out);
double orc_integrate(const orc_space*, const double* lset_vertex, int dt, int order,
                     int ex, int ey, int ez, const uint64_t* defined_on);
/* Integrate of sum_m coef[m] x^e3[3m] y^e3[3m+1] z^e3[3m+2] F0 F1 over the
 * straight cut rule, F0 = f[f0[m]] (d0[m] = -1) or its derivative along
 * x_d0[m], F1 likewise; field i: order f_order[i], element coefficients
 * f_el[i] [ne][nd_i] (at most 8 fields; f = -1: no factor; d0 / d1 NULL:
 * values only). */
double orc_integrate_fields(const orc_space*, const double* lset_vertex, int dt, int order, int nf,
                            const int* f_order, const double* const* f_el, int nm, const double* coef,
                            const int* e3, const int* f0, const int* f1, const int* d0, const int* d1,
                            const uint64_t* defined_on, const double* theta_mesh /* [ne][6][3] or NULL */);

/* Element matrix of the sum of volume terms on element e (row = test, col = trial). */
int orc_element_matrix(const orc_space*, const double* lset_vertex, const orc_term* terms, int nterms,
                       int e, double* elmat);
/* Facet-patch matrix of patch terms on facet f: (2n)^2, dofs [el1, el2]. */
int orc_patch_matrix(const orc_space*, const orc_term* terms, int nterms, int f, double* elmat);
/* Facet matrix of facet f: its patch terms plus its skeleton terms (row = test,
 * col = trial, dofs [el1, el2]).  dn_fd = 0: exact normal derivatives; 1: the
 * reference's central finite differences of DiffOpDuDnk (ghostpenalty.cpp:
 * 221-365, version 2, accuracy 4) for the ORC_TERM_SKEL_DN* terms. */
int orc_facet_matrix(const orc_space*, const double* lset_vertex, const orc_term* terms, int nterms, int f,
                     int dn_fd, double* elmat);
/* Central finite-difference stencil of DiffOpDuDnk for the k-th derivative at
 * accuracy acc: c[0 .. 2w] on the offsets -w .. w (returns w) and the step
 * factor of GetOptimalEps (times the element size h). */
int orc_fd_stencil(int k, int acc, double* c, double* eps);
/* Subdivision cut rules of a higher-order level set (the reference's
 * CutIntegrationRule with subdivlvl, cutint/xintegration.cpp:1626-1754 and
 * NumericalIntegrationStrategy::MakeQuadRule): lset_coefs are the level set's
 * coefficients in the space s (H1 of order 1..3).  orc_subdiv_rule returns the
 * number of points of element e (physical points, 3 per point, and physical
 * weights) or an error; orc_integrate_subdiv integrates x^ex y^ey z^ez over
 * the domain (status: the first rule error, 0 if none). */
int orc_subdiv_rule(const orc_space* s, const double* lset_coefs, int e, int dt, int order, int subdivlvl,
                    double* pts, double* wts, int maxpts);
double orc_integrate_subdiv(const orc_space* s, const double* lset_coefs, int dt, int order, int subdivlvl, int ex,
                            int ey, int ez, const uint64_t* defined_on, int* status);
/* NEG moments (35, monomials of degree <= 4) of n P2 level sets on the
 * reference tetrahedron (values at the vertices and edge midpoints) by the
 * subdivision rule of the given level. */
int orc_subdiv_moments_p2(int64_t n, const double* vals10, int levels, double* out35, int nthreads);
/* Discontinuous (L2) space of order k: the same element basis with element-
 * local dofs, dof(e, i) = e * ndof_el + i. */
orc_space* orc_space_create_l2(int D, int nv, const double* coords, int ne, const int32_t* elv, int order);

typedef struct orc_csr orc_csr;
/* Full assembly: volume terms over their elements, patch terms over their facets,
 * summed into a CSR over all dofs (rows of untouched dofs are empty). */
orc_csr* orc_assemble(const orc_space*, const double* lset_vertex, const orc_term* terms, int nterms,
                      int nthreads);
/* A term on a region of several level sets: the integrand of kind (MASS,
 * LAPLACE, NGRADU_V, U_NGRADV, CONV) over the union of ntup domain tuples
 * dts [ntup][M]; the normal of NGRADU_V / U_NGRADV is grad(l)/|grad(l)| of the
 * P1 level set normal_lset. */
typedef struct {
  int kind, order, hpow, normal_lset;
  double coef;
  double b[3];
  int ntup;
  const int* dts;
  const uint64_t* defined_on; /* element bits; NULL = all */
} orc_mlterm;
/* Assembly of terms on regions of M level sets (lsets [M][nv], vertex values)
 * plus facet-patch terms (GHOST_MASS with their facet sets). */
orc_csr* orc_mlset_assemble(const orc_space* s, int M, const double* lsets, const orc_mlterm* terms, int nterms,
                            const orc_term* patch_terms, int npatch, int nthreads);
/* A boundary term (dCut(lset, domain, vb=BND)): c * u * v over the domain
 * part of the BND elements (the boundary facets in facet order) in its set. */
typedef struct {
  int kind;        /* ORC_TERM_MASS */
  int domain;      /* ORC_NEG / ORC_POS */
  int order, hpow; /* h of the owning element */
  double coef;
  const uint64_t* defined_on; /* BND element bits; NULL = all */
} orc_bterm;
orc_csr* orc_assemble_bnd(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms,
                          const orc_bterm* bterms, int nbterms, int nthreads, int dn_fd);
/* A volume term with a coefficient field: the integrand of kind (MASS,
 * LAPLACE, NGRADU_V, U_NGRADV, CONV, NGRADU_NGRADV) times c h^hpow x^e gf(x),
 * evaluated at the points of the straight cut rule (domain ORC_WHOLE: the
 * element's own rule, cut or not, as dx(definedonelements=...)); gf given
 * per element in the element's basis order ([ne][ndof_el(D, gf_order)]),
 * gf_order 0 = none. */
typedef struct {
  int kind, domain, order, hpow;
  double coef;
  double b[3];
  int e[3];
  int gf_order;
  const double* gf_el;
  const uint64_t* defined_on;
  const double* theta_el; /* [ne][6][3] deformation (orc_iso_theta_mesh) or NULL: the term on the deformed mesh */
} orc_cterm;
/* theta_patch: the mesh deformation per element ([ne][6][3], orc_iso_theta_mesh)
 * for the facet-patch terms (MapPatchIntegrationPoint on the deformed maps),
 * or NULL. */
orc_csr* orc_assemble_full(const orc_space* s, const double* lset_vertex, const orc_term* terms, int nterms,
                           const orc_bterm* bterms, int nbterms, const orc_cterm* cterms, int ncterms,
                           const double* theta_patch, int nthreads, int dn_fd);
/* orc_assemble with the normal-derivative mode of orc_facet_matrix. */
orc_csr* orc_assemble_ex(const orc_space*, const double* lset_vertex, const orc_term* terms, int nterms,
                         int nthreads, int dn_fd);
int64_t orc_csr_nnz(const orc_csr*);
void orc_csr_get(const orc_csr*, int64_t* rowptr, int32_t* cols, double* vals);
void orc_csr_destroy(orc_csr*);

/* --- space-time (P1 space level set x P_kt time, Gauss-Lobatto time nodes) --- */
typedef struct {
  int kind, domain, order, hpow;
  double coef;
  double b[3];
  const uint64_t* defined_on;
  double tref;          /* < 0: over the slab; >= 0: fixed time tau = tref (spatial rule of the trace) */
  double bc[3], bs[3];  /* convection b(t) = b + bc cos(omega t) + bs sin(omega t) */
  double omega, t0, dt; /* t = t0 + dt * tau */
} orc_st_term;
int orc_time_basis(int kt, double tau, double* psi, double* dpsi);
/* lset: (kt+1)*(D+1) time-major; points: 4 doubles (xi, eta, zeta, tau). */
int orc_spacetime_cut_rule(int D, const double* elc, const double* lset, int kt, int dt, int order_space,
                           int order_time, double* pts, double* wts, int maxpts);
/* lset_st: (kt+1)*nv time-major */
int orc_cutinfo_st(const orc_space*, const double* lset_st, int kt, uint8_t* dom, double* ratio, uint64_t* bits,
                   int nthreads);
int orc_st_element_matrix(const orc_space*, const double* lset_st, int kt_l, int kt, int order_time,
                          const orc_st_term* terms, int nterms, int e, double* elmat);
double orc_integrate_st(const orc_space*, const double* lset_st, int kt, int dt, int order_space, int order_time);
/* space-time assembly; dof (it, j) -> it*ndof_space + j */
orc_csr* orc_assemble_st(const orc_space*, const double* lset_st, int kt_l, int kt, int order_time,
                         const orc_st_term* terms, int nterms, int nthreads);

/* --- isoparametric rules for P2 level sets (xg_oracle_iso.cpp) ------------ */
/* P2 nodal values: D+1 vertex values, then the edge midpoints of (0,1),(0,2),(1,2)
 * (trig) / (0,1),(0,2),(0,3),(1,2),(1,3),(2,3) (tet).  The per-element
 * deformation of LevelSetMeshAdaptation (edge coefficients, reference frame,
 * nedges*D doubles); returns 1 if the element was deformed (relevant band). */
int orc_iso_deformation(int D, const double* elc, const double* p2vals, double threshold, double* theta,
                        int* nonconv);
/* Cut rule of the deformed element: points = deformed reference points, weights
 * = physical measure (|det J A|, and |(J A)^-T n| on IF).  deform = 0: the plain
 * straight cut rule of the P1 interpolant with the same weights convention. */
int orc_iso_cut_rule(int D, const double* elc, const double* p2vals, int dt, int order, double threshold,
                     int deform, double* pts, double* wts, int maxpts, int* nonconv);
/* Integral of 1 over the dt part of a whole mesh with the mesh-level
 * deformation (shared edge dofs averaged over the band elements, all elements
 * deformed), as Integrate(levelset_domain, cf=1, order) after
 * mesh.SetDeformation(CalcDeformation(lset_ho)).  p2vals: ne x nnodes per
 * element (element-local node order above). */
/* The mesh-level deformation of orc_iso_integrate_mesh per element: theta_out
 * [ne][6][3] = the averaged edge coefficients in each element's reference
 * frame (edges (0,1),(0,2),(1,2) / the six tet edges, unused rows 0). */
int orc_iso_theta_mesh(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* p2vals,
                       double threshold, double* theta_out, int* nonconv);
double orc_iso_integrate_mesh(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* p2vals,
                              int dt, int order, double threshold, int deform, int* nonconv);
/* NEG-part moments (35, degree <= 4, graded order) of the reference tet for n
 * P2 value sets (10 each); nonconv[i] = non-converged searches (-1: rule error). */
int orc_iso_moments_tet(int64_t n, const double* vals10, int order, int deform, double* out35, int32_t* nonconv,
                        int nthreads);
/* The same moments of the exact NEG part {phi_P2 < 0}, approximated by `levels`
 * red refinements with the straight cut rule of the P1 interpolant on each leaf. */
int orc_subdiv_moments_tet(const double* vals10, int levels, double* out35);

/* --- linear forms ---------------------------------------------------------- */
enum { ORC_LTERM_SOURCE = 0, /* coef * x^e0 y^e1 z^e2 * v */
       ORC_LTERM_SOURCE_GF = 1, /* coef * u_h * v, u_h = gf (dof vector of the same space) */
       ORC_LTERM_SOURCE_BND = 2 /* coef * x^e0 y^e1 z^e2 * v on the domain part of the BND elements (vb=BND);
                                   defined_on: bits over the BND elements */ };
typedef struct {
  int kind, domain, order;  /* order -1: 2k */
  int e[3];
  double coef;
  const double* gf;
  const uint64_t* defined_on;
} orc_lterm;
int orc_linear_form(const orc_space*, const double* lset_vertex, const orc_lterm* terms, int nterms, double* out);

/* Whole CPU pipeline (CutInfo + facet marking + assembly) for timing: returns nnz. */
int64_t orc_pipeline(const orc_space*, const double* lset_vertex, const orc_term* terms, int nterms,
                     int ghost_facets, int nthreads);

/* --- quadrilaterals and hexahedra (xg_oracle_quad.cpp) ------------------------
 * Vertex order of an element: (0,0),(1,0),(1,1),(0,1) [then the same at z = 1];
 * policy: 0 FIRST_ALLOWED, 1 FIND_OPTIMAL, 2 ALWAYS_NONE (utils/ngsxstd.hpp:10).
 * Returns the point count, -1 for "no rule", or -(status) - 1 on an error
 * (status as xg_status: 3 capacity, 4 plain cut, 5 decomposition, 7 NaN bound,
 * 9 interface scaling bound). */
int orc_quad_cut_rule(int D, const double* lset_vals, int dt, int order, int policy, double* pts, double* wts,
                      int maxpts);
/* The same rule with the interface weights of the bilinear / trilinear element
 * with vertices xv[nv][3] (StraightCutIntegrationRule; an empty cut rule is
 * "no rule", -1). */
int orc_quad_straight_cut_rule(int D, const double* xv, const double* lset_vals, int dt, int order, int policy,
                               double* pts, double* wts, int maxpts);
/* CutInfo.Update on a quad / hex mesh: dom, ratio, bits[8][ceil(ne/64)] as orc_cutinfo. */
int orc_quad_cutinfo(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* lset, int policy,
                     uint8_t* dom, double* ratio, uint64_t* bits);
/* Bilinear form on a quad / hex mesh with the Q1 space (dofs = vertices):
 * SymbolicCutBFI on ET_QUAD / ET_HEX (xfem/symboliccutbfi.cpp:76-486), the
 * rule of StraightCutIntegrationRule for quads (straightcutrule.cpp:582-677),
 * terms of kind MASS, LAPLACE, NGRADU_V, U_NGRADV (normal: the pointwise
 * unit gradient of the multilinear level set), CONV; default order 2 (trial +
 * test order, no derivative reduction on quads); h = |det J|^(1/D) at the
 * point.  An element is active for a term if it is in the term's set and its
 * domain type is the term's domain or IF.  CSR over all nv dofs. */
orc_csr* orc_quad_assemble(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* lset,
                           const orc_term* terms, int nterms, int policy, int nthreads, int* status);
/* CSR from element matrices alone (el_slot[e] < 0: inactive), per dof its
 * elements ascending. */
orc_csr* orc_csr_from_elements(int64_t ndof, int n, int ne, const int32_t* el_dofs, const int32_t* el_slot,
                               const double* elm, int64_t nslots, int nthreads);
/* Integrate(x^ex y^ey z^ez * dCut) on a quad / hex mesh: coords[nv][D], elv[ne][2^D]. */
double orc_quad_integrate(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* lset,
                          int dt, int order, int policy, int ex, int ey, int ez, int* status);
/* The same on nthreads host threads (contiguous element ranges, partial sums
 * added in range order). */
double orc_quad_integrate_mt(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* lset,
                             int dt, int order, int policy, int ex, int ey, int ez, int nthreads, int* status);

/* --- several level sets on simplices (xg_oracle_mlset.cpp) --------------------
 * lsets: M level sets' values, [M][D+1] at the element's vertices (rule) or
 * [M][nv] at the mesh vertices (Integrate); dts: ntup domain tuples of M
 * entries (NEG / POS / IF), their rules concatenated
 * (CreateMultiLevelsetCutIntegrationRule).  The rule returns the point count,
 * -1 for no rule or -(status)-1. */
int orc_mlset_cut_rule(int D, const double* elc, int M, const double* lsets, int ntup, const int* dts, int order,
                       double* pts, double* wts, int maxpts);
double orc_mlset_integrate(int D, int nv, const double* coords, int ne, const int32_t* elv, int M,
                           const double* lsets, int ntup, const int* dts, int order, int ex, int ey, int ez,
                           int* status);
/* MultiLevelsetCutInfo element markers: mode 0 GetElementsOfType (exact level-set
 * domain types), 1 GetElementsWithContribution (positive weight sum of the
 * region's order-0 rule).  Returns 0 or the first error status. */
int orc_mlset_mark(int D, int nv, const double* coords, int ne, const int32_t* elv, int M, const double* lsets,
                   int ntup, const int* dts, int mode, uint64_t* bits);
/* Integrate(x^ex y^ey z^ez * dCut(lset, dt, vb=BND)) over the boundary elements of
 * a simplex mesh (elements' facets that belong to one element); IF on 2D
 * boundary segments is the point measure (each intersection point counts 1). */
double orc_integrate_bnd(int D, int nv, const double* coords, int ne, const int32_t* elv, const double* lset, int dt,
                         int order, int ex, int ey, int ez, const uint8_t* defined_on, int* status);
/* The rule of one boundary element (xv[D][3], l[D]): physical points xs (3 per
 * point), weights ws = w * measure; the number of points, -1 above cap, or
 * -(error code). */
int orc_bnd_element_rule(int D, const double* xv, const double* l, int dt, int order, double* xs, double* ws, int cap);
/* The share of one boundary element (vertices xv[D][3], values l[D]). */
double orc_bnd_element_integral(int D, const double* xv, const double* l, int dt, int order, int ex, int ey, int ez,
                                int* status);

#ifdef __cplusplus
}
#endif
#endif

/*
 * xg.h -- C ABI of libxg, the GB300 (sm_103a) cut-element assembly library.
 *
 * The library replaces ngsxfem's cut-element hot path:
 *   CutInfo element marking        -> xg_cutinfo_update
 *   GetFacetsWithNeighborTypes     -> xg_facets_with_neighbor_types
 *   StraightCutIntegrationRule     -> xg_cut_rules
 *   SymbolicCutBFI / SymbolicFacetPatchBFI element matrices + the sparse
 *   scatter of BilinearForm::Assemble -> xg_form_assemble
 *   Integrate(cf * dCut(...))      -> xg_integrate
 *
 * Conventions
 *  - Plain pointers and sizes only.  Arguments named d_* are device pointers,
 *    h_* host pointers.  `stream` is a cudaStream_t passed as void* (NULL = the
 *    legacy default stream).
 *  - Every entry point returns an xg_status; none throws across the ABI.
 *    xg_status_string() names a status; xg_last_error() gives the last message
 *    of the calling thread.
 *  - The caller owns every buffer it passes in (level-set values, bitsets,
 *    CSR output).  Objects (xg_mesh, xg_space, xg_form) own their device
 *    workspace; calls on different objects may run concurrently from
 *    different threads, calls on one object must be serialised.
 *  - Launch entry points enqueue work on `stream` and return without a host
 *    synchronisation, so a whole assembly step can be captured in a CUDA graph.
 *    Device-side failures (bad decomposition, capacity overflow, non-finite
 *    weights) are recorded in the object's device error word and read by
 *    xg_*_check() after the stream has been synchronised.
 *  - Bitsets: bit i of element/facet i lives in 64-bit word i/64, bit i%64.
 *
 * Domain types and combined domain types use ngsxfem's values
 * (utils/ngsxstd.hpp:16-35).
 */
#ifndef XG_H
#define XG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  XG_OK = 0,
  XG_ERR_ARG = 1,          /* invalid argument */
  XG_ERR_CUDA = 2,         /* CUDA runtime error (message in xg_last_error) */
  XG_ERR_CAPACITY = 3,     /* an output or workspace capacity was too small */
  XG_ERR_PLAIN_CUT = 4,    /* cut of an uncut sub-simplex: straightcutrule.cpp:43-48 */
  XG_ERR_BAD_DECOMP = 5,   /* unsupported cut topology: straightcutrule.cpp:148,193 */
  XG_ERR_UNSUPPORTED = 6,  /* element type / order / term not supported */
  XG_ERR_NONFINITE = 7,    /* a non-finite weight or matrix entry was produced */
  XG_ERR_NO_DEVICE = 8,    /* no CUDA device, or the library was not built for it */
  XG_ERR_IF_BOUND = 9,     /* quad / hex interface scaling above 1/sqrt(1-0.999^2):
                              straightcutrule.cpp:273-286 */
  XG_ERR_TIMEOUT = 10      /* a bounded device-side wait gave up (the kernel stopped its work) */
} xg_status;

enum { XG_NEG = 0, XG_POS = 1, XG_IF = 2, XG_WHOLE = 3 /* skeleton terms: the whole facet */ };
enum {
  XG_CDOM_NO = 0, XG_CDOM_NEG = 1, XG_CDOM_POS = 2, XG_CDOM_UNCUT = 3,
  XG_CDOM_IF = 4, XG_CDOM_HASNEG = 5, XG_CDOM_HASPOS = 6, XG_CDOM_ANY = 7
};

/* Integrand menu of the bilinear-form terms (the CoefficientFunction trees the
 * reference interprets, symboliccutbfi.cpp:168-194, reduced to the products
 * the cut forms use).  u = trial, v = test, n = grad(lset)/|grad(lset)| of the
 * P1 level set, b = constant vector, u' / v' = the neighbour's polynomial
 * extended over the facet patch (u.Other()). */
typedef enum {
  XG_TERM_MASS = 0,       /* c * u * v                      */
  XG_TERM_LAPLACE = 1,    /* c * grad u . grad v            */
  XG_TERM_NGRADU_V = 2,   /* c * (n . grad u) * v           */
  XG_TERM_U_NGRADV = 3,   /* c * u * (n . grad v)           */
  XG_TERM_CONV = 4,       /* c * (b . grad u) * v           */
  XG_TERM_GHOST_MASS = 5, /* c * (u - u') * (v - v') on a facet patch (dFacetPatch) */
  XG_TERM_DT_U_V = 6,     /* space-time: c * v * d/dtau u (dtref), space-time forms only */
  /* Skeleton terms on interior facets F (SymbolicCutFacetBilinearFormIntegrator,
   * symboliccutbfi.cpp:886-1572, for domain XG_NEG / XG_POS: F cut to the
   * domain by the P1 level set; SymbolicFacetBilinearFormIntegrator2,
   * :1574-1735, for XG_WHOLE: all of F).  u / v live on the facet's first
   * element, u' / v' on the second, n_F is the unit normal of F out of the
   * first element; d_defined_on holds facet bits.  Integrated exactly with the
   * reference's facet rule order 2 * order of the space (the term's order is
   * not used).  XG_IF (codim-2 skeleton rules) is not supported. */
  XG_TERM_SKEL_JUMP = 7,   /* c * (u - u') * (v - v')                                   */
  XG_TERM_SKEL_FLUX = 8,   /* c * ((grad u + grad u') . n_F) * (v - v')                 */
  XG_TERM_SKEL_FLUX_T = 9, /* c * (u - u') * ((grad v + grad v') . n_F)                 */
  XG_TERM_SKEL_DN1 = 10,   /* c * [d_n u][d_n v], [d^k_n w] = d^k_nF w - d^k_nF w'; the
                              reference's dn(w, k) - (-1)^k dn(w.Other(), k)
                              (DiffOpDuDnk, ghostpenalty.cpp:221-365, python_xfem.cpp:1068) */
  XG_TERM_SKEL_DN2 = 11,   /* c * [d^2_n u][d^2_n v] */
  XG_TERM_SKEL_DN3 = 12,   /* c * [d^3_n u][d^3_n v] */
  XG_TERM_NGRADU_NGRADV = 13 /* c * (n . grad u) * (n . grad v): the normal-diffusion term of
                                TraceFEM; coefficient terms (xg_cterm) only */
} xg_term_kind;

typedef enum { XG_PREC_FP64 = 0, XG_PREC_MIXED = 1 } xg_precision;

/* One integrator: SymbolicBFI(cf * dCut(lset, domain, order, definedonelements))
 * or cf * dFacetPatch(definedonelements).  c = coef * h^hpow with
 * h = |det F|^(1/dim) of the element (of the first element of a patch). */
typedef struct {
  int32_t kind;              /* xg_term_kind */
  int32_t domain;            /* XG_NEG / XG_POS / XG_IF (ignored for patches) */
  int32_t order;             /* -1: ngsxfem's default, symboliccutbfi.cpp:100-111 */
  int32_t hpow;
  double coef;
  double b[3];               /* XG_TERM_CONV only */
  const uint64_t* d_defined_on; /* element bits (volume) / facet bits (patch); NULL = all */
} xg_term;

typedef struct xg_mesh xg_mesh;
typedef struct xg_space xg_space;
typedef struct xg_form xg_form;

/* ---- status ------------------------------------------------------------- */
const char* xg_status_string(int status);
const char* xg_last_error(void);
/* Device count visible to the library and whether it carries sm_103a code. */
int xg_device_ok(int* ok);

/* ---- mesh (ngcomp::MeshAccess stand-in) ---------------------------------- */
/* (xg_cutinfo_update also accepts quadrilateral / hexahedral meshes,
 * xg_mesh_create_tensor: element part only, from the order-0 cut rules of
 * LevelsetCutQuadrilateral with the FIND_OPTIMAL policy.) */
/* Builds edges, faces and the facet->element table on the host and uploads
 * coordinates (SoA) and topology to the current device.
 * h_coords: nv*dim (AoS), h_elv: ne*(dim+1).  dim 2 (trig) or 3 (tet). */
int xg_mesh_create(int dim, int32_t nv, const double* h_coords, int32_t ne, const int32_t* h_elv,
                   xg_mesh** out);
/* Quadrilateral (dim 2) or hexahedral (dim 3) mesh: h_elv ne*2^dim with the
 * corner order (0,0),(1,0),(1,1),(0,1) [then the same at z = 1]
 * (cutint/straightcutrule.hpp:76-90); the element map is the bilinear /
 * trilinear interpolation of the corners.  Such a mesh serves xg_cut_rules(_ex)
 * and xg_integrate(_ex); entry points that need facet topology or H1 spaces
 * return XG_ERR_UNSUPPORTED for it. */
int xg_mesh_create_tensor(int dim, int32_t nv, const double* h_coords, int32_t ne, const int32_t* h_elv,
                          xg_mesh** out);
int xg_mesh_destroy(xg_mesh* mesh);
/* out: [dim, nv, ne, nedges, nfaces, nfacets] */
int xg_mesh_info(const xg_mesh* mesh, int64_t* h_out6);
/* Host copies of the facet->element table (nfacets*2, -1 = boundary). */
int xg_mesh_facet_elements(const xg_mesh* mesh, int32_t* h_out);

/* ---- H1 space (ngcomp::H1HighOrderFESpace stand-in) ---------------------- */
/* Dof numbering: vertices, then (order-1) dofs per edge (edges sorted by
 * vertex pair), then for order 3 one bubble per face (3D) / cell (2D). */
int xg_space_create(xg_mesh* mesh, int order, xg_space** out);
/* Discontinuous space (L2(mesh, order, dgjumps=True) of the reference's
 * discontinuous-Galerkin forms): the element basis of xg_space_create with
 * element-local dofs, dof(e, i) = e * ndof_per_element + i. */
int xg_space_create_l2(xg_mesh* mesh, int order, xg_space** out);
int xg_space_destroy(xg_space* space);
/* out: [ndof, ndof_per_element, order] */
int xg_space_info(const xg_space* space, int64_t* h_out3);
int xg_space_element_dofs(const xg_space* space, int32_t* h_out /* ne*ndof_el */);

/* ---- level set preparation ----------------------------------------------- */
/* InterpolateToP1's vertex perturbation, utils/p1interpol.cpp:104-107:
 * |v| < eps -> v = eps. */
int xg_interpolate_p1_perturb(double* d_vals, int64_t n, double eps, void* stream);

/* ---- marking -------------------------------------------------------------- */
/* CutInformation::Update (xfem/cutinfo.cpp:61-132): per element the NEG/POS
 * volume fractions of the order-0 cut rules give cut_ratio = NEG/(NEG+POS)
 * and the domain type; d_bits receives the 8 COMBINED_DOMAIN_TYPE bitsets
 * ([8][ceil(ne/64)] words, row c = XG_CDOM value c).
 * Replaces CutInformation::Update(cf, subdivlvl=0, time_order=-1, lh).
 * The marking uses a list of cut elements owned by the mesh: calls of
 * xg_cutinfo_update, xg_cutinfo_update_bnd and xg_cutinfo_update_st on one mesh
 * must not overlap (the forms' steps use their own lists and may). */
int xg_cutinfo_update(xg_mesh* mesh, const double* d_lset, uint8_t* d_dom, double* d_cut_ratio,
                      uint64_t* d_bits, void* stream);
/* CutInformation::Update for the BND elements (xfem/cutinfo.cpp:83-131 with
 * vb == BND): the mesh's boundary facets in facet order (xg_mesh_boundary),
 * each an (dim-1)-simplex with its vertices in ascending order; outputs as
 * xg_cutinfo_update over the nbnd BND elements. */
int xg_cutinfo_update_bnd(xg_mesh* mesh, const double* d_lset, uint8_t* d_dom, double* d_cut_ratio,
                          uint64_t* d_bits, void* stream);
/* BND elements: their number and (h_facets, optional) their facet numbers. */
int xg_mesh_boundary(const xg_mesh* mesh, int64_t* h_nbnd, int32_t* h_facets);
/* CutInformation::Update, node part (xfem/cutinfo.cpp:134-224), from the VOL
 * domain types and cut ratios of xg_cutinfo_update: cut-neighbouring bitsets of
 * vertices, edges, faces (3D; NULL in 2D) and elements, and the domain type of
 * every vertex, edge, face (3D) and cell (XG_NEG if the node belongs to a NEG
 * element, else XG_POS; cells: cut ratio > 0.5). */
int xg_cutinfo_nodes(xg_mesh* mesh, const uint8_t* d_dom, const double* d_cut_ratio, uint64_t* d_nb_vertices,
                     uint64_t* d_nb_edges, uint64_t* d_nb_faces, uint64_t* d_nb_elements, uint8_t* d_dom_vertices,
                     uint8_t* d_dom_edges, uint8_t* d_dom_faces, uint8_t* d_dom_cells, void* stream);
/* GetElementsWithThresholdContribution (xfem/cutinfo.cpp:263-284): bit e set if
 * ratio[e] >= threshold (dt = XG_NEG) or ratio[e] <= 1 - threshold (XG_POS). */
int xg_elements_with_threshold(const double* d_cut_ratio, int64_t n, int dt, double threshold, uint64_t* d_out,
                               void* stream);
/* Device error word of the mesh (decomposition failures during marking or
 * rule export); synchronise the stream first. Resets the word. */
int xg_mesh_check(xg_mesh* mesh);
/* GetFacetsWithNeighborTypes (xfem/cutinfo.cpp:476-538). */
int xg_facets_with_neighbor_types(xg_mesh* mesh, const uint64_t* d_a, const uint64_t* d_b, int bnd_val_a,
                                  int bnd_val_b, int use_and, uint64_t* d_out, void* stream);
/* GetElementsWithNeighborFacets (xfem/cutinfo.cpp:540-566). */
int xg_elements_with_neighbor_facets(xg_mesh* mesh, const uint64_t* d_facets, uint64_t* d_out, void* stream);

/* ---- quadrature ------------------------------------------------------------ */
/* StraightCutIntegrationRule (cutint/straightcutrule.cpp:582-677) for the n
 * elements in d_elems: element i writes d_counts[i] points (-1 = no rule, the
 * reference's nullptr) into d_pts[(i*max_pts + q)*3 + c] (reference
 * coordinates) and d_wts[i*max_pts + q] (interface weights already carry
 * |F^-T n_ref|, to be multiplied by |det F|). */
int xg_cut_rules(xg_mesh* mesh, const double* d_lset, const int32_t* d_elems, int32_t n, int dt, int order,
                 int32_t max_pts, int32_t* d_counts, double* d_pts, double* d_wts, void* stream);
/* Direction policy of the quadrilateral / hexahedral rules
 * (SWAP_DIMENSIONS_POLICY, utils/ngsxstd.hpp:10; Python FIRST / OPTIMAL /
 * FALLBACK).  xg_cut_rules and xg_integrate use FIND_OPTIMAL, the reference's
 * default (cutint/lsetintdomain.hpp:21); simplex meshes ignore it. */
enum { XG_QUAD_FIRST_ALLOWED = 0, XG_QUAD_FIND_OPTIMAL = 1, XG_QUAD_ALWAYS_NONE = 2 };
/* xg_cut_rules with the direction policy: LevelsetCutQuadrilateral
 * (cutint/straightcutrule.cpp:206-501) on quadrilateral / hexahedral meshes. */
int xg_cut_rules_ex(xg_mesh* mesh, const double* d_lset, const int32_t* d_elems, int32_t n, int dt, int order,
                    int quad_dir_policy, int32_t max_pts, int32_t* d_counts, double* d_pts, double* d_wts,
                    void* stream);
/* Most points a quadrilateral (dim 2) / hexahedral (dim 3) rule of (dt, order)
 * can have (a sufficient max_pts), or -1 for bad arguments. */
int xg_quad_rule_capacity(int dim, int dt, int order);
/* Number of points of the rule family for (element dim d, order p). */
int xg_base_rule_size(int d, int p);
/* Host copy of that rule (NGSolve's SelectIntegrationRule(ET, p) stand-in):
 * h_pts[3*q + c], h_wts[q]; returns the point count or -1 if max_pts is too small. */
int xg_base_rule(int d, int p, double* h_pts, double* h_wts, int max_pts);

/* Integrate(x^ex y^ey z^ez * dCut(lset, dt, order)) over the elements in
 * d_defined_on (NULL = all): cutint/cutintegral.cpp:126-212.  The sum is
 * formed in a fixed order (deterministic) and written to d_result[0]. */
int xg_integrate(xg_mesh* mesh, const double* d_lset, int dt, int order, int ex, int ey, int ez,
                 const uint64_t* d_defined_on, double* d_result, void* stream);

/* One product of an xg_integrate_fields integrand:
 * coef * x^e[0] y^e[1] z^e[2] * F0 * F1 with F0 = field[f0] (d0 = -1) or its
 * derivative along x_d0 (d0 = 0..dim-1), F1 likewise (f0, f1 = -1: no factor). */
typedef struct {
  double coef;
  int32_t e[3];
  int32_t f0, f1;
  int32_t d0, d1;
} xg_fmono;
/* Integrate(cf * dCut(lset, dt, order)) with cf a sum of nmonos (<= 16)
 * xg_fmono products over nfields (<= 4) GridFunctions: spaces[i] (host array)
 * a spatial H1 or L2 space of order 1..3 on `mesh`, d_fields[i] (host array
 * of device pointers) its coefficient vector.  The reference's Integrate with
 * a CoefficientFunction of GridFunctions evaluated at the points of the
 * straight cut rule (cutint/cutintegral.cpp:126-212), e.g. the L2 and H1
 * errors (gfu - gfex)^2, (grad gfu - grad gfex)^2 of its demos.  Simplex meshes.  Deterministic fixed-order
 * sum into d_result[0]; shares the mesh's scratch with xg_integrate (calls on
 * one mesh are serialised on one stream).  d_deform (xg_iso_deformation's
 * [nedges][3], or NULL): on the deformed mesh, the straight cut rule of the P1
 * level set mapped by xhat + Theta(xhat) as in xg_cterm.d_deform. */
int xg_integrate_fields(xg_mesh* mesh, const double* d_lset, int dt, int order, int32_t nfields,
                        xg_space* const* spaces, const double* const* d_fields, int32_t nmonos,
                        const xg_fmono* monos, const uint64_t* d_defined_on, const double* d_deform,
                        double* d_result, void* stream);

/* Several level sets on a simplex mesh (cutint/mlsetintegration.cpp:6-180,
 * cutint/straightcutrule.cpp:679-812): d_lsets holds nlsets (1..8) P1 level
 * sets, [nlsets][nv] vertex values; the domain is the union of ndomains
 * (1..256) tuples h_domains[ndomains][nlsets] (host, XG_NEG / XG_POS / XG_IF;
 * a tuple with k IF entries is a codimension-k set).  Integrate of
 * x^ex y^ey z^ez over that domain, deterministic fixed-order sum. */
int xg_integrate_mlset(xg_mesh* mesh, const double* d_lsets, int32_t nlsets, const int8_t* h_domains,
                       int32_t ndomains, int order, int ex, int ey, int ez, const uint64_t* d_defined_on,
                       double* d_result, void* stream);
/* The per-element rules of such a domain for listed elements (the tuples'
 * parts concatenated; counts -1 = no rule), as xg_cut_rules. */
int xg_cut_rules_mlset(xg_mesh* mesh, const double* d_lsets, int32_t nlsets, const int8_t* h_domains,
                       int32_t ndomains, const int32_t* d_elems, int32_t n, int order, int32_t max_pts,
                       int32_t* d_counts, double* d_pts, double* d_wts, void* stream);
/* MultiLevelsetCutInfo element markers (xfem/cutinfo.cpp:306-419) into d_bits
 * (ceil(ne/64) words): mode 0 = GetElementsOfType (the level sets' domain types
 * on the element equal one of the tuples), 1 = GetElementsWithContribution
 * (the region's order-0 rule on the element has a positive weight sum). */
int xg_mlset_mark(xg_mesh* mesh, const double* d_lsets, int32_t nlsets, const int8_t* h_domains, int32_t ndomains,
                  int mode, uint64_t* d_bits, void* stream);
/* Integrate(x^ex y^ey z^ez * dCut(lset, dt, vb=BND)) over the boundary
 * elements of a simplex mesh (the boundary facets; cutint/straightcutrule.cpp:
 * 582-677): NEG / POS parts of the boundary, and for dt = XG_IF in 2D the
 * intersection points of the interface with the boundary, each counting 1
 * (the point measure of :641-651).  XG_IF in 3D: XG_ERR_UNSUPPORTED.
 * d_defined_on (optional): bitset over the BND elements (xg_mesh_boundary
 * order), the definedon / definedonelements restriction of dCut. */
int xg_integrate_bnd(xg_mesh* mesh, const double* d_lset, int dt, int order, int ex, int ey, int ez,
                     const uint64_t* d_defined_on, double* d_result, void* stream);
/* A sufficient max_pts for xg_cut_rules_mlset, or -1 for bad arguments. */
int xg_mlset_rule_capacity(int dim, int32_t nlsets, int32_t ndomains, int order);
/* Mesh-level isoparametric integration of a P2 level set (LevelSetMeshAdaptation
 * + Integrate: python/lsetcurv.py:281-356, lsetcurving/projshift.cpp:58-197,
 * shiftintegrators.cpp:38-122, calcpointshift.cpp:143-201) on a simplex mesh:
 * d_p2vals [ne][(D+1)(D+2)/2] the level set's values at each element's
 * vertices, then edge midpoints (edges (0,1),(0,2),(1,2) / (0,1),(0,2),(0,3),
 * (1,2),(1,3),(2,3)).  deform = 0 integrates the straight cut of the P1
 * interpolant.  threshold < 0: no clipping of the shifts.  d_result[0] =
 * integral of x^ex y^ey z^ez over the domain dt of the deformed mesh;
 * d_nonconv[0] = Newton searches that did not converge. */
/* The deformation of xg_iso_integrate_mesh alone: d_gdef[edge][3] (edges in
 * the mesh's edge numbering) = the physical edge coefficients J theta of the
 * P2 shift, averaged over the band elements sharing the edge; 0 off the
 * band.  For bilinear forms on the deformed mesh (xg_cterm.d_deform).  It
 * uses the mesh's isoparametric workspace, as xg_iso_integrate_mesh does:
 * those calls on one mesh must not overlap on the GPU. */
int xg_iso_deformation(xg_mesh* mesh, const double* d_p2vals, double threshold, double* d_gdef, int32_t* d_nonconv,
                       void* stream);
int xg_iso_integrate_mesh(xg_mesh* mesh, const double* d_p2vals, int dt, int order, double threshold, int deform,
                          int ex, int ey, int ez, double* d_result, int32_t* d_nonconv, void* stream);
/* xg_integrate with the quadrilateral / hexahedral direction policy. */
int xg_integrate_ex(xg_mesh* mesh, const double* d_lset, int dt, int order, int quad_dir_policy, int ex, int ey,
                    int ez, const uint64_t* d_defined_on, double* d_result, void* stream);
/* Allocation-free variant of xg_integrate (no counterpart in the reference).
 * For callers that cannot allocate device memory when they integrate:
 * real-time loops that forbid allocator calls (a cudaMalloc can synchronise
 * the device and take milliseconds), and host applications whose device
 * memory belongs to their own allocator or budget.  Simplex meshes only
 * (quadrilateral / hexahedral meshes get XG_ERR_UNSUPPORTED; xg_integrate
 * takes them).  It calls no cudaMalloc/cudaFree; its per-block partial sums live
 * in a static 128 KiB device array that every GPU loading the library keeps
 * until exit, which limits it to meshes of at most 16384*4096 = 67,108,864
 * elements (larger meshes get XG_ERR_CAPACITY and a message).  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current; make that first call before any stream capture.  All
 * calls share the array: calls that overlap on the GPU (different streams,
 * concurrent graphs) race and must be serialised by the caller.  The result
 * equals xg_integrate's up to the summation order (a fixed order per mesh). */
int xg_integrate_noalloc(xg_mesh* mesh, const double* d_lset, int dt, int order, int ex, int ey, int ez,
                         const uint64_t* d_defined_on, double* d_result, void* stream);

/* Integrate(x^ex y^ey z^ez * dCut(lset_h, dt, order, subdivlvl)) for a level
 * set of order 1..3 given by its coefficients d_lset_coefs in the H1 space
 * `space` (the reference's CutIntegrationRule for level sets that are not P1,
 * cutint/xintegration.cpp:102-116, 1626-1754): each element's simplex is
 * checked on a lattice of spacing 2^-subdivlvl, cut simplices are refined by
 * the reference's children down to level 0, and cut level-0 simplices get
 * the straight cut of their vertex values.  subdivlvl 0..6. */
int xg_integrate_subdiv(xg_space* space, const double* d_lset_coefs, int dt, int order, int subdivlvl, int ex,
                        int ey, int ez, const uint64_t* d_defined_on, double* d_result, void* stream);
/* The same rule on n reference tetrahedra with a P2 level set given by its
 * values at the vertices (1,0,0),(0,1,0),(0,0,1),(0,0,0) and the midpoints
 * of the edges (0,1),(0,2),(0,3),(1,2),(1,3),(2,3) (d_vals10: n x 10): the 35
 * NEG moments x^a y^b z^c, a + b + c <= 4 (by degree, then a, then b
 * descending) per element, order-4 rules (d_out35: n x 35).  Rule errors go
 * to d_err (may be NULL).  The trees are built level by level with
 * stream-ordered scratch (cudaMallocAsync): the call synchronises the stream
 * once per tree level to size the next level's lists, so it cannot be
 * captured into a CUDA graph. */
int xg_subdiv_moments_tet(const double* d_vals10, int64_t n, int subdivlvl, double* d_out35, int* d_err,
                          void* stream);

/* ---- bilinear forms ---------------------------------------------------------- */
/* A form is a list of integrators over one space (H1 or L2; trial = test
 * space).  Volume terms run on their element sets with the cut rule of their
 * domain; patch and skeleton terms run on their facet sets (the facet's
 * matrix is the sum of both kinds).  Creation uploads the term table and
 * sizes the workspace for the whole mesh (no allocation during assembly).
 * In xg_cutfem_step the skeleton terms run on the facets between two HASNEG
 * (XG_NEG) or two HASPOS (XG_POS) elements and on the ghost facets
 * (XG_WHOLE), as in demos/fictdom_dg.py.  Space-time forms take no skeleton
 * terms. */
int xg_form_create(xg_space* space, const xg_term* terms, int32_t nterms, int precision, xg_form** out);
int xg_form_destroy(xg_form* form);
/* Replace the element/facet set of term t (device bitset, NULL = all). */
int xg_form_set_defined_on(xg_form* form, int32_t t, const uint64_t* d_defined_on);

/* Boundary terms (dCut(lset, dt, vb=BND) in a BilinearForm): c * h^hpow * u * v
 * over the domain part (XG_NEG / XG_POS; XG_IF in 2D: the cut points) of the
 * BND elements in d_defined_on (bits over the BND elements, which are the
 * boundary facets in facet order; NULL = all), with the straight cut of the
 * P1 level set on the boundary facet and h of the owning element.  The
 * reference's SymbolicCutBFI on boundary elements
 * (xfem/symboliccutbfi.cpp:76-486 with vb == BND, the rule of
 * cutint/straightcutrule.cpp:582-677).  The owner of a BND element in a
 * term's set whose domain type (CheckIfStraightCut of its vertex values) is
 * the term's domain or IF joins the active elements; its matrix is the sum
 * of its volume and boundary terms.  Spatial forms on simplex meshes; order
 * -1 = 2k. */
typedef struct {
  int32_t kind;   /* XG_TERM_MASS */
  int32_t domain; /* XG_NEG, XG_POS, XG_IF (2D) */
  int32_t order;
  int32_t hpow;
  double coef;
  const uint64_t* d_defined_on;
} xg_bterm;
/* Replace the form's boundary terms (at most 8; nterms 0 removes them). */
int xg_form_set_bnd_terms(xg_form* form, const xg_bterm* terms, int32_t nterms);

/* Volume terms with a coefficient field (`gf * u * v * dCut(...)`,
 * `gf * grad(u) * grad(v) * dCut(...)`, x^e factors): the integrand of kind
 * XG_TERM_MASS, _LAPLACE, _NGRADU_V, _U_NGRADV, _CONV or _NGRADU_NGRADV times
 * c * h^hpow * x^e0 y^e1 z^e2 * gf(x), evaluated at the points of the
 * domain's cut rule (the reference evaluates any CoefficientFunction at the
 * rule's points, xfem/symboliccutbfi.cpp:168-194; default order: the
 * kind's, trial + test order minus the derivatives, :107-111).  gf is a
 * GridFunction of an H1 space of order 1..3 on the form's mesh (gf_space,
 * d_gf its coefficients) or absent (gf_space NULL).  The elements of the
 * term's set whose domain type is the term's domain or IF join the active
 * elements; their matrices are the sums of all their terms.  Domain XG_WHOLE
 * (`dx(definedonelements=...)`, e.g. TraceFEM's normal diffusion): the
 * element's own rule on every element of the set, cut or not.  Spatial forms
 * on simplex meshes. */
typedef struct {
  int32_t kind;
  int32_t domain; /* XG_NEG, XG_POS, XG_IF, XG_WHOLE */
  int32_t order;  /* -1: the kind's default */
  int32_t hpow;
  double coef;
  double b[3];    /* convection vector (XG_TERM_CONV) */
  int32_t e[3];   /* exponents of the monomial factor */
  const xg_space* gf_space;
  const double* d_gf;
  const uint64_t* d_defined_on;
  /* the mesh deformation (xg_iso_deformation: [nedges][3] physical edge
   * coefficients of the P2 shift) or NULL: with it the term is integrated on
   * the deformed mesh (dCut(..., deformation=...)): the straight cut rule of
   * the P1 level set on the reference element mapped by xhat + Theta(xhat),
   * weights times |det(J A)| (IF: times |(J A)^-T n_ref|), gradients by
   * (J A)^-T, h = |det(J A)|^(1/D) at the point, x the deformed point. */
  const double* d_deform;
} xg_cterm;
/* Replace the form's coefficient terms (at most 8; nterms 0 removes them). */
int xg_form_set_coef_terms(xg_form* form, const xg_cterm* terms, int32_t nterms);
/* The form's facet-patch terms on the deformed mesh (dFacetPatch(...,
 * deformation=...); d_gdef from xg_iso_deformation, NULL = undeformed):
 * SymbolicFacetPatchBFI::T_CalcFacetMatrix with MapPatchIntegrationPoint on
 * the deformed maps (xfem/symboliccutbfi.cpp:1747-1846, 1982-2377): each
 * element's rule of the term's order, every point sent into the other
 * element by the vertex-based guess and Newton steps with the deformed
 * Jacobian, weights |det (J A)| of the point's own element. */
int xg_form_set_deformation(xg_form* form, const double* d_gdef);

/* Output matrix in compressed-row form over the form's active dofs (the dofs
 * of elements and facet patches that carry a term, numbered ascending as
 * ngcomp::CompressedFESpace / Restrict() does):
 *   d_row_dof[r]  global dof of row r (= of column index r)
 *   d_rowptr[r]   start of row r, r = 0..nrows
 *   d_cols[k]     compressed column index, ascending within a row
 *   d_vals[k]     value (FP64)
 *   d_counts[0]   nrows, d_counts[1] nnz (device, written by the step)
 * Capacities are the caller's allocation sizes; xg_form_capacity() gives
 * sufficient ones. */
typedef struct {
  int32_t* d_row_dof;
  int64_t* d_rowptr;
  int32_t* d_cols;
  double* d_vals;
  int64_t* d_counts;
  int64_t cap_rows;
  int64_t cap_nnz;
} xg_csr;

/* Bilinear forms of the Q1 space (dofs = the mesh's vertices) on a
 * quadrilateral / hexahedral mesh (xg_mesh_create_tensor): SymbolicCutBFI on
 * ET_QUAD / ET_HEX (xfem/symboliccutbfi.cpp:76-486) with the quad branch of
 * StraightCutIntegrationRule (cutint/straightcutrule.cpp:206-501, 582-677;
 * policy: XG_QUAD_FIRST_ALLOWED / _FIND_OPTIMAL / _ALWAYS_NONE).  Terms (xg_term):
 * MASS, LAPLACE, NGRADU_V / U_NGRADV (normal: the unit gradient of the
 * multilinear level set at the point), CONV, on NEG / POS / IF; order -1 = 2
 * (trial + test order); h = |det J|^(1/D) at the point.  An element is active
 * for a term if it is in the term's set and its domain type is the term's
 * domain or IF.  Output as xg_form_assemble (xg_csr over the active vertices,
 * ascending), values summed in a fixed order.  Device errors go to the mesh's
 * error word (xg_mesh_check). */
typedef struct xg_quad_form xg_quad_form;
int xg_quad_form_create(xg_mesh* mesh, const xg_term* terms, int32_t nterms, int policy, xg_quad_form** out);
int xg_quad_form_destroy(xg_quad_form* form);
/* out: [rows, nnz] sufficient for every level set (all elements active). */
int xg_quad_form_capacity(const xg_quad_form* form, int64_t* out2);
int xg_quad_form_assemble(xg_quad_form* form, const double* d_lset, xg_csr* out, void* stream);

/* out: [cap_rows, cap_nnz] sufficient for any level set on this mesh. */
int xg_form_capacity(const xg_form* form, int64_t* h_out2);

/* BilinearForm::Assemble for the form: element matrices of all volume terms
 * (SymbolicCutBilinearFormIntegrator::T_CalcElementMatrixAdd,
 * xfem/symboliccutbfi.cpp:76-486, summed per element), facet-patch matrices of
 * the patch terms (SymbolicFacetPatchBilinearFormIntegrator::T_CalcFacetMatrix,
 * :1982-2377) and their deterministic row-wise scatter into `out`.  d_dom is
 * the per-element domain type from xg_cutinfo_update for d_lset. */
int xg_form_assemble(xg_form* form, const double* d_lset, const uint8_t* d_dom, xg_csr* out, void* stream);
/* Device error word of the form; synchronise the stream first. Resets it. */
int xg_form_check(xg_form* form);
/* Profiling hook: with n = 8 cudaEvent_t handles (passed as void*), every
 * xg_cutfem_step records them on its stream at the stage boundaries
 *   [0] start, [1] marking done, [2] work lists done, [3] uncut element
 *   matrices, [4] cut element matrices, [5] facet-patch matrices,
 *   [6] row pattern counted, [7] values scattered.
 * n = 0 switches it off.  The events are the caller's. */
int xg_form_stage_events(xg_form* form, void* const* events, int n);

/* ---- bilinear forms on regions of several level sets ------------------- */
/* SymbolicCutBFI with a multi-level-set LevelsetIntegrationDomain
 * (symboliccutbfi.cpp:76-486 on the rules of cutint/mlsetintegration.cpp:
 * 6-180, e.g. tests/pytests/test_mlset_poisson.py): a region term integrates
 * its kind over the union of ntup domain tuples of the M level sets (entries
 * XG_NEG / XG_POS / XG_IF, the codimension given by the IF entries); the
 * normal of XG_TERM_NGRADU_V / _U_NGRADV is grad(l)/|grad(l)| of the P1
 * level set normal_lset (an outer normal pointing into POS; a sign goes into
 * coef). */
typedef struct {
  int32_t kind;             /* XG_TERM_MASS .. XG_TERM_CONV */
  int32_t order;            /* -1: the default of the kind */
  int32_t hpow;
  int32_t normal_lset;
  double coef;
  double b[3];              /* XG_TERM_CONV */
  int32_t ntup;             /* 1..256 */
  const int8_t* h_tuples;   /* host [ntup][M] */
  const uint64_t* d_defined_on; /* element bits, NULL = all */
} xg_mlterm;
/* patch_terms: XG_TERM_GHOST_MASS terms with their facet sets (d_defined_on). */
int xg_mlset_form_create(xg_space* space, int32_t M, const xg_mlterm* terms, int32_t nterms,
                         const xg_term* patch_terms, int32_t npatch, int precision, xg_form** out);
/* d_lsets: [M][nv] P1 vertex values.  The active elements are the union of
 * the region terms' element sets; the CSR as xg_form_assemble's. */
int xg_mlset_form_assemble(xg_form* form, const double* d_lsets, xg_csr* out, void* stream);

/* ---- linear forms (xfem/symboliccutlfi.cpp) --------------------------------- */
typedef enum {
  XG_LTERM_SOURCE = 0,     /* coef * x^e0 y^e1 z^e2 * v                         */
  XG_LTERM_SOURCE_GF = 1,  /* coef * u_h * v, u_h = d_gf (dof vector of gf_space, NULL: the form's space) */
  XG_LTERM_SOURCE_BND = 2  /* coef * x^e0 y^e1 z^e2 * v * dCut(lset, domain, vb=BND): the
                              domain part of the BND elements (xg_integrate_bnd's rule, the
                              trace of the owning element's basis); d_defined_on: bits over
                              the BND elements; XG_IF in 2D only */
} xg_lterm_kind;
/* One SymbolicCutLFI(cf * v * dCut(lset, domain, order, definedonelements)). */
typedef struct {
  int32_t kind;               /* xg_lterm_kind */
  int32_t domain;             /* XG_NEG / XG_POS / XG_IF */
  int32_t order;              /* -1: 2k (symboliccutlfi.cpp:93-94) */
  int32_t e[3];               /* exponents of XG_LTERM_SOURCE */
  double coef;
  const double* d_gf;         /* XG_LTERM_SOURCE_GF */
  const uint64_t* d_defined_on; /* element bits; NULL = all */
  const xg_space* gf_space;   /* XG_LTERM_SOURCE_GF: u_h's space (spatial H1 / L2 of order 1..3 on the
                                 form's mesh); NULL: the form's space */
} xg_lterm;
typedef struct xg_lform xg_lform;
/* At most 8 terms on a spatial H1 space. */
int xg_lform_create(xg_space* space, const xg_lterm* terms, int32_t nterms, xg_lform** out);
/* The form's volume terms on the deformed mesh (d_gdef from xg_iso_deformation,
 * NULL = undeformed): the straight cut rule mapped by xhat + Theta(xhat),
 * weights |det (J A)| (IF: times |(J A)^-T n_ref|), x the deformed point. */
int xg_lform_set_deformation(xg_lform* form, const double* d_gdef);
int xg_lform_destroy(xg_lform* lform);
/* LinearForm::Assemble: element vectors (SymbolicCutLinearFormIntegrator::
 * T_CalcElementVector, symboliccutlfi.cpp:57-180) summed per dof in ascending
 * element order into d_out[ndof]; d_dom from xg_cutinfo_update for d_lset. */
int xg_lform_assemble(xg_lform* lform, const double* d_lset, const uint8_t* d_dom, double* d_out, void* stream);
int xg_lform_check(xg_lform* lform);

/* ---- space-time (cutint/spacetimecutrule.cpp, spacetime/) ------------------------ */
/* Space-time level sets are P1 in space and P_kt in time on the reference slab
 * tau in [0,1] (nodal Gauss-Lobatto time basis: kt=1 nodes {0,1}, kt=2 nodes
 * {0,1/2,1}), stored time-major: d_lset_st[i*nv + v] = value of vertex v at
 * time node i.  Space-time dofs: (time dof i, spatial dof j) -> i*ndof_space + j. */
int xg_space_create_st(xg_mesh* mesh, int order, int order_time, xg_space** out);
/* out: [ndof, ndof_per_element, order, order_time, ndof_space, ndof_per_element_space] */
int xg_space_info_st(const xg_space* space, int64_t* h_out6);
/* CutInformation::Update(lset_st, time_order=0) (xfem/cutinfo.cpp:61-132 with
 * SpaceTimeCutIntegrationRule of orders 0/0): cut ratios, domain types and the
 * combined-domain bitsets of the space-time prisms. */
int xg_cutinfo_update_st(xg_mesh* mesh, const double* d_lset_st, int kt_lset, uint8_t* d_dom, double* d_cut_ratio,
                         uint64_t* d_bits, void* stream);
/* SpaceTimeCutIntegrationRule (cutint/spacetimecutrule.cpp:106-244): points get
 * 4 doubles (xi, eta, zeta, tau); weights carry w * w_t * (t1 - t0).
 * order_space -1 selects 5 as the reference does. */
int xg_st_cut_rules(xg_mesh* mesh, const double* d_lset_st, int kt_lset, const int32_t* d_elems, int32_t n, int dt,
                    int order_space, int order_time, int32_t max_pts, int32_t* d_counts, double* d_pts, double* d_wts,
                    void* stream);
/* A space-time integrator: dCut(lset_st, domain, time_order=...) over the slab
 * (tref < 0) or dCut(lset_trace, domain, tref=...) at a fixed reference time,
 * and dFacetPatch(time_order=...) patch terms (spatial patch rule x time rule).
 * The convection field may depend on time:
 *   b(t) = base.b + bc cos(omega t) + bs sin(omega t),  t = t0 + dt * tau. */
typedef struct {
  xg_term base;
  double tref;
  double bc[3], bs[3];
  double omega, t0, dt;
} xg_st_term;
/* kt_lset: time order of the level set; order_time: time rule order (<= 7). */
int xg_st_form_create(xg_space* st_space, int kt_lset, int order_time, const xg_st_term* terms, int32_t nterms,
                      int precision, xg_form** out);
/* The space-time CutFEM step of demos/spacetime/spacetimeDG_unfitted.py:143-185:
 * space-time CutInfo, ghost facets (HASNEG, IF), element matrices of the
 * slab / fixed-time terms on HASNEG (IF terms on IF, POS terms on HASPOS) and
 * the patch terms on the ghost facets, scattered into `out`. */
int xg_st_cutfem_step(xg_form* form, const double* d_lset_st, xg_csr* out, void* stream);

/* ---- the CutFEM step (demos/fictdom.py:95-133) ----------------------------- */
/* One call runs the whole cut-assembly step on `stream`: CutInfo marking,
 * HASNEG / IF / HASPOS element sets, ghost facets (HASNEG, IF) when the form
 * has patch terms, and xg_form_assemble with NEG terms on HASNEG, IF terms on
 * IF, POS terms on HASPOS and patch terms on the ghost facets.  The level set
 * is the P1 vertex vector (already perturbed).  Graph-capturable. */
int xg_cutfem_step(xg_form* form, const double* d_lset, xg_csr* out, void* stream);
/* Device views of the marking of the last step (owned by the form). */
int xg_cutfem_marking(xg_form* form, const uint8_t** d_dom, const double** d_cut_ratio, const uint64_t** d_bits,
                      const uint64_t** d_facets);

/* ---- P2 level sets on tetrahedra: isoparametric and learned cut quadrature ---- */
/* P2 nodal values per element (10 doubles): the 4 vertex values, then the
 * edge midpoints of (0,1),(0,2),(0,3),(1,2),(1,3),(2,3); reference tet
 * (1,0,0),(0,1,0),(0,0,1),(0,0,0).  Moments: x^a y^b z^c of the NEG part,
 * a+b+c <= 4, graded order (t = 0..4, a = t..0, b = t-a..0): 35 doubles.
 *
 * xg_iso_moments_tet: the reference's P2 workflow on a one-element mesh -
 * LevelSetMeshAdaptation's deformation (lsetcurving/shiftintegrators.cpp:38-122,
 * calcpointshift.cpp:143-201, projshift.cpp:58-135) followed by the straight
 * cut rule of the P1 interpolant on the deformed element (rule order `order`);
 * deform = 0 gives the straight cut rule alone.  d_nonconv (optional): number
 * of point searches that did not converge per element (-1: bad decomposition). */
int xg_iso_moments_tet(const double* d_vals10, int64_t n, int order, int deform, double* d_out35,
                       int32_t* d_nonconv, void* stream);
/* The learned cut quadrature (no counterpart in the reference): straight cut
 * rule of the P1 interpolant + 24 weights at a fixed point set predicted by an
 * MLP 10 -> 256 -> 256 -> 24 (SiLU) from the normalised nodal values; FP32
 * master parameters, BF16 copies in every product, FP32 accumulation. */
typedef struct xg_mlp xg_mlp;
int xg_mlp_param_count(int64_t* h_out);
/* the 24 fixed points (reference coordinates, 72 doubles) */
int xg_learned_points(double* h_pts72);
int xg_mlp_create(uint64_t seed, xg_mlp** out);
int xg_mlp_destroy(xg_mlp* mlp);
/* FP32 master parameters, flat: W1[10][256], b1[256], W2[256][256], b2[256], W3[256][24], b3[24] */
int xg_mlp_get_params(const xg_mlp* mlp, float* d_out, void* stream);
int xg_mlp_set_params(xg_mlp* mlp, const float* d_in, void* stream);
/* y[B][24] = MLP(x[B][10]) (x from xg_learned_features); B <= 4,194,240 */
int xg_mlp_forward(xg_mlp* mlp, const float* d_x, int64_t B, float* d_y, void* stream);
/* The same forward pass on the sm_103a tensor cores (tcgen05.mma, BF16
 * operands including the activations, FP32 accumulation in tensor memory),
 * the three layers fused per tile of 128 rows; xg_learned_moments_tet uses it.
 * Its device status (XG_ERR_TIMEOUT if a bounded wait gave up) is read and
 * cleared by xg_mlp_check. */
int xg_mlp_forward_tc(xg_mlp* mlp, const float* d_x, int64_t B, float* d_y, void* stream);
int xg_mlp_check(xg_mlp* mlp);
/* mean over the batch of sum_a ((U y / 256 - t)_a / s)^2, V = U R the thin QR of
 * V[a][i] = p_i^a (weights at the points: R^-1 y); t[B][35]
 * the moment defects, s[B] the scales; gradient into d_grad (flat, like the
 * parameters; NULL: internal buffer used by xg_mlp_adam_step). */
int xg_mlp_loss_grad(xg_mlp* mlp, const float* d_x, const float* d_t35, const float* d_s, int64_t B, float* d_loss,
                     float* d_grad, void* stream);
/* Adam (0.9, 0.999, 1e-8) step t >= 1 with d_grad (NULL: the internal gradient). */
int xg_mlp_adam_step(xg_mlp* mlp, const float* d_grad, float lr, int64_t t, void* stream);
/* the network's input features of n elements (10 floats each): u = v / max|v|,
 * the 4 vertex values of u, then the 6 edge-midpoint deviations
 * u_e - (u_a + u_b) / 2 */
int xg_learned_features(const double* d_vals10, int64_t n, float* d_x10, void* stream);
/* learned NEG moments of n <= 4,194,240 elements: straight cut part (FP64) +
 * the network's correction kOutScale * U y with kOutScale = 1/256 (FP64).
 * kappa_max >= 0: elements in the relevant band whose curvature indicator
 * max_e |u_e - (u_a + u_b) / 2| exceeds kappa_max take the isoparametric rule
 * (order 8) instead; their number goes to d_nfallback (optional). */
int xg_learned_moments_tet(xg_mlp* mlp, const double* d_vals10, int64_t n, double kappa_max, double* d_out35,
                           int32_t* d_nfallback, void* stream);
/* xg_learned_moments_tet with the plain rule chosen: plain_subdivlvl < 0 the
 * isoparametric rule (as above); 0..6 the subdivision rule of that level
 * (xg_subdiv_moments_tet), the reference's own rule for a P2 level set
 * without mesh deformation (cutint/xintegration.cpp:1626-1754), which then
 * serves as the fallback (the stream is synchronised as for
 * xg_subdiv_moments_tet, once more to read the fallback count).  Rule errors
 * go to the network's status word (xg_mlp_check). */
int xg_learned_moments_tet_ex(xg_mlp* mlp, const double* d_vals10, int64_t n, double kappa_max, int plain_subdivlvl,
                              double* d_out35, int32_t* d_nfallback, void* stream);

/* ---- batched steps in one CUDA graph --------------------------------------- */
/* No counterpart in the reference, which assembles one form per
 * BilinearForm::Assemble call (NGSolve's TaskManager parallelises inside it).
 * Captures, once, the steps (forms[i], d_lsets[i], outs[i]) i < n -
 * xg_cutfem_step for plain forms, xg_st_cutfem_step for space-time ones - into
 * one CUDA graph: the steps of distinct forms are independent branches that
 * run concurrently, repeated entries of the same form run in list order.
 * Pointers are baked into the graph, so level sets and outputs must stay at
 * the same addresses (the caller updates their contents between launches);
 * distinct forms must write distinct outputs.  Stage events are off inside the
 * graph.  Check each form with xg_form_check after a launch. */
typedef struct xg_step_graph xg_step_graph;
/* Spatial forms whose patch matrices come from the basis-change kernel (patch
 * terms of order >= 2k), taking one step each in the graph, share one
 * persistent launch for those matrices: work items (form, batch of facets)
 * from a queue ordered by decreasing cost per item, taken by the blocks from
 * an atomic counter (work stealing); the matrices are bit-identical to the
 * per-form kernel's. */
int xg_step_graph_create(xg_form* const* forms, const double* const* d_lsets, const xg_csr* outs, int32_t n,
                         xg_step_graph** out);
int xg_step_graph_launch(xg_step_graph* graph, void* stream);
/* Number of kernel nodes of the graph (the kernels one launch runs). */
int xg_step_graph_kernel_count(const xg_step_graph* graph, int64_t* h_out);
int xg_step_graph_destroy(xg_step_graph* graph);

/* ---- autotuner --------------------------------------------------------------- */
/* No counterpart in the reference.  Times, on this form and level set
 * (d_lset, output out as for xg_cutfem_step; several steps run), the launch
 * choices of the spatial step per (device, dimension, order, precision):
 * elements per block of the uncut element kernel (16, 32), rows per block of
 * the row passes (4 or 8 warps) and accumulator copies of the row sums (1..4,
 * which fix their summation order: every choice is deterministic), blocks per
 * SM of the basis-change patch kernel; keeps the fastest of each (median of
 * three timed steps of its stage) in a per-process table that forms created
 * later with the same key use.  Space-time forms: nothing to tune (XG_OK). */
int xg_form_autotune(xg_form* form, const double* d_lset, xg_csr* out, void* stream);
/* The table as JSON text into buf (cap bytes, NUL-terminated, truncated if
 * short); returns the bytes the full text needs. */
int64_t xg_autotune_table(char* buf, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif

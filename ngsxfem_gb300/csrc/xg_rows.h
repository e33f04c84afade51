// Row-major contribution layout of the spatial scatter (host interface of
// xg_rows.cu; the element kernels of xg_asm.cu write into it).
//
// NGSolve's BilinearForm::Assemble adds every element matrix into the sparse
// matrix (A[dofs_i, dofs_j] += elmat) and the facet-patch matrices of the
// ghost penalty likewise (xfem/symboliccutbfi.cpp:1982-2377 per facet); the
// pattern is the graph of the active elements and facets
// (utils/restrictedblf.cpp:7-168).  Here:
//
//   element rows   row i of element e is written at adjacency slot a = the
//                  position of (e, i) in the dof -> element adjacency of
//                  dof(e, i) (el_rowslot[e * nd + i] = a), so the rows that
//                  one dof row receives from its elements are contiguous, in
//                  ascending element order; their columns' positions in the
//                  dof's full-pattern row are static (pos_rows[a * nd + j]);
//   patch rows     the facet-patch matrices stay compact by active-facet slot
//                  fs (full rows of 2 nd); a patch row reaches a dof row
//                  through a candidate c = a * nfl + lf (adjacency entry a,
//                  local facet lf of its element): per step k_fa_mark records
//                  cand_fs[c] = fs * 2nd + p for the active facets, and the
//                  positions of the neighbour element's columns in the dof's
//                  full row are static (nbpos[c * nd + j], form creation).
//
// k_rows_accum (warp per active row) sums the row's element rows (adjacency
// order) and patch rows (candidate order) in FP64 in shared memory, writes the
// row's active columns and values compacted at the row's full-pattern offset,
// and counts them; after the row-pointer scan k_rows_copy moves each row into
// the output.  No atomics touch values: the sums are formed in the same order
// on every run.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace xg {

struct RowsArgs {
  int ne, nd, nfl, n2;        // elements, dofs per element, facets per element, 2 nd
  int W;                      // 32-bit words of a row (full rows up to 32 W columns)
  int copies;                 // accumulator copies per warp in the accumulation pass (1..4)
  int warps;                  // warps (rows in flight) per block of the row passes (<= kRowsMaxWarps)
  const int32_t* el_dofs;     // [ne][nd]
  const int32_t* el_facets;   // [ne][nfl]
  const int2* fel;            // [nf] first / second element of a facet (-1: boundary)
  const int32_t* adj_ptr;     // [ndof + 1]
  const int32_t* adj;         // (element << 5) | local index, elements ascending per dof
  const int32_t* l_fa;        // active-facet slot -> facet
  const int32_t* rows;        // row -> dof (active dofs, ascending)
  const int32_t* dof_row;     // dof -> row
  const int* counts;          // [2] active facets, [3] active rows
  const int64_t* full_ptr;    // [ndof + 1] full-pattern row offsets
  const int32_t* tmp_cols;    // full-pattern columns of every dof row (sorted)
  int32_t* el_rowslot;        // [ne][nd] static element row slots (form creation)
  uint16_t* pos_rows;         // [ne * nd][nd] full-row positions of the element rows (form creation)
  uint16_t* nbpos;            // [ne * nd * nfl][nd] positions of the neighbour's columns (form creation;
                              // nullptr without patch terms)
  uint8_t* act_slot;          // [ne * nd] 1 for the adjacency slots of this step's active elements
                              // (set by the dof marking, cleared by the accumulation pass)
  int32_t* cand_fs;           // [ne * nd * nfl] patch row of a candidate this step, -1 otherwise
                              // (nullptr without patch terms)
  int32_t* vcols;             // [full_nnz] compacted columns (global dofs) of each active row at its full offset
  double* vvals;              // [full_nnz] compacted values likewise (both nullptr for forms whose full
                              // pattern is too large: a counting pass and the scan come first and the
                              // accumulation pass writes into the output)
  int64_t* rowcnt;            // [ndof] active columns per row
  int64_t cap_fa;
  long long* bsum;            // scan block sums
  int nbsum;
  int* err;
};

// Form creation: el_rowslot, pos_rows and (has_patch) nbpos from the
// adjacency and the full pattern; cand_fs cleared.
int rows_static_build(const RowsArgs& A, bool has_patch, cudaStream_t s);
// Per step, after the active lists, the element and patch kernels and the
// active rows: the candidates' patch rows, the sums, the row pointers
// (out_rowptr, out_counts = {nrows, nnz}, capacity checked against cap_nnz)
// and the compressed output.  elrows / farows hold the element and patch rows
// (FP64, or FP32 for the mixed form).
int rows_scatter(const RowsArgs& A, int64_t ndof, bool has_patch, bool fp64, const void* elrows,
                 const void* farows, int64_t* out_rowptr, int64_t* out_counts, int32_t* cols, double* vals,
                 int64_t cap_nnz, int grid, size_t smem, cudaStream_t s);
// Shared bytes per block of the accumulation pass and its grid (blocks of
// A.warps warps); 0 from rows_accum_grid if the element type is not
// supported or the shared memory is too large.
size_t rows_accum_smem(const RowsArgs& A);
int rows_accum_grid(const RowsArgs& A, bool fp64, size_t smem);
constexpr int kRowsMaxWarps = 8;

}  // namespace xg

// Boundary terms of linear forms, one BND element (host and device):
// coef * x^e0 y^e1 z^e2 * v over the domain part of the boundary element
// (the rule of ml::bnd_rule: straightcutrule.cpp:582-677 on a boundary
// element) with v the trace of the owning element's H1 basis, evaluated at the
// rule's physical points through the inverse of the owner's affine map
// (symboliccutlfi.cpp:57-180 with vb == BND).  The GPU kernel k_lf_bnd
// (xg_lf.cu) runs it per BND element; tests/native/lf_bnd_check.cu runs the
// same code on the host against the oracle.
#pragma once

#include "xg.h"
#include "xg_basis.cuh"
#include "xg_mlset.cuh"

namespace xg {
namespace lfb {

XG_QHD bool bit(const uint64_t* b, int64_t i) { return (b[i >> 6] >> (i & 63)) & 1ull; }

XG_QHD double ipow(double x, int e) {
  double r = 1.0;
  for (int k = 0; k < e; k++) r *= x;
  return r;
}

// x0 = owner vertex D, Finv = (x_k - x_D)_k ^-1 (adjugate / determinant)
template <int D>
XG_QHD void owner_inverse(const double (*xv)[3], double* x0, double (*Finv)[3]) {
  double F[3][3];
  for (int i = 0; i < D; i++) {
    x0[i] = xv[D][i];
    for (int k = 0; k < D; k++) F[i][k] = xv[k][i] - xv[D][i];
  }
  if (D == 2) {
    const double id = 1.0 / (F[0][0] * F[1][1] - F[0][1] * F[1][0]);
    Finv[0][0] = F[1][1] * id;
    Finv[0][1] = -F[0][1] * id;
    Finv[1][0] = -F[1][0] * id;
    Finv[1][1] = F[0][0] * id;
  } else {
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        // cofactor of F[j][i]
        const int r0 = (j + 1) % 3, r1 = (j + 2) % 3, c0 = (i + 1) % 3, c1 = (i + 2) % 3;
        Finv[i][j] = F[r0][c0] * F[r1][c1] - F[r0][c1] * F[r1][c0];
      }
    const double det = F[0][0] * Finv[0][0] + F[0][1] * Finv[1][0] + F[0][2] * Finv[2][0];
    const double id = 1.0 / det;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) Finv[i][j] *= id;
  }
}

// acc[N] = the vector of BND element b (owner vertices xv, ids gv; boundary
// vertices xb ascending with level-set values lb) over the XG_LTERM_SOURCE_BND
// terms; returns 0 or the first xg status
template <int D, int K>
XG_QNI int element_vector(const RuleTable* Rp, const double (*xv)[3], const int* gv, const double (*xb)[3],
                          const double* lb, const xg_lterm* terms, int nterms, int64_t b, double* acc) {
  constexpr int N = ndof_el(D, K);
  double x0[3], Finv[3][3];
  owner_inverse<D>(xv, x0, Finv);
  int desc[N];
  for (int i = 0; i < N; i++) {
    desc[i] = fn_desc<D, K>(i, gv);
    acc[i] = 0.0;
  }
  int status = 0;
  for (int t = 0; t < nterms; t++) {
    const xg_lterm& T = terms[t];
    if (T.kind != XG_LTERM_SOURCE_BND || (T.d_defined_on && !bit(T.d_defined_on, b))) continue;
    const int p = T.order >= 0 ? (T.order < kMaxOrder ? T.order : kMaxOrder) : 2 * K;
    auto emit = [&](const double* x, double w, double meas) {
      double lam[D + 1], sl = 0.0;
      for (int k = 0; k < D; k++) {
        double s = 0.0;
        for (int c = 0; c < D; c++) s += Finv[k][c] * (x[c] - x0[c]);
        lam[k] = s;
        sl += s;
      }
      lam[D] = 1.0 - sl;
      const double g = T.coef * ipow(x[0], T.e[0]) * ipow(x[1], T.e[1]) * (D == 3 ? ipow(x[2], T.e[2]) : 1.0);
      const double wq = w * meas * g;
      for (int i = 0; i < N; i++) acc[i] += wq * eval_fn_value<D, double>(desc[i], lam);
    };
    const int st = ml::bnd_rule<D>(Rp, xb, lb, T.domain, p, emit);
    if (st && !status) status = st;
  }
  return status;
}

}  // namespace lfb
}  // namespace xg

// Thin C driver around the reference's own header-only linear-algebra
// primitives (linalgebra/interface/*.hpp of the reference project), compiled
// from the reference tree in place by oracle/build_oracle.py into
// oracle/_ref/libref_linalgebra.so. TEST INFRASTRUCTURE ONLY: the tests use it
// to pin the oracle's restatement of those primitives bit for bit.
//
// The headers need no third-party code; fused_cholesky_substitution_with_eigen.hpp
// only needs a matrix type with operator()(i,j) and a vector type with
// operator()(i), which the two small accessors below provide.

#include <cmath>

#include "cholesky.hpp"
#include "common.hpp"
#include "fused_cholesky_substitution.hpp"
#include "fused_cholesky_substitution_with_eigen.hpp"
#include "substitution.hpp"

namespace {
struct RowMajorView {
  const double* p;
  int ld;
  double operator()(int i, int j) const { return p[i * ld + j]; }
};
struct VecView {
  const double* p;
  double operator()(int i) const { return p[i]; }
};
}  // namespace

extern "C" {
void ref_cholesky_decomp(double* M, double* L, int full, int view) { cholesky_decomp(M, L, full, view); }
void ref_forward(double* L, double* b, double* y, int full, int view) { solve_forward_substitution(L, b, y, full, view); }
void ref_backward(double* L, double* y, double* x, int full, int view) { solve_backward_substitution(L, y, x, full, view); }
void ref_rc_addition(double* M, double* L, double* b, double* y, int full, int view) {
  fused_cholesky_forward_substitution_solver_rcaddition(M, L, b, y, full, view);
}
void ref_inbetween_removal(double* M, double* L, double* b, double* y, int position, int full, int view) {
  fused_cholesky_forward_substitution_solver_inbetween_removal(M, L, b, y, position, full, view);
}
void ref_eigen_rc_addition(const double* M, double* L, const double* b, double* y, int full, int view) {
  eigen_fused_cholesky_forward_substitution_solver_rcaddition(RowMajorView{M, full}, L, VecView{b}, y, full, view);
}
void ref_eigen_inbetween_removal(const double* M, double* L, const double* b, double* y, int position, int full,
                                 int view) {
  eigen_fused_cholesky_forward_substitution_solver_inbetween_removal(RowMajorView{M, full}, L, VecView{b}, y, position,
                                                                     full, view);
}
void ref_swap_row_column(double* M, int i, int j, int full, int view) { swap_row_column(M, i, j, full, view); }
}

// Driver around the UNMODIFIED DelFEM2 reference headers for scalar (ndim 1)
// and 2x2 (ndim 2) blocks, compiled in place by oracle/Makefile into
// oracle/_ref/libdfm2ref.so next to ref_driver.cpp.
//
// TEST INFRASTRUCTURE ONLY: the reference's own CMatrixSparse,
// CPreconditionerILU, Solve_PCG, Solve_PBiCGStab and the Poisson / 2-D solid
// assembly loops behind the C signatures of the restatement's orc_nd_* and
// orc_assemble_* functions (prefix ref_), so the tests can pin the
// restatement and the fixture script can record the reference's outputs.
#include <climits>
#include <cstdint>
#include <cstring>
#include <vector>

// ls_block_sparse.h must precede fem_poisson.h (its templates call Merge).
// fem_solidlinear.h defines non-inline functions and is included by
// ref_driver.cpp alone, which holds the 2-D solid assembly call.
#include "delfem2/ls_block_sparse.h"
#include "delfem2/fem_poisson.h"
#include "delfem2/ls_ilu_block_sparse.h"
#include "delfem2/lsitrsol.h"
#include "delfem2/vecxitrsol.h"
#include "delfem2/view_vectorx.h"

namespace dfm2 = delfem2;

namespace {

dfm2::CMatrixSparse<double> make_matrix_nd(uint32_t nblk, uint32_t ndim, const uint32_t *row_start,
                                           const uint32_t *col, const double *vcrs, const double *vdia) {
  dfm2::CMatrixSparse<double> m;
  m.Initialize(nblk, ndim, true);
  m.SetPattern(row_start, nblk + 1, col, row_start[nblk]);
  const size_t bb = (size_t)ndim * ndim;
  if (vcrs) std::memcpy(m.val_crs_.data(), vcrs, sizeof(double) * bb * row_start[nblk]);
  if (vdia) std::memcpy(m.val_dia_.data(), vdia, sizeof(double) * bb * nblk);
  return m;
}

void read_back(const dfm2::CMatrixSparse<double> &m, uint32_t nblk, uint32_t ndim, const uint32_t *row_start,
               double *vcrs, double *vdia) {
  const size_t bb = (size_t)ndim * ndim;
  std::memcpy(vcrs, m.val_crs_.data(), sizeof(double) * bb * row_start[nblk]);
  std::memcpy(vdia, m.val_dia_.data(), sizeof(double) * bb * nblk);
}

// CPreconditionerILU filled in place (its copy constructor does not compile).
void fill_ilu_nd(dfm2::CPreconditionerILU<double> &ilu, uint32_t nblk, uint32_t ndim, const uint32_t *row_start,
                 const uint32_t *col, const uint32_t *dia_ind, const double *vcrs, const double *vdia) {
  const size_t bb = (size_t)ndim * ndim;
  ilu.nblk = nblk;
  ilu.ndim = ndim;
  ilu.colInd.assign(row_start, row_start + nblk + 1);
  ilu.rowPtr.assign(col, col + row_start[nblk]);
  ilu.m_diaInd.assign(dia_ind, dia_ind + nblk);
  ilu.valCrs.assign(vcrs, vcrs + bb * (size_t)row_start[nblk]);
  if (vdia) {
    ilu.valDia.assign(vdia, vdia + bb * (size_t)nblk);
  } else {
    ilu.valDia.assign(bb * (size_t)nblk, 0.0);
  }
}

}  // namespace

extern "C" {

void ref_nd_matvec(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                   const double *vcrs, const double *vdia, double *y, double alpha, const double *x,
                   double beta) {
  auto m = make_matrix_nd(nblk, ndim, row_start, col, vcrs, vdia);
  m.MatVec(y, alpha, x, beta);
}

int ref_nd_merge(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                 double *vdia, uint32_t nnoel, const uint32_t *nodes, const double *emat, uint32_t *merge_buffer) {
  (void)merge_buffer;
  auto m = make_matrix_nd(nblk, ndim, row_start, col, vcrs, vdia);
  std::vector<unsigned int> buf(nblk, UINT_MAX);
  const bool ok = dfm2::Mearge(m, nnoel, nodes, nnoel, nodes, ndim * ndim, emat, buf);
  read_back(m, nblk, ndim, row_start, vcrs, vdia);
  return ok ? 0 : 1;
}

void ref_nd_set_fixed_bc(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                         double *vcrs, double *vdia, const int *bc) {
  auto m = make_matrix_nd(nblk, ndim, row_start, col, vcrs, vdia);
  m.SetFixedBC(bc);
  read_back(m, nblk, ndim, row_start, vcrs, vdia);
}

// CopyValue into the pattern Initialize_ILUk(m, lev_fill) builds for the
// matrix (the caller's irow_start / col_ilu must equal it; nothing is written
// otherwise).
void ref_nd_ilu_copy_value(uint32_t nblk, uint32_t ndim, const uint32_t *mrow_start, const uint32_t *col_mat,
                           const double *mat_vcrs, const double *mat_vdia, int lev_fill,
                           const uint32_t *irow_start, const uint32_t *col_ilu, double *ilu_vcrs,
                           double *ilu_vdia) {
  auto m = make_matrix_nd(nblk, ndim, mrow_start, col_mat, mat_vcrs, mat_vdia);
  dfm2::CPreconditionerILU<double> ilu;
  ilu.Initialize_ILUk(m, lev_fill);
  if (ilu.rowPtr.size() != irow_start[nblk]) return;
  for (size_t s = 0; s < ilu.rowPtr.size(); ++s)
    if (ilu.rowPtr[s] != col_ilu[s]) return;
  ilu.CopyValue(m);
  std::memcpy(ilu_vcrs, ilu.valCrs.data(), sizeof(double) * ilu.valCrs.size());
  std::memcpy(ilu_vdia, ilu.valDia.data(), sizeof(double) * ilu.valDia.size());
}

int ref_nd_ilu_decompose(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                         const uint32_t *dia_ind, double *vcrs, double *vdia, int *n_singular) {
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu_nd(ilu, nblk, ndim, row_start, col, dia_ind, vcrs, vdia);
  const bool ok = ilu.Decompose();
  std::memcpy(vcrs, ilu.valCrs.data(), sizeof(double) * ilu.valCrs.size());
  std::memcpy(vdia, ilu.valDia.data(), sizeof(double) * ilu.valDia.size());
  if (n_singular) *n_singular = -1;  // the reference only prints the count
  return ok ? 0 : 1;
}

void ref_nd_ilu_forward(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                        const uint32_t *dia_ind, const double *vcrs, const double *vdia, double *vec) {
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu_nd(ilu, nblk, ndim, row_start, col, dia_ind, vcrs, vdia);
  ilu.ForwardSubstitution(vec);
}

void ref_nd_ilu_backward(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                         const uint32_t *dia_ind, const double *vcrs, double *vec) {
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu_nd(ilu, nblk, ndim, row_start, col, dia_ind, vcrs, nullptr);
  ilu.BackwardSubstitution(vec);
}

uint32_t ref_nd_solve_pcg(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                          const double *vcrs, const double *vdia, const uint32_t *ilu_row_start,
                          const uint32_t *ilu_col, const uint32_t *dia_ind, const double *ilu_vcrs,
                          const double *ilu_vdia, double *r, double *x, double tol, uint32_t max_iter,
                          double *hist, uint32_t hist_cap) {
  auto m = make_matrix_nd(nblk, ndim, row_start, col, vcrs, vdia);
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu_nd(ilu, nblk, ndim, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia);
  const size_t n = (size_t)nblk * ndim;
  std::vector<double> Pr(n), p(n);
  auto h = dfm2::Solve_PCG(dfm2::ViewAsVectorXd(r, n), dfm2::ViewAsVectorXd(x, n), dfm2::ViewAsVectorXd(Pr),
                           dfm2::ViewAsVectorXd(p), tol, max_iter, m, ilu);
  for (size_t k = 0; k < h.size() && k < hist_cap; ++k) hist[k] = h[k];
  return static_cast<uint32_t>(h.size());
}

uint32_t ref_nd_solve_pbicgstab(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                                const double *vcrs, const double *vdia, const uint32_t *ilu_row_start,
                                const uint32_t *ilu_col, const uint32_t *dia_ind, const double *ilu_vcrs,
                                const double *ilu_vdia, double *r, double *x, double tol, uint32_t max_iter,
                                double *hist, uint32_t hist_cap) {
  auto m = make_matrix_nd(nblk, ndim, row_start, col, vcrs, vdia);
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu_nd(ilu, nblk, ndim, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia);
  auto h = dfm2::Solve_PBiCGStab(r, x, tol, max_iter, m, ilu);
  for (size_t k = 0; k < h.size() && k < hist_cap; ++k) hist[k] = h[k];
  return static_cast<uint32_t>(h.size());
}

// MergeLinSys_Poission_MeshTet3D (fem_poisson.h:128-162) into a scalar matrix.
int ref_assemble_poisson_tet(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                             double *vdia, double *b, double alpha, double source, const double *xyz,
                             const uint32_t *tet, size_t ntet, const double *val) {
  auto m = make_matrix_nd(nblk, 1, row_start, col, vcrs, vdia);
  std::vector<double> zero(nblk, 0.0);
  dfm2::MergeLinSys_Poission_MeshTet3D(m, b, alpha, source, xyz, nblk, tet, ntet, val ? val : zero.data());
  read_back(m, nblk, 1, row_start, vcrs, vdia);
  return 0;
}

// MergeLinSys_Poission_MeshTri2D (fem_poisson.h:92-127) into a scalar
// matrix; called by ref_assemble_tri2 (ref_driver.cpp) for ndim 1.
int ref_poisson_tri2(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs, double *vdia,
                     double *b, double alpha, double source, const double *xy, const uint32_t *tri, size_t ntri,
                     const double *val) {
  auto m = make_matrix_nd(nblk, 1, row_start, col, vcrs, vdia);
  std::vector<double> zero(nblk, 0.0);
  dfm2::MergeLinSys_Poission_MeshTri2D(m, b, alpha, source, xy, nblk, tri, ntri, val ? val : zero.data());
  read_back(m, nblk, 1, row_start, vcrs, vdia);
  return 0;
}

}  // extern "C"

// Driver around the UNMODIFIED DelFEM2 reference headers (header-only C++17),
// compiled in place by oracle/Makefile into oracle/_ref/libdfm2ref.so.
//
// TEST INFRASTRUCTURE ONLY: it exposes the reference's own code for the
// 3x3 block ILU(0)-PCG path behind the same C signatures as the plain-C
// restatement (dfm2_oracle.h, prefix ref_ instead of orc_), so the tests can
// pin the restatement against the reference and the fixture script
// (tests/golden/make_golden.py) can record the reference's outputs.
// Nothing here is part of the product library.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

// ls_block_sparse.h must precede fem_solidlinear.h (whose templates call Merge).
#include "delfem2/ls_block_sparse.h"
#include "delfem2/fem_solidlinear.h"
#include "delfem2/gridvoxel.h"
#include "delfem2/jagarray.h"
#include "delfem2/ls_ilu_block_sparse.h"
#include "delfem2/lsitrsol.h"
#include "delfem2/msh_topology_uniform.h"
#include "delfem2/view_vectorx.h"
#include "delfem2/vecxitrsol.h"

namespace dfm2 = delfem2;

namespace {

dfm2::CMatrixSparse<double> make_matrix(uint32_t nblk, const uint32_t *row_start,
                                        const uint32_t *col, const double *vcrs,
                                        const double *vdia) {
  dfm2::CMatrixSparse<double> m;
  m.Initialize(nblk, 3, true);
  m.SetPattern(row_start, nblk + 1, col, row_start[nblk]);
  if (vcrs) std::memcpy(m.val_crs_.data(), vcrs, sizeof(double) * 9 * row_start[nblk]);
  if (vdia) std::memcpy(m.val_dia_.data(), vdia, sizeof(double) * 9 * nblk);
  return m;
}

// CPreconditionerILU's copy constructor does not compile (it names a member
// that does not exist), so the preconditioner is filled in place.
void fill_ilu(dfm2::CPreconditionerILU<double> &ilu, uint32_t nblk, const uint32_t *row_start,
              const uint32_t *col, const uint32_t *dia_ind, const double *vcrs,
              const double *vdia) {
  ilu.nblk = nblk;
  ilu.ndim = 3;
  ilu.colInd.assign(row_start, row_start + nblk + 1);
  ilu.rowPtr.assign(col, col + row_start[nblk]);
  ilu.m_diaInd.assign(dia_ind, dia_ind + nblk);
  ilu.valCrs.assign(vcrs, vcrs + 9 * (size_t)row_start[nblk]);
  ilu.valDia.assign(vdia, vdia + 9 * (size_t)nblk);
}

}  // namespace

extern "C" {

void ref_voxel_tet_mesh(uint32_t nx, uint32_t ny, uint32_t nz, double scale, double *xyz,
                        uint32_t *tet) {
  std::vector<double> aXYZ;
  std::vector<int> aTet;
  std::vector<int> vox(nx * ny * nz, 1);
  dfm2::MeshTet3D_VoxelGrid(aXYZ, aTet, nx, ny, nz, vox);
  for (size_t i = 0; i < aXYZ.size(); ++i) xyz[i] = aXYZ[i] * scale;
  for (size_t i = 0; i < aTet.size(); ++i) tet[i] = static_cast<uint32_t>(aTet[i]);
}

static void psup_build(const uint32_t *elem, size_t nelem, uint32_t nnoel, size_t np,
                       std::vector<unsigned int> &ind, std::vector<unsigned int> &psup) {
  dfm2::JArray_PSuP_MeshElem(ind, psup, elem, nelem, nnoel, np);
  dfm2::JArray_Sort(ind, psup);
}

size_t ref_psup_count(const uint32_t *elem, size_t nelem, uint32_t nnoel, size_t np,
                      uint32_t *psup_ind) {
  std::vector<unsigned int> ind, psup;
  psup_build(elem, nelem, nnoel, np, ind, psup);
  std::memcpy(psup_ind, ind.data(), sizeof(uint32_t) * (np + 1));
  return psup.size();
}

void ref_psup_fill(const uint32_t *elem, size_t nelem, uint32_t nnoel, size_t np,
                   const uint32_t *psup_ind, uint32_t *psup_out) {
  (void)psup_ind;
  std::vector<unsigned int> ind, psup;
  psup_build(elem, nelem, nnoel, np, ind, psup);
  std::memcpy(psup_out, psup.data(), sizeof(uint32_t) * psup.size());
}

void ref_bsr_matvec(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                    const double *vcrs, const double *vdia, double *y, double alpha,
                    const double *x, double beta) {
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  m.MatVec(y, alpha, x, beta);
}

void ref_bsr_matvec_f32(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                        const float *vcrs, const float *vdia, float *y, float alpha,
                        const float *x, float beta) {
  dfm2::CMatrixSparse<float> m;
  m.Initialize(nblk, 3, true);
  m.SetPattern(row_start, nblk + 1, col, row_start[nblk]);
  std::memcpy(m.val_crs_.data(), vcrs, sizeof(float) * 9 * row_start[nblk]);
  std::memcpy(m.val_dia_.data(), vdia, sizeof(float) * 9 * nblk);
  m.MatVec(y, alpha, x, beta);
}

int ref_merge(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
              double *vdia, uint32_t nnoel, const uint32_t *nodes, const double *emat,
              uint32_t *merge_buffer) {
  (void)merge_buffer;
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  std::vector<unsigned int> buf(nblk, UINT_MAX);
  bool ok = dfm2::Mearge(m, nnoel, nodes, nnoel, nodes, 9u, emat, buf);
  std::memcpy(vcrs, m.val_crs_.data(), sizeof(double) * 9 * row_start[nblk]);
  std::memcpy(vdia, m.val_dia_.data(), sizeof(double) * 9 * nblk);
  return ok ? 0 : 1;
}

void ref_set_fixed_bc(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      double *vcrs, double *vdia, const int *bc) {
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  m.SetFixedBC(bc);
  std::memcpy(vcrs, m.val_crs_.data(), sizeof(double) * 9 * row_start[nblk]);
  std::memcpy(vdia, m.val_dia_.data(), sizeof(double) * 9 * nblk);
}

void ref_rhs_zero(double *b, const int *bc, size_t ndof) {
  std::vector<double> vb(b, b + ndof);
  std::vector<int> vf(bc, bc + ndof);
  dfm2::setRHS_Zero(vb, vf, 0);
  std::memcpy(b, vb.data(), sizeof(double) * ndof);
}

void ref_emat_tet_linear(const double P[4][3], double myu, double lambda,
                         double emat[4][4][3][3], double *vol_out) {
  double eres[4][3] = {{0}};
  double disp[4][3] = {{0}};
  for (int i = 0; i < 144; ++i) (&emat[0][0][0][0])[i] = 0.0;
  dfm2::EMat_SolidLinear_Static_Tet(emat, eres, myu, lambda, P, disp, true);
  if (vol_out) *vol_out = dfm2::femutil::TetVolume3D(P[0], P[1], P[2], P[3]);
}

// Per-tet Young's modulus: the caller loop of
// MergeLinSys_SolidLinear_Static_MeshTet3D (fem_solidlinear.h:192-237) with
// (myu, lambda) taken per element.
int ref_assemble_tet_linear(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                            double *vcrs, double *vdia, double *b, const double *xyz,
                            const uint32_t *tet, size_t ntet, const double *young, double nu,
                            double rho, const double g[3], const double *disp) {
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  std::vector<unsigned int> buf(nblk, UINT_MAX);
  bool ok = true;
  for (size_t e = 0; e < ntet && ok; ++e) {
    const unsigned int *aIP = tet + e * 4;
    double P[4][3], U[4][3];
    dfm2::FetchData<4, 3>(P, aIP, xyz);
    if (disp) {
      dfm2::FetchData<4, 3>(U, aIP, disp);
    } else {
      for (auto &u : U) u[0] = u[1] = u[2] = 0.0;
    }
    const double E = young[e];
    const double lambda = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    const double myu = E / (2.0 * (1.0 + nu));
    double eres[4][3];
    const double vol = dfm2::femutil::TetVolume3D(P[0], P[1], P[2], P[3]);
    for (auto &r : eres) {
      r[0] = vol * rho * g[0] * 0.25;
      r[1] = vol * rho * g[1] * 0.25;
      r[2] = vol * rho * g[2] * 0.25;
    }
    double emat[4][4][3][3];
    for (int i = 0; i < 144; ++i) (&emat[0][0][0][0])[i] = 0.0;
    dfm2::EMat_SolidLinear_Static_Tet(emat, eres, myu, lambda, P, U, true);
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) b[aIP[i] * 3 + a] += eres[i][a];
    ok = dfm2::Merge<4, 4, 3, 3, double>(m, aIP, aIP, emat, buf);
  }
  std::memcpy(vcrs, m.val_crs_.data(), sizeof(double) * 9 * row_start[nblk]);
  std::memcpy(vdia, m.val_dia_.data(), sizeof(double) * 9 * nblk);
  return ok ? 0 : 1;
}

void ref_ilu_pattern0(uint32_t nblk, const uint32_t *row_start, const uint32_t *col_in,
                      uint32_t *col_out, uint32_t *dia_ind) {
  auto m = make_matrix(nblk, row_start, col_in, nullptr, nullptr);
  dfm2::CPreconditionerILU<double> ilu;
  ilu.Initialize_ILUk(m, 0);
  std::memcpy(col_out, ilu.rowPtr.data(), sizeof(uint32_t) * ilu.rowPtr.size());
  std::memcpy(dia_ind, ilu.m_diaInd.data(), sizeof(uint32_t) * nblk);
}

// Initialize_ILUk(m, lev_fill) itself; same contract as orc_ilu_pattern_k.
size_t ref_ilu_pattern_k(uint32_t nblk, const uint32_t *row_start, const uint32_t *col_in, int lev_fill,
                         uint32_t *row_start_out, uint32_t *col_out, size_t cap, uint32_t *dia_ind) {
  auto m = make_matrix(nblk, row_start, col_in, nullptr, nullptr);
  dfm2::CPreconditionerILU<double> ilu;
  ilu.Initialize_ILUk(m, lev_fill);
  std::memcpy(row_start_out, ilu.colInd.data(), sizeof(uint32_t) * (nblk + 1));
  const size_t tot = ilu.rowPtr.size();
  if (col_out && cap >= tot) {
    std::memcpy(col_out, ilu.rowPtr.data(), sizeof(uint32_t) * tot);
    std::memcpy(dia_ind, ilu.m_diaInd.data(), sizeof(uint32_t) * nblk);
  }
  return tot;
}

// CopyValue into the pattern Initialize_ILUk(m, lev_fill) builds (which the
// caller passes as irow_start / col_ilu; nothing is written if they differ).
void ref_ilu_copy_value_k(uint32_t nblk, const uint32_t *mrow_start, const uint32_t *col_mat,
                          const double *mat_vcrs, const double *mat_vdia, int lev_fill,
                          const uint32_t *irow_start, const uint32_t *col_ilu, double *ilu_vcrs,
                          double *ilu_vdia) {
  auto m = make_matrix(nblk, mrow_start, col_mat, mat_vcrs, mat_vdia);
  dfm2::CPreconditionerILU<double> ilu;
  ilu.Initialize_ILUk(m, lev_fill);
  if (ilu.rowPtr.size() != irow_start[nblk]) return;
  for (size_t s = 0; s < ilu.rowPtr.size(); ++s)
    if (ilu.rowPtr[s] != col_ilu[s]) return;
  ilu.CopyValue(m);
  std::memcpy(ilu_vcrs, ilu.valCrs.data(), sizeof(double) * 9 * irow_start[nblk]);
  std::memcpy(ilu_vdia, ilu.valDia.data(), sizeof(double) * 9 * nblk);
}

void ref_ilu_copy_value(uint32_t nblk, const uint32_t *row_start, const uint32_t *col_ilu,
                        double *ilu_vcrs, double *ilu_vdia, const uint32_t *col_mat,
                        const double *mat_vcrs, const double *mat_vdia) {
  auto m = make_matrix(nblk, row_start, col_mat, mat_vcrs, mat_vdia);
  dfm2::CPreconditionerILU<double> ilu;
  ilu.SetPattern0(m);
  // SetPattern0 re-derives the sorted pattern; it must equal the caller's.
  for (size_t s = 0; s < ilu.rowPtr.size(); ++s)
    if (ilu.rowPtr[s] != col_ilu[s]) return;
  ilu.CopyValue(m);
  std::memcpy(ilu_vcrs, ilu.valCrs.data(), sizeof(double) * ilu.valCrs.size());
  std::memcpy(ilu_vdia, ilu.valDia.data(), sizeof(double) * ilu.valDia.size());
}

int ref_ilu_decompose(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      const uint32_t *dia_ind, double *vcrs, double *vdia, int *n_singular) {
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu(ilu, nblk, row_start, col, dia_ind, vcrs, vdia);
  const bool ok = ilu.Decompose();
  std::memcpy(vcrs, ilu.valCrs.data(), sizeof(double) * ilu.valCrs.size());
  std::memcpy(vdia, ilu.valDia.data(), sizeof(double) * ilu.valDia.size());
  if (n_singular) *n_singular = -1;  // the reference only prints the count
  return ok ? 0 : 1;
}

void ref_ilu_forward(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                     const uint32_t *dia_ind, const double *vcrs, const double *vdia,
                     double *vec) {
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu(ilu, nblk, row_start, col, dia_ind, vcrs, vdia);
  ilu.ForwardSubstitution(vec);
}

void ref_ilu_backward(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      const uint32_t *dia_ind, const double *vcrs, double *vec) {
  std::vector<double> dummy_dia(9 * (size_t)nblk, 0.0);
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu(ilu, nblk, row_start, col, dia_ind, vcrs, dummy_dia.data());
  ilu.BackwardSubstitution(vec);
}

uint32_t ref_solve_pcg(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                       const double *vcrs, const double *vdia, const uint32_t *ilu_col,
                       const uint32_t *dia_ind, const double *ilu_vcrs, const double *ilu_vdia,
                       double *r, double *x, double tol, uint32_t max_iter, double *hist,
                       uint32_t hist_cap) {
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu(ilu, nblk, row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia);
  const size_t n = (size_t)nblk * 3;
  std::vector<double> Pr(n), p(n);
  auto h = dfm2::Solve_PCG(dfm2::ViewAsVectorXd(r, n), dfm2::ViewAsVectorXd(x, n),
                           dfm2::ViewAsVectorXd(Pr), dfm2::ViewAsVectorXd(p), tol, max_iter, m,
                           ilu);
  for (size_t k = 0; k < h.size() && k < hist_cap; ++k) hist[k] = h[k];
  return static_cast<uint32_t>(h.size());
}

uint32_t ref_solve_pcg_k(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                         const double *vcrs, const double *vdia, const uint32_t *ilu_row_start,
                         const uint32_t *ilu_col, const uint32_t *dia_ind, const double *ilu_vcrs,
                         const double *ilu_vdia, double *r, double *x, double tol, uint32_t max_iter,
                         double *hist, uint32_t hist_cap) {
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu(ilu, nblk, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia);
  const size_t n = (size_t)nblk * 3;
  std::vector<double> Pr(n), p(n);
  auto h = dfm2::Solve_PCG(dfm2::ViewAsVectorXd(r, n), dfm2::ViewAsVectorXd(x, n),
                           dfm2::ViewAsVectorXd(Pr), dfm2::ViewAsVectorXd(p), tol, max_iter, m,
                           ilu);
  for (size_t k = 0; k < h.size() && k < hist_cap; ++k) hist[k] = h[k];
  return static_cast<uint32_t>(h.size());
}

// Solve_PBiCGStab (vecxitrsol.h:350-437) itself, with CPreconditionerILU.
uint32_t ref_solve_pbicgstab(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, const double *vcrs,
                             const double *vdia, const uint32_t *ilu_row_start, const uint32_t *ilu_col,
                             const uint32_t *dia_ind, const double *ilu_vcrs, const double *ilu_vdia, double *r,
                             double *x, double tol, uint32_t max_iter, double *hist, uint32_t hist_cap) {
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  dfm2::CPreconditionerILU<double> ilu;
  fill_ilu(ilu, nblk, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia);
  auto h = dfm2::Solve_PBiCGStab(r, x, tol, max_iter, m, ilu);
  for (size_t k = 0; k < h.size() && k < hist_cap; ++k) hist[k] = h[k];
  return static_cast<uint32_t>(h.size());
}

uint32_t ref_solve_cg(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      const double *vcrs, const double *vdia, double *r, double *x, double tol,
                      uint32_t max_iter, double *hist, uint32_t hist_cap) {
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  const size_t n = (size_t)nblk * 3;
  std::vector<double> Ap(n), p(n);
  auto h = dfm2::Solve_CG(dfm2::ViewAsVectorXd(r, n), dfm2::ViewAsVectorXd(x, n),
                          dfm2::ViewAsVectorXd(Ap), dfm2::ViewAsVectorXd(p), tol, max_iter, m);
  for (size_t k = 0; k < h.size() && k < hist_cap; ++k) hist[k] = h[k];
  return static_cast<uint32_t>(h.size());
}

// MergeLinSys_SolidLinear_BEuler_MeshTet3D (fem_solidlinear.h:381-443) or,
// with rot, MergeLinSys_SolidStiffwarp_BEuler_MeshTet3D (445-530), into the
// given 3x3 matrix; the contract of orc_assemble_tet_beuler.
int ref_assemble_tet_beuler(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                            double *vdia, double *b, double myu, double lambda, double rho, const double g[3],
                            double dt, const double *xyz, const uint32_t *tet, size_t ntet, const double *disp,
                            const double *velo, const double *rot) {
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  if (rot) {
    std::vector<double> aR(rot, rot + (size_t)nblk * 9);
    dfm2::MergeLinSys_SolidStiffwarp_BEuler_MeshTet3D(m, b, myu, lambda, rho, g, dt, xyz, nblk, tet,
                                                      (unsigned)ntet, disp, velo, aR);
  } else {
    dfm2::MergeLinSys_SolidLinear_BEuler_MeshTet3D(m, b, myu, lambda, rho, g, dt, xyz, nblk, tet, (unsigned)ntet,
                                                   disp, velo);
  }
  std::memcpy(vcrs, m.val_crs_.data(), sizeof(double) * 9 * row_start[nblk]);
  std::memcpy(vdia, m.val_dia_.data(), sizeof(double) * 9 * nblk);
  return 0;
}

// MergeLinSys_SolidLinear_NewmarkBeta_MeshTet3D (fem_solidlinear.h:331-379).
int ref_assemble_tet_newmark(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                             double *vdia, double *b, double myu, double lambda, double rho, const double g[3],
                             double dt, double gamma, double beta, const double *xyz, const uint32_t *tet,
                             size_t ntet, const double *disp, const double *velo, const double *acc) {
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  dfm2::MergeLinSys_SolidLinear_NewmarkBeta_MeshTet3D(m, b, myu, lambda, rho, g, dt, gamma, beta, xyz, nblk, tet,
                                                      ntet, disp, velo, acc);
  std::memcpy(vcrs, m.val_crs_.data(), sizeof(double) * 9 * row_start[nblk]);
  std::memcpy(vdia, m.val_dia_.data(), sizeof(double) * 9 * nblk);
  return 0;
}

// elemMatRes_LinearSolidGravity3_Static_Q1 (fem_solidlinear.cpp:238-281).
void ref_emat_hex_q1(const double P[8][3], double myu, double lambda, double rho, const double g[3],
                     const double disp[8][3], double emat[8][8][3][3], double eres[8][3]) {
  dfm2::elemMatRes_LinearSolidGravity3_Static_Q1(myu, lambda, rho, g, P, disp, emat, eres);
}

// The element loop of MergeLinSys_LinearSolid3D_Static_Q1 (fem_solidlinear.h:
// 239-276: elemMatRes_LinearSolidGravity3_Static_Q1, b += r_e, Merge<8,8,3,3>)
// run here on a CMatrixSparse, without the function's own zeroing, whose
// `mat_A.SetZero()` names a member CMatrixSparse does not have (`setZero`).
int ref_assemble_hex_q1(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs, double *vdia,
                        double *b, double myu, double lambda, double rho, const double g[3], const double *xyz,
                        const uint32_t *hex, size_t nhex, const double *disp) {
  auto m = make_matrix(nblk, row_start, col, vcrs, vdia);
  std::vector<unsigned int> buf(nblk, UINT_MAX);
  std::vector<double> zero((size_t)nblk * 3, 0.0);
  const double *u = disp ? disp : zero.data();
  bool ok = true;
  static double emat[8][8][3][3];
  for (size_t e = 0; e < nhex && ok; ++e) {
    const unsigned int *aIP = hex + e * 8;
    double coords[8][3], disps[8][3], eres[8][3];
    dfm2::FetchData<8, 3>(coords, aIP, xyz);
    dfm2::FetchData<8, 3>(disps, aIP, u);
    dfm2::elemMatRes_LinearSolidGravity3_Static_Q1(myu, lambda, rho, g, coords, disps, emat, eres);
    for (int k = 0; k < 8; ++k)
      for (int d = 0; d < 3; ++d) b[aIP[k] * 3 + d] += eres[k][d];
    ok = dfm2::Merge<8, 8, 3, 3, double>(m, aIP, aIP, emat, buf);
  }
  std::memcpy(vcrs, m.val_crs_.data(), sizeof(double) * 9 * row_start[nblk]);
  std::memcpy(vdia, m.val_dia_.data(), sizeof(double) * 9 * nblk);
  return ok ? 0 : 1;
}

int ref_poisson_tri2(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs, double *vdia,
                     double *b, double alpha, double source, const double *xy, const uint32_t *tri, size_t ntri,
                     const double *val);  // ref_driver_nd.cpp

// MergeLinSys_SolidLinear_Static_MeshTri2D (fem_solidlinear.h:155-187,
// ndim 2, param = {myu, lambda, rho, gx, gy}) or, for ndim 1,
// MergeLinSys_Poission_MeshTri2D (param = {alpha, source}); the contract of
// orc_assemble_tri2.
int ref_assemble_tri2(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                      double *vdia, double *b, const double *param, const double *xy, const uint32_t *tri,
                      size_t ntri, const double *val) {
  if (ndim == 1) return ref_poisson_tri2(nblk, row_start, col, vcrs, vdia, b, param[0], param[1], xy, tri, ntri, val);
  dfm2::CMatrixSparse<double> m;
  m.Initialize(nblk, 2, true);
  m.SetPattern(row_start, nblk + 1, col, row_start[nblk]);
  std::memcpy(m.val_crs_.data(), vcrs, sizeof(double) * 4 * row_start[nblk]);
  std::memcpy(m.val_dia_.data(), vdia, sizeof(double) * 4 * nblk);
  std::vector<double> zero((size_t)nblk * 2, 0.0);
  dfm2::MergeLinSys_SolidLinear_Static_MeshTri2D(m, b, param[0], param[1], param[2], param[3], param[4], xy, nblk,
                                                 tri, ntri, val ? val : zero.data());
  std::memcpy(vcrs, m.val_crs_.data(), sizeof(double) * 4 * row_start[nblk]);
  std::memcpy(vdia, m.val_dia_.data(), sizeof(double) * 4 * nblk);
  return 0;
}

}  // extern "C"

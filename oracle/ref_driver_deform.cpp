// Driver around the UNMODIFIED DelFEM2 reference headers for the two
// deformers that solve through the block ILU-PCG path: the ARAP deformer
// (Deformer_Arap, defarap.cpp: per-point ARAP elements merged with the
// runtime-size Merge, ILU(0), Solve_PCG to 1e-7) and the linear Laplacian
// deformer (CDef_LaplacianLinear, deflap.cpp: dual-Laplacian elements, ILU(20)
// of the matrix with the boundary penalties, Solve_PCG over its own MatVec).
//
// TEST INFRASTRUCTURE ONLY (compiled by oracle/Makefile into
// oracle/_ref/libdfm2ref.so): the fixture script records the element matrices
// these callers hand to Merge, the ILU(20) pattern and the reference's own
// solves, so the GPU tests can drive the same systems through the C ABI.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "delfem2/ls_block_sparse.h"
#include "delfem2/defarap.h"
#include "delfem2/deflap.h"
#include "delfem2/jagarray.h"
#include "delfem2/ls_ilu_block_sparse.h"
#include "delfem2/lsitrsol.h"
#include "delfem2/mat3.h"
#include "delfem2/msh_topology_uniform.h"
#include "delfem2/vec3.h"

namespace dfm2 = delfem2;

namespace {

// 1-ring of every point of a triangle mesh, sorted (as Deformer_Arap::Init).
void one_ring(std::vector<unsigned> &ind, std::vector<unsigned> &psup, uint32_t np, uint32_t ntri,
              const uint32_t *tri) {
  dfm2::JArray_PSuP_MeshElem(ind, psup, tri, ntri, 3, np);
  dfm2::JArray_Sort(ind, psup);
}

// Per-point matrix of Deformer_Arap::Init: inverse of sum_j CrossCross(x_j - x_i).
void arap_precomp(std::vector<double> &precomp, uint32_t np, const double *xyz0, const std::vector<unsigned> &ind,
                  const std::vector<unsigned> &psup) {
  precomp.resize(np * 9);
  for (unsigned ip = 0; ip < np; ++ip) {
    const dfm2::CVec3d Pi(xyz0 + ip * 3);
    dfm2::CMat3d LM;
    LM.setZero();
    for (unsigned k = ind[ip]; k < ind[ip + 1]; ++k) {
      const dfm2::CVec3d v0 = dfm2::CVec3d(xyz0 + psup[k] * 3) - Pi;
      LM += dfm2::Mat3_CrossCross(v0);
    }
    dfm2::CMat3d LMi = LM.Inverse();
    LMi.CopyTo(precomp.data() + ip * 9);
  }
}

}  // namespace

extern "C" {

// Sizes of the ARAP elements of a mesh: sum of element sizes (1-ring + self)
// and of their 9 n^2 matrix entries.
void ref_arap_sizes(uint32_t np, uint32_t ntri, const uint32_t *tri, uint64_t *n_idx, uint64_t *n_mat) {
  std::vector<unsigned> ind, psup;
  one_ring(ind, psup, np, ntri, tri);
  uint64_t a = 0, b = 0;
  for (unsigned ip = 0; ip < np; ++ip) {
    const uint64_t n = ind[ip + 1] - ind[ip] + 1;
    a += n;
    b += 9 * n * n;
  }
  *n_idx = a;
  *n_mat = b;
}

// The element of each point as Deformer_Arap::Deform builds it (points of
// the 1-ring, then the point itself; dWddW_ArapEnergy's matrix and residual),
// concatenated: elem_ptr[np+1] offsets into elem_idx / eR (3 per entry), and
// eM at 9 n^2 per element in the same order.
void ref_arap_elements(uint32_t np, const double *xyz0, uint32_t ntri, const uint32_t *tri, const double *xyz1,
                       const double *quat1, uint32_t *elem_ptr, uint32_t *elem_idx, double *eM_out,
                       double *eR_out) {
  std::vector<unsigned> ind, psup;
  one_ring(ind, psup, np, ntri, tri);
  std::vector<double> precomp;
  arap_precomp(precomp, np, xyz0, ind, psup);
  const std::vector<double> X0(xyz0, xyz0 + np * 3), X1(xyz1, xyz1 + np * 3), Q1(quat1, quat1 + np * 4);
  uint64_t p = 0, pm = 0;
  for (unsigned ip = 0; ip < np; ++ip) {
    std::vector<unsigned> aIP;
    for (unsigned k = ind[ip]; k < ind[ip + 1]; ++k) aIP.push_back(psup[k]);
    aIP.push_back(ip);
    std::vector<double> eM, eR;
    dfm2::deflap::dWddW_ArapEnergy(eM, eR, precomp.data() + ip * 9, aIP, X0, X1, Q1);
    elem_ptr[ip] = (uint32_t)p;
    for (unsigned k = 0; k < aIP.size(); ++k) {
      elem_idx[p + k] = aIP[k];
      for (int d = 0; d < 3; ++d) eR_out[(p + k) * 3 + d] = eR[k * 3 + d];
    }
    std::memcpy(eM_out + pm, eM.data(), sizeof(double) * eM.size());
    p += aIP.size();
    pm += eM.size();
  }
  elem_ptr[np] = (uint32_t)p;
}

// One Deformer_Arap::Deform (ILU(0)-preconditioned): xyz1 updated in place
// (xyz1 -= update), hist the convergence history (absolute |r|).
uint32_t ref_arap_deform(uint32_t np, const double *xyz0, uint32_t ntri, const uint32_t *tri, double *xyz1,
                         double *quat1, const int *bcflag, double *hist, uint32_t hist_cap) {
  dfm2::Deformer_Arap def;
  const std::vector<double> X0(xyz0, xyz0 + np * 3);
  const std::vector<unsigned> T(tri, tri + ntri * 3);
  def.Init(X0, T, true);
  std::vector<double> X1(xyz1, xyz1 + np * 3), Q1(quat1, quat1 + np * 4);
  const std::vector<int> bc(bcflag, bcflag + np * 3);
  def.Deform(X1, Q1, X0, bc);
  std::memcpy(xyz1, X1.data(), sizeof(double) * np * 3);
  const uint32_t nh = (uint32_t)def.convergence_history.size();
  for (uint32_t k = 0; k < nh && k < hist_cap; ++k) hist[k] = def.convergence_history[k];
  return nh;
}

// The linear Laplacian deformer: its matrix pattern (1-ring extended to the
// 2-ring), the dual-Laplacian element of each point (DualLaplacianSymbolic_3x3,
// 9 n^2 entries), the ILU(20) pattern of that matrix, and one Deform from
// xyz_def with the given fixed DOFs (penalty weight_bc = 100, conv_tol 1e-5).
void ref_lap_sizes(uint32_t np, uint32_t ntri, const uint32_t *tri, uint64_t *n_pat, uint64_t *n_idx,
                   uint64_t *n_mat, uint64_t *n_ilu) {
  dfm2::CDef_LaplacianLinear def;
  std::vector<double> X0(np * 3, 0.0);
  for (unsigned i = 0; i < np * 3; ++i) X0[i] = (double)i;  // positions do not enter the pattern
  def.Init(X0, std::vector<unsigned>(tri, tri + ntri * 3), true);
  *n_pat = def.Mat.row_ptr_.size();
  *n_ilu = def.Prec.rowPtr.size();
  std::vector<unsigned> ind, psup;
  one_ring(ind, psup, np, ntri, tri);
  uint64_t a = 0, b = 0;
  for (unsigned ip = 0; ip < np; ++ip) {
    const uint64_t n = ind[ip + 1] - ind[ip] + 1;
    a += n;
    b += 9 * n * n;
  }
  *n_idx = a;
  *n_mat = b;
}

uint32_t ref_lap_deform(uint32_t np, const double *xyz0, uint32_t ntri, const uint32_t *tri, const int *bcflag,
                        double *xyz_def, uint32_t *pat_start, uint32_t *pat_col, uint32_t *elem_ptr,
                        uint32_t *elem_idx, double *eM_out, uint32_t *ilu_start, uint32_t *ilu_col, double *hist,
                        uint32_t hist_cap) {
  dfm2::CDef_LaplacianLinear def;
  const std::vector<double> X0(xyz0, xyz0 + np * 3);
  def.Init(X0, std::vector<unsigned>(tri, tri + ntri * 3), true);
  std::memcpy(pat_start, def.Mat.col_ind_.data(), sizeof(uint32_t) * (np + 1));
  std::memcpy(pat_col, def.Mat.row_ptr_.data(), sizeof(uint32_t) * def.Mat.row_ptr_.size());
  std::memcpy(ilu_start, def.Prec.colInd.data(), sizeof(uint32_t) * (np + 1));
  std::memcpy(ilu_col, def.Prec.rowPtr.data(), sizeof(uint32_t) * def.Prec.rowPtr.size());
  std::vector<unsigned> ind, psup;
  one_ring(ind, psup, np, ntri, tri);
  uint64_t p = 0, pm = 0;
  for (unsigned ip = 0; ip < np; ++ip) {
    std::vector<unsigned> aIP;
    for (unsigned k = ind[ip]; k < ind[ip + 1]; ++k) aIP.push_back(psup[k]);
    aIP.push_back(ip);
    std::vector<double> eM;
    dfm2::defarap::DualLaplacianSymbolic_3x3(eM, aIP);
    elem_ptr[ip] = (uint32_t)p;
    for (unsigned k = 0; k < aIP.size(); ++k) elem_idx[p + k] = aIP[k];
    std::memcpy(eM_out + pm, eM.data(), sizeof(double) * eM.size());
    p += aIP.size();
    pm += eM.size();
  }
  elem_ptr[np] = (uint32_t)p;
  def.aBCFlag.assign(bcflag, bcflag + np * 3);
  def.SetValueToPreconditioner();
  std::vector<double> Xd(xyz_def, xyz_def + np * 3);
  def.Deform(Xd, X0);
  std::memcpy(xyz_def, Xd.data(), sizeof(double) * np * 3);
  const uint32_t nh = (uint32_t)def.aConvHist.size();
  for (uint32_t k = 0; k < nh && k < hist_cap; ++k) hist[k] = def.aConvHist[k];
  return nh;
}

}  // extern "C"

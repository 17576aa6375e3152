// Cloth part of the reference driver (TEST INFRASTRUCTURE ONLY): the
// UNMODIFIED DelFEM2 cloth functions behind the C signatures of the plain-C
// restatement (dfm2_oracle.h, prefix ref_ instead of orc_). Compiled with
// ref_driver.cpp into oracle/_ref/libdfm2ref.so by oracle/Makefile.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

// ls_block_sparse.h must precede the element headers (their templates call Merge).
#include "delfem2/ls_block_sparse.h"
#include "delfem2/cloth_internal.h"
#include "delfem2/fem_quadratic_bending.h"
#include "delfem2/fem_stvk.h"
#include "delfem2/femcloth.h"
#include "delfem2/ls_ilu_block_sparse.h"
#include "delfem2/lsitrsol.h"
#include "delfem2/view_vectorx.h"

namespace {

class NoContact : public delfem2::CInput_Contact {
 public:
  double penetrationNormal(double &, double &, double &, double, double, double) const override { return -100; }
};

bool uniform(const double *v, size_t n) {
  for (size_t i = 1; i < n; ++i)
    if (v[i] != v[0]) return false;
  return true;
}

}  // namespace

extern "C" {

void ref_cloth_square(uint32_t ndiv, double size, double *xyz0, uint32_t *tri, uint32_t *quad) {
  std::vector<double> x;
  std::vector<int> bc;
  std::vector<unsigned int> t, q;
  SetClothShape_Square(x, bc, t, q, (int)ndiv, size);
  std::memcpy(xyz0, x.data(), sizeof(double) * x.size());
  std::memcpy(tri, t.data(), sizeof(unsigned) * t.size());
  std::memcpy(quad, q.data(), sizeof(unsigned) * q.size());
}

void ref_make_pd_sim22(const double s2[3], double s3[3]) { MakePositiveDefinite_Sim22(s2, s3); }

void ref_wdwddw_cst(const double C[3][3], const double c[3][3], double lambda, double myu, double *W,
                    double dW[3][3], double ddW[3][3][3][3]) {
  delfem2::WdWddW_CST(*W, dW, ddW, C, c, lambda, myu);
}

void ref_wdwddw_bend(const double C[4][3], const double c[4][3], double stiff, double *W, double dW[4][3],
                     double ddW[4][4][3][3]) {
  delfem2::WdWddW_Bend(*W, dW, ddW, C, c, stiff);
}

// MergeLinSys_Cloth itself when every triangle has the same modulus, else its
// loop with per-triangle (lambda, myu).
double ref_cloth_assemble(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                          double *vdia, double *dW, const double *xyz0, const double *xyz, const uint32_t *tri,
                          size_t ntri, const uint32_t *quad, size_t nquad, const double *young_tri, double nu,
                          double stiff_bend) {
  delfem2::CMatrixSparse<double> m;
  m.Initialize(nblk, 3, true);
  m.SetPattern(row_start, nblk + 1, col, row_start[nblk]);
  std::memcpy(m.val_crs_.data(), vcrs, sizeof(double) * 9 * row_start[nblk]);
  std::memcpy(m.val_dia_.data(), vdia, sizeof(double) * 9 * nblk);
  double W = 0;
  if (ntri == 0 || uniform(young_tri, ntri)) {
    const double E = ntri ? young_tri[0] : 0.0;
    W = delfem2::MergeLinSys_Cloth(m, dW, E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu)), stiff_bend,
                                   xyz0, nblk, 3, tri, (unsigned)ntri, quad, (unsigned)nquad, xyz);
  } else {
    std::vector<unsigned int> buf(nblk, UINT_MAX);
    for (size_t t = 0; t < ntri; ++t) {
      const unsigned int *ip = tri + t * 3;
      double C[3][3], c[3][3], e, de[3][3], dde[3][3][3][3];
      for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 3; ++d) {
          C[a][d] = xyz0[ip[a] * 3 + d];
          c[a][d] = xyz[ip[a] * 3 + d];
        }
      const double E = young_tri[t];
      delfem2::WdWddW_CST(e, de, dde, C, c, E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu)));
      W += e;
      for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 3; ++d) dW[ip[a] * 3 + d] += de[a][d];
      delfem2::Merge<3, 3, 3, 3, double>(m, ip, ip, dde, buf);
    }
    for (size_t q = 0; q < nquad; ++q) {
      const unsigned int *ip = quad + q * 4;
      double C[4][3], c[4][3], e, de[4][3], dde[4][4][3][3];
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) {
          C[a][d] = xyz0[ip[a] * 3 + d];
          c[a][d] = xyz[ip[a] * 3 + d];
        }
      delfem2::WdWddW_Bend(e, de, dde, C, c, stiff_bend);
      W += e;
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) dW[ip[a] * 3 + d] += de[a][d];
      delfem2::Merge<4, 4, 3, 3, double>(m, ip, ip, dde, buf);
    }
  }
  std::memcpy(vcrs, m.val_crs_.data(), sizeof(double) * 9 * row_start[nblk]);
  std::memcpy(vdia, m.val_dia_.data(), sizeof(double) * 9 * nblk);
  return W;
}

// StepTime_InternalDynamicsILU (cloth_internal.h:179-269) itself when the
// moduli are uniform and the solver settings are its own (1e-4, 100), else
// the same sequence with per-triangle moduli and the given tolerance.
uint32_t ref_cloth_step(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *xyz, double *uvw,
                        const double *xyz0, const int *bc, const uint32_t *tri, size_t ntri, const uint32_t *quad,
                        size_t nquad, const double *young_tri, double nu, double stiff_bend, const double g[3],
                        double mass, double dt, double tol, uint32_t max_iter) {
  const size_t n = (size_t)nblk * 3;
  delfem2::CMatrixSparse<double> m;
  m.Initialize(nblk, 3, true);
  m.SetPattern(row_start, nblk + 1, col, row_start[nblk]);
  delfem2::CPreconditionerILU<double> ilu;
  ilu.SetPattern0(m);
  std::vector<double> X(xyz, xyz + n), V(uvw, uvw + n), X0(xyz0, xyz0 + n);
  std::vector<int> BC(bc, bc + n);
  std::vector<unsigned int> T(tri, tri + ntri * 3), Q(quad, quad + nquad * 4);
  if (uniform(young_tri, ntri) && tol == 1.0e-4 && max_iter == 100) {
    const double E = young_tri[0];
    NoContact nc;
    StepTime_InternalDynamicsILU(X, V, m, ilu, X0, BC, T, Q, dt, E * nu / ((1 + nu) * (1 - 2 * nu)),
                                 E / (2 * (1 + nu)), stiff_bend, g, mass, 0.0, 0.0, nc);
    std::memcpy(xyz, X.data(), sizeof(double) * n);
    std::memcpy(uvw, V.data(), sizeof(double) * n);
    return 0;
  }
  std::vector<double> b(n, 0.0);
  m.setZero();
  {
    std::vector<double> vc(m.val_crs_.size(), 0.0), vd(m.val_dia_.size(), 0.0);
    ref_cloth_assemble(nblk, row_start, col, vc.data(), vd.data(), b.data(), xyz0, xyz, tri, ntri, quad, nquad,
                       young_tri, nu, stiff_bend);
    m.val_crs_ = vc;
    m.val_dia_ = vd;
  }
  AddWdW_Gravity(b, X, g, mass);
  for (size_t i = 0; i < n; ++i) b[i] = -b[i] + mass * V[i] / dt;
  for (uint32_t ip = 0; ip < nblk; ++ip)
    for (int d = 0; d < 3; ++d) m.val_dia_[ip * 9 + d * 4] += mass / (dt * dt);
  m.SetFixedBC(bc);
  for (size_t i = 0; i < n; ++i)
    if (bc[i] != 0) b[i] = 0.0;
  ilu.CopyValue(m);
  ilu.Decompose();
  std::vector<double> dx(n), t0(n), t1(n);
  auto hist = delfem2::Solve_PCG(delfem2::ViewAsVectorXd(b), delfem2::ViewAsVectorXd(dx),
                                 delfem2::ViewAsVectorXd(t0), delfem2::ViewAsVectorXd(t1), tol, max_iter, m, ilu);
  for (size_t i = 0; i < n; ++i) {
    if (bc[i] != 0) continue;
    xyz[i] += dx[i];
    uvw[i] = dx[i] / dt;
  }
  return static_cast<uint32_t>(hist.size());
}

}  // extern "C"

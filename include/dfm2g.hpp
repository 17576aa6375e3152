// dfm2g.hpp — C++ drop-in over the dfm2g C ABI for DelFEM2 callers.
//
// Mirrors the reference types a caller uses on the implicit-FEM solve path,
// in namespace delfem2::gb300, with the reference's member names:
//   CMatrixSparse<double>      include/delfem2/ls_block_sparse.h:24-204
//   Merge<nrow,ncol,3,3,double> include/delfem2/ls_block_sparse.h:260-310
//   CPreconditionerILU<double> include/delfem2/ls_ilu_block_sparse.h:21-60
//   Solve_PCG                  include/delfem2/lsitrsol.h:80-148
// Storage is on the GPU; vectors passed by the caller are host memory (as in
// the reference) unless a member says otherwise. Only 3x3 blocks.
// Two ways to solve: Solve_PCG below runs the whole iteration on the device
// (fast path); DeviceVectorView lets the reference's own Solve_PCG template
// drive device vectors through the ADL primitives (compatibility path).
#pragma once

#include <climits>
#include <stdexcept>
#include <string>
#include <vector>

#include "dfm2g.h"

namespace delfem2 {
namespace gb300 {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string &what) : std::runtime_error(what), status(status) {}
  int status;
};

inline void check(int s, const char *where) {
  if (s != DFM2G_OK) throw Error(s, std::string(where) + ": " + dfm2g_last_error());
}

template <typename T>
class CMatrixSparse;

template <>
class CMatrixSparse<double> {
 public:
  CMatrixSparse() = default;
  CMatrixSparse(const CMatrixSparse &) = delete;
  CMatrixSparse &operator=(const CMatrixSparse &) = delete;
  ~CMatrixSparse() { dfm2g_bsr_destroy(h_); }

  void Initialize(size_t nblk, unsigned int len, bool is_dia) {
    if (!is_dia) throw Error(DFM2G_ERR_UNSUPPORTED, "Initialize: is_dia must be true");
    dfm2g_bsr_destroy(h_);
    h_ = nullptr;
    check(dfm2g_bsr_create(&h_, (unsigned)nblk, len), "Initialize");
    nrowblk_ = ncolblk_ = (unsigned)nblk;
    nrowdim_ = ncoldim_ = len;
  }
  void SetPattern(const unsigned int *colind, size_t ncolind, const unsigned int *rowptr, size_t nrowptr) {
    check(dfm2g_bsr_set_pattern(h_, colind, ncolind, rowptr, nrowptr), "SetPattern");
  }
  bool setZero() {
    check(dfm2g_bsr_set_zero(h_), "setZero");
    return true;
  }
  void MatVec(double *y, double alpha, const double *x, double beta) const {
    check(dfm2g_bsr_matvec(h_, DFM2G_F64, y, alpha, x, beta, DFM2G_MEM_HOST), "MatVec");
  }
  void SetFixedBC(const int *bc_flag) { check(dfm2g_bsr_set_fixed_bc(h_, bc_flag, DFM2G_MEM_HOST), "SetFixedBC"); }
  void AddDia(double eps) { check(dfm2g_bsr_add_dia(h_, eps), "AddDia"); }
  // Batched Merge: nelem elements of nno nodes, emat row-major [e][irow][jcol][ndim][ndim].
  void MergeBatch(unsigned nelem, unsigned nno, const unsigned *elem, const double *emat) {
    check(dfm2g_bsr_merge(h_, nelem, nno, elem, emat, DFM2G_MEM_HOST), "Merge");
  }
  dfm2g_bsr handle() const { return h_; }

  unsigned int nrowblk_ = 0, ncolblk_ = 0, nrowdim_ = 0, ncoldim_ = 0;

 private:
  dfm2g_bsr h_ = nullptr;
};

// Merge<nrow,ncol,ndim,ndim,double> (ls_block_sparse.h:260-310) and the
// scalar Merge<nrow,ncol,double> (313-358) for one element (aIpRow == aIpCol,
// as every FEM caller passes). One call is one device launch: callers merging
// many elements should collect them and use CMatrixSparse::MergeBatch.
template <int nrow, int ncol, int ndimrow, int ndimcol, typename T>
bool Merge(CMatrixSparse<T> &A, const unsigned int aIpRow[nrow], const unsigned int aIpCol[ncol],
           const T emat[nrow][ncol][ndimrow][ndimcol], std::vector<unsigned int> &merge_buffer) {
  static_assert(nrow == ncol && ndimrow == ndimcol, "square element matrices of square blocks");
  (void)merge_buffer;
  if (A.nrowdim_ != (unsigned)ndimrow) throw Error(DFM2G_ERR_ARG, "Merge: block size differs from the matrix's");
  for (int i = 0; i < nrow; ++i)
    if (aIpRow[i] != aIpCol[i]) throw Error(DFM2G_ERR_UNSUPPORTED, "Merge: aIpRow must equal aIpCol");
  const int s = dfm2g_bsr_merge(A.handle(), 1, nrow, aIpRow, &emat[0][0][0][0], DFM2G_MEM_HOST);
  if (s == DFM2G_ERR_MISSING_SLOT) return false;
  check(s, "Merge");
  return true;
}

template <int nrow, int ncol, typename T>
bool Merge(CMatrixSparse<T> &A, const unsigned int *aIpRow, const unsigned int *aIpCol, const T emat[nrow][ncol],
           std::vector<unsigned int> &merge_buffer) {
  static_assert(nrow == ncol, "square element matrices");
  (void)merge_buffer;
  if (A.nrowdim_ != 1) throw Error(DFM2G_ERR_ARG, "Merge: scalar element matrix on a block matrix");
  for (int i = 0; i < nrow; ++i)
    if (aIpRow[i] != aIpCol[i]) throw Error(DFM2G_ERR_UNSUPPORTED, "Merge: aIpRow must equal aIpCol");
  const int s = dfm2g_bsr_merge(A.handle(), 1, nrow, aIpRow, &emat[0][0], DFM2G_MEM_HOST);
  if (s == DFM2G_ERR_MISSING_SLOT) return false;
  check(s, "Merge");
  return true;
}

template <typename T>
class CPreconditionerILU;

template <>
class CPreconditionerILU<double> {
 public:
  CPreconditionerILU() { check(dfm2g_ilu_create(&h_), "CPreconditionerILU"); }
  CPreconditionerILU(const CPreconditionerILU &) = delete;
  CPreconditionerILU &operator=(const CPreconditionerILU &) = delete;
  ~CPreconditionerILU() { dfm2g_ilu_destroy(h_); }

  void SetPattern0(const CMatrixSparse<double> &m) { check(dfm2g_ilu_set_pattern0(h_, m.handle()), "SetPattern0"); }
  void Initialize_ILUk(const CMatrixSparse<double> &m, int fill_level) {
    check(dfm2g_ilu_set_pattern_k(h_, m.handle(), fill_level), "Initialize_ILUk");
  }
  void CopyValue(const CMatrixSparse<double> &m) { check(dfm2g_ilu_copy_value(h_, m.handle()), "CopyValue"); }
  bool Decompose() {
    int ns = 0;
    const int s = dfm2g_ilu_decompose(h_, &ns);
    if (s == DFM2G_ERR_SINGULAR_PIVOT) return false;
    check(s, "Decompose");
    return true;
  }
  void ForwardSubstitution(double *vec) const {
    check(dfm2g_ilu_forward(h_, DFM2G_F64, vec, DFM2G_MEM_HOST), "ForwardSubstitution");
  }
  void BackwardSubstitution(double *vec) const {
    check(dfm2g_ilu_backward(h_, DFM2G_F64, vec, DFM2G_MEM_HOST), "BackwardSubstitution");
  }
  void SolvePrecond(double *vec) const {
    check(dfm2g_ilu_solve_precond(h_, DFM2G_F64, vec, DFM2G_MEM_HOST), "SolvePrecond");
  }
  dfm2g_ilu handle() const { return h_; }

 private:
  dfm2g_ilu h_ = nullptr;
};

// Non-owning host vector view, the role ViewAsVectorX plays (view_vectorx.h:26-55).
struct VectorView {
  double *p;
  size_t n;
  VectorView(double *p_, size_t n_) : p(p_), n(n_) {}
  VectorView(std::vector<double> &v) : p(v.data()), n(v.size()) {}
};

// Solve_PCG(r, x, Pr, p, tol, max_iter, K, ilu): same arguments and result
// (absolute residual history) as the reference; the whole iteration runs on
// the GPU, so Pr and p are not used as scratch.
inline std::vector<double> Solve_PCG(VectorView r_vec, VectorView x_vec, VectorView /*Pr_vec*/,
                                     VectorView /*p_vec*/, double conv_ratio_tol, unsigned int max_nitr,
                                     const CMatrixSparse<double> &mat, const CPreconditionerILU<double> &ilu) {
  std::vector<double> hist(max_nitr + 2);
  unsigned n = 0;
  const int s = dfm2g_solve_pcg(mat.handle(), ilu.handle(), r_vec.p, x_vec.p, conv_ratio_tol, max_nitr, hist.data(),
                                (unsigned)hist.size(), &n, DFM2G_MEM_HOST, nullptr);
  if (s != DFM2G_ERR_NOT_CONVERGED) check(s, "Solve_PCG");
  hist.resize(n < hist.size() ? n : hist.size());
  return hist;
}

// Solve_PBiCGStab(r, x, tol, max_niter, K, ilu), vecxitrsol.h:350-437: same
// arguments and result (RELATIVE residual per iteration); runs on the GPU.
inline std::vector<double> Solve_PBiCGStab(double *r_vec, double *x_vec, double conv_ratio_tol,
                                           unsigned int max_niter, const CMatrixSparse<double> &mat,
                                           const CPreconditionerILU<double> &ilu) {
  std::vector<double> hist(max_niter + 2);
  unsigned n = 0;
  const int s = dfm2g_solve_pbicgstab(mat.handle(), ilu.handle(), r_vec, x_vec, conv_ratio_tol, max_niter,
                                      hist.data(), (unsigned)hist.size(), &n, DFM2G_MEM_HOST, nullptr);
  if (s != DFM2G_ERR_NOT_CONVERGED) check(s, "Solve_PBiCGStab");
  hist.resize(n < hist.size() ? n : hist.size());
  return hist;
}

// Compatibility path: a non-owning view of a device vector with the members
// and ADL primitives the reference's generic Solve_PCG<MAT, VEC, PREC>
// (lsitrsol.h:80-148) calls (view_vectorx.h:26-109), so that template runs
// unchanged on GPU-resident vectors; each Dot returns to the host. Copy
// construction copies the view, assignment copies the contents (as the
// reference's `Pr_vec = r_vec`).
struct DeviceVectorView {
  double *p;
  size_t n;
  DeviceVectorView(double *p_, size_t n_) : p(p_), n(n_) {}
  DeviceVectorView(const DeviceVectorView &) = default;
  DeviceVectorView &operator=(const DeviceVectorView &o) {
    if (o.n != n) throw Error(DFM2G_ERR_ARG, "DeviceVectorView: size mismatch");
    if (o.p != p) check(dfm2g_dev_copy(p, o.p, sizeof(double) * n, DFM2G_COPY_D2D), "operator=");
    return *this;
  }
  void setZero() { check(dfm2g_vec_set_zero(p, n, DFM2G_MEM_DEVICE), "setZero"); }
};

inline double Dot(const DeviceVectorView &x, const DeviceVectorView &y) {
  double d = 0.0;
  check(dfm2g_vec_dot(x.p, y.p, x.n, &d, DFM2G_MEM_DEVICE), "Dot");
  return d;
}
inline void AddScaledVec(DeviceVectorView &y, double alpha, const DeviceVectorView &x) {
  check(dfm2g_vec_axpy(y.p, alpha, x.p, y.n, DFM2G_MEM_DEVICE), "AddScaledVec");
}
inline void ScaleAndAddVec(DeviceVectorView &y, double beta, const DeviceVectorView &x) {
  check(dfm2g_vec_scale_add(y.p, beta, x.p, y.n, DFM2G_MEM_DEVICE), "ScaleAndAddVec");
}
// lhs = scale_lhs * lhs + scale_rhs * mat * rhs
inline void AddMatVec(DeviceVectorView &lhs, double scale_lhs, double scale_rhs, const CMatrixSparse<double> &mat,
                      const DeviceVectorView &rhs) {
  check(dfm2g_bsr_matvec(mat.handle(), DFM2G_F64, lhs.p, scale_rhs, rhs.p, scale_lhs, DFM2G_MEM_DEVICE),
        "AddMatVec");
}
inline void SolvePrecond(DeviceVectorView &v, const CPreconditionerILU<double> &ilu) {
  check(dfm2g_ilu_solve_precond(ilu.handle(), DFM2G_F64, v.p, DFM2G_MEM_DEVICE), "SolvePrecond");
}

// Owning device buffer for callers without CUDA of their own.
class DeviceVector {
 public:
  explicit DeviceVector(size_t n) : n_(n) { check(dfm2g_dev_alloc((void **)&p_, sizeof(double) * n), "alloc"); }
  DeviceVector(const DeviceVector &) = delete;
  DeviceVector &operator=(const DeviceVector &) = delete;
  ~DeviceVector() { dfm2g_dev_free(p_); }
  DeviceVectorView view() { return DeviceVectorView(p_, n_); }
  void upload(const double *h) { check(dfm2g_dev_copy(p_, h, sizeof(double) * n_, DFM2G_COPY_H2D), "upload"); }
  void download(double *h) const { check(dfm2g_dev_copy(h, p_, sizeof(double) * n_, DFM2G_COPY_D2H), "download"); }

 private:
  double *p_ = nullptr;
  size_t n_;
};

// The FP32-inner / FP64-refinement variant (no reference counterpart).
inline dfm2g_solve_stats Solve_PCG_Mixed(const double *b, double *x, double tol, const CMatrixSparse<double> &mat,
                                         const CPreconditionerILU<double> &ilu, double inner_tol = 1e-4) {
  dfm2g_solve_stats st{};
  check(dfm2g_solve_pcg_mixed(mat.handle(), ilu.handle(), b, x, tol, inner_tol, 1000000u, 1000u, DFM2G_MEM_HOST,
                              &st),
        "Solve_PCG_Mixed");
  return st;
}

}  // namespace gb300
}  // namespace delfem2

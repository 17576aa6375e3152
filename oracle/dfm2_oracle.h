/*
 * CPU oracle for the 3x3 block-CSR assembly -> ILU(0) -> PCG path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of DelFEM2's serial
 * algorithms, used by the tests, by __graft_entry__.smoke() and by bench.py's
 * CPU-baseline leg as the checker. The product library (delfem2_gb300) never
 * links, loads or calls it.
 *
 * Index naming follows DelFEM2's CMatrixSparse: `row_start` is what the
 * reference calls col_ind_ (size nblk+1, row offsets) and `col` is what it
 * calls row_ptr_ (column id per off-diagonal block). Diagonal blocks live in a
 * separate array `vdia` (nblk * 9), off-diagonal blocks in `vcrs` (nnz * 9),
 * both row-major 3x3.
 */
#ifndef DFM2_ORACLE_H
#define DFM2_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* --- mesh + pattern --------------------------------------------------- */
void orc_voxel_tet_mesh(uint32_t nx, uint32_t ny, uint32_t nz, double scale,
                        double *xyz, uint32_t *tet);
size_t orc_psup_count(const uint32_t *elem, size_t nelem, uint32_t nnoel,
                      size_t np, uint32_t *psup_ind);
void orc_psup_fill(const uint32_t *elem, size_t nelem, uint32_t nnoel,
                   size_t np, const uint32_t *psup_ind, uint32_t *psup);

/* --- block sparse matrix ---------------------------------------------- */
void orc_bsr_matvec(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                    const double *vcrs, const double *vdia,
                    double *y, double alpha, const double *x, double beta);
void orc_bsr_matvec_f32(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                        const float *vcrs, const float *vdia,
                        float *y, float alpha, const float *x, float beta);
int orc_merge(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
              double *vcrs, double *vdia, uint32_t nnoel, const uint32_t *nodes,
              const double *emat, uint32_t *merge_buffer);
void orc_set_fixed_bc(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      double *vcrs, double *vdia, const int *bc);
void orc_rhs_zero(double *b, const int *bc, size_t ndof);

/* --- linear-tet elasticity -------------------------------------------- */
void orc_emat_tet_linear(const double P[4][3], double myu, double lambda,
                         double emat[4][4][3][3], double *vol_out);
int orc_assemble_tet_linear(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                            double *vcrs, double *vdia, double *b,
                            const double *xyz, const uint32_t *tet, size_t ntet,
                            const double *young, double nu, double rho,
                            const double g[3], const double *disp);
void orc_tet_dLdE(const double *xyz, const uint32_t *tet, size_t ntet,
                  const double *young, double nu, const double *u,
                  const double *lam, double *dLdE);

/* --- ILU(0) -------------------------------------------------------------- */
void orc_ilu_pattern0(uint32_t nblk, const uint32_t *row_start, const uint32_t *col_in,
                      uint32_t *col_out, uint32_t *dia_ind);
void orc_ilu_copy_value(uint32_t nblk, const uint32_t *row_start, const uint32_t *col_ilu,
                        double *ilu_vcrs, double *ilu_vdia,
                        const uint32_t *col_mat, const double *mat_vcrs,
                        const double *mat_vdia);
int orc_ilu_decompose(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      const uint32_t *dia_ind, double *vcrs, double *vdia,
                      int *n_singular);
void orc_ilu_forward(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                     const uint32_t *dia_ind, const double *vcrs, const double *vdia,
                     double *vec);
void orc_ilu_backward(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      const uint32_t *dia_ind, const double *vcrs, double *vec);
uint32_t orc_ilu_levels(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                        const uint32_t *dia_ind, int backward, uint32_t *level,
                        uint32_t *order, uint32_t *level_start);

/* --- Krylov ------------------------------------------------------------ */
uint32_t orc_solve_pcg(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                       const double *vcrs, const double *vdia,
                       const uint32_t *ilu_col, const uint32_t *dia_ind,
                       const double *ilu_vcrs, const double *ilu_vdia,
                       double *r, double *x, double tol, uint32_t max_iter,
                       double *hist, uint32_t hist_cap);
uint32_t orc_solve_cg(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      const double *vcrs, const double *vdia, double *r, double *x,
                      double tol, uint32_t max_iter, double *hist, uint32_t hist_cap);
uint32_t orc_solve_pcg_k(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                         const double *vcrs, const double *vdia, const uint32_t *ilu_row_start,
                         const uint32_t *ilu_col, const uint32_t *dia_ind,
                         const double *ilu_vcrs, const double *ilu_vdia,
                         double *r, double *x, double tol, uint32_t max_iter,
                         double *hist, uint32_t hist_cap);
uint32_t orc_solve_pbicgstab(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, const double *vcrs,
                             const double *vdia, const uint32_t *ilu_row_start, const uint32_t *ilu_col,
                             const uint32_t *dia_ind, const double *ilu_vcrs, const double *ilu_vdia, double *r,
                             double *x, double tol, uint32_t max_iter, double *hist, uint32_t hist_cap);
double orc_dot(const double *a, const double *b, size_t n);

/* --- cloth ------------------------------------------------------------- */
void orc_cloth_square(uint32_t ndiv, double size, double *xyz0, uint32_t *tri, uint32_t *quad);
void orc_make_pd_sim22(const double s2[3], double s3[3]);
void orc_wdwddw_cst(const double C[3][3], const double c[3][3], double lambda, double myu, double *W,
                    double dW[3][3], double ddW[3][3][3][3]);
void orc_wdwddw_bend(const double C[4][3], const double c[4][3], double stiff, double *W, double dW[4][3],
                     double ddW[4][4][3][3]);
double orc_cloth_assemble(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                          double *vdia, double *dW, const double *xyz0, const double *xyz, const uint32_t *tri,
                          size_t ntri, const uint32_t *quad, size_t nquad, const double *young_tri, double nu,
                          double stiff_bend);
uint32_t orc_cloth_step(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *xyz, double *uvw,
                        const double *xyz0, const int *bc, const uint32_t *tri, size_t ntri, const uint32_t *quad,
                        size_t nquad, const double *young_tri, double nu, double stiff_bend, const double g[3],
                        double mass, double dt, double tol, uint32_t max_iter);
size_t orc_ilu_pattern_k(uint32_t nblk, const uint32_t *row_start, const uint32_t *col_in, int lev_fill,
                         uint32_t *row_start_out, uint32_t *col_out, size_t cap, uint32_t *dia_ind);
void orc_ilu_copy_value_k(uint32_t nblk, const uint32_t *mrow_start, const uint32_t *col_mat,
                          const double *mat_vcrs, const double *mat_vdia, int lev_fill,
                          const uint32_t *irow_start, const uint32_t *col_ilu, double *ilu_vcrs,
                          double *ilu_vdia);
void orc_pd_sim22_jac(const double s2[3], double J[3][3]);
void orc_cloth_adjoint_terms(const double *xyz0, const double *xyz, const uint32_t *tri, size_t ntri,
                             const uint32_t *quad, size_t nquad, const double *young_tri, double nu,
                             double stiff_bend, const double *mu, const double *dx, double *xbar, double *Ebar);

/* --- scalar (ndim 1) and 2x2 (ndim 2) blocks; ndim 3 runs the 3x3 code ---- */
void orc_nd_matvec(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                   const double *vcrs, const double *vdia, double *y, double alpha, const double *x,
                   double beta);
int orc_nd_merge(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                 double *vdia, uint32_t nnoel, const uint32_t *nodes, const double *emat, uint32_t *merge_buffer);
void orc_nd_set_fixed_bc(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                         double *vcrs, double *vdia, const int *bc);
void orc_nd_ilu_copy_value(uint32_t nblk, uint32_t ndim, const uint32_t *mrow_start, const uint32_t *col_mat,
                           const double *mat_vcrs, const double *mat_vdia, int lev_fill,
                           const uint32_t *irow_start, const uint32_t *col_ilu, double *ilu_vcrs,
                           double *ilu_vdia);
int orc_nd_ilu_decompose(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                         const uint32_t *dia_ind, double *vcrs, double *vdia, int *n_singular);
void orc_nd_ilu_forward(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                        const uint32_t *dia_ind, const double *vcrs, const double *vdia, double *vec);
void orc_nd_ilu_backward(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                         const uint32_t *dia_ind, const double *vcrs, double *vec);
uint32_t orc_nd_solve_pcg(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                          const double *vcrs, const double *vdia, const uint32_t *ilu_row_start,
                          const uint32_t *ilu_col, const uint32_t *dia_ind, const double *ilu_vcrs,
                          const double *ilu_vdia, double *r, double *x, double tol, uint32_t max_iter,
                          double *hist, uint32_t hist_cap);
uint32_t orc_nd_solve_pbicgstab(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                                const double *vcrs, const double *vdia, const uint32_t *ilu_row_start,
                                const uint32_t *ilu_col, const uint32_t *dia_ind, const double *ilu_vcrs,
                                const double *ilu_vdia, double *r, double *x, double tol, uint32_t max_iter,
                                double *hist, uint32_t hist_cap);
void orc_emat_poisson_tet(const double P[4][3], double alpha, double source, const double value[4],
                          double emat[4][4], double eres[4]);
int orc_assemble_poisson_tet(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                             double *vdia, double *b, double alpha, double source, const double *xyz,
                             const uint32_t *tet, size_t ntet, const double *val);
void orc_emat_poisson_tri2(const double P[3][2], double alpha, double source, const double value[3],
                           double emat[3][3], double eres[3]);
void orc_emat_solid_tri2(const double P[3][2], double myu, double lambda, double rho, double gx, double gy,
                         const double disp[3][2], double emat[3][3][2][2], double eres[3][2]);
int orc_assemble_tri2(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                      double *vdia, double *b, const double *param, const double *xy, const uint32_t *tri,
                      size_t ntri, const double *val);

/* --- dynamic linear tets ------------------------------------------------ */
int orc_assemble_tet_beuler(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                            double *vdia, double *b, double myu, double lambda, double rho, const double g[3],
                            double dt, const double *xyz, const uint32_t *tet, size_t ntet, const double *disp,
                            const double *velo, const double *rot);
int orc_assemble_tet_newmark(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                             double *vdia, double *b, double myu, double lambda, double rho, const double g[3],
                             double dt, double gamma, double beta, const double *xyz, const uint32_t *tet,
                             size_t ntet, const double *disp, const double *velo, const double *acc);

/* --- trilinear hexahedra (Q1) ------------------------------------------- */
void orc_emat_hex_q1(const double P[8][3], double myu, double lambda, double rho, const double g[3],
                     const double disp[8][3], double emat[8][8][3][3], double eres[8][3]);
int orc_assemble_hex_q1(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs, double *vdia,
                        double *b, double myu, double lambda, double rho, const double g[3], const double *xyz,
                        const uint32_t *hex, size_t nhex, const double *disp);

#ifdef __cplusplus
}
#endif
#endif

/*
 * CPU oracle for DelFEM2's 3x3 block-CSR assembly -> ILU(0) -> PCG path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product): a plain-C
 * restatement of the reference's serial algorithms. Each function names the
 * reference file:line it follows (paths relative to the DelFEM2 source tree).
 * Its results are pinned against the reference itself (oracle/ref_driver.cpp,
 * built from the unmodified reference headers) by tests/test_oracle_*.py and
 * by the committed fixtures under tests/golden/.
 */
#include "dfm2_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_UNSET 0xFFFFFFFFu

/* ---------------------------------------------------------------------- */
/* Mesh: include/delfem2/gridvoxel.cpp:194-271 (MeshTet3D_VoxelGrid with   */
/* every voxel active). Lattice node (ix,iy,iz) has id                      */
/* ix*(ny+1)*(nz+1) + iy*(nz+1) + iz and integer coordinates; `scale`       */
/* multiplies them (1/n maps the lattice onto the unit cube). Each voxel is */
/* split into six tets around its 0-6 diagonal, in the reference's order.   */
void orc_voxel_tet_mesh(uint32_t nx, uint32_t ny, uint32_t nz, double scale,
                        double *xyz, uint32_t *tet) {
  const uint32_t my = ny + 1, mz = nz + 1;
  size_t ip = 0;
  for (uint32_t ix = 0; ix <= nx; ++ix)
    for (uint32_t iy = 0; iy <= ny; ++iy)
      for (uint32_t iz = 0; iz <= nz; ++iz) {
        xyz[ip * 3 + 0] = (double)ix * scale;
        xyz[ip * 3 + 1] = (double)iy * scale;
        xyz[ip * 3 + 2] = (double)iz * scale;
        ++ip;
      }
  /* corner k of the voxel -> (dx,dy,dz) */
  static const uint32_t corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                        {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  static const int split[6][4] = {{0, 1, 2, 6}, {0, 1, 6, 5}, {0, 4, 5, 6},
                                  {0, 2, 3, 6}, {0, 3, 7, 6}, {0, 4, 6, 7}};
  size_t it = 0;
  for (uint32_t vx = 0; vx < nx; ++vx)
    for (uint32_t vy = 0; vy < ny; ++vy)
      for (uint32_t vz = 0; vz < nz; ++vz) {
        uint32_t id[8];
        for (int k = 0; k < 8; ++k)
          id[k] = (vx + corner[k][0]) * my * mz + (vy + corner[k][1]) * mz + (vz + corner[k][2]);
        for (int s = 0; s < 6; ++s) {
          for (int k = 0; k < 4; ++k) tet[it * 4 + k] = id[split[s][k]];
          ++it;
        }
      }
}

/* ---------------------------------------------------------------------- */
/* Pattern: node-to-node adjacency excluding self,                          */
/* include/delfem2/msh_topology_uniform.cpp:19-51 (elements around a point), */
/* 250-299 (one-ring with a marker array, self marked first at 262) and     */
/* 301-316 (the composition); rows then sorted ascending as                 */
/* include/delfem2/jagarray.cpp:72-92 does (its bubble sort and the         */
/* insertion sort here give the same order: the ids in a row are distinct). */
static void orc_elsup(const uint32_t *elem, size_t nelem, uint32_t nnoel, size_t np,
                      uint32_t **ind_out, uint32_t **elsup_out) {
  uint32_t *ind = (uint32_t *)calloc(np + 1, sizeof(uint32_t));
  for (size_t e = 0; e < nelem; ++e)
    for (uint32_t k = 0; k < nnoel; ++k) ind[elem[e * nnoel + k] + 1] += 1;
  for (size_t p = 0; p < np; ++p) ind[p + 1] += ind[p];
  uint32_t *cursor = (uint32_t *)malloc((np + 1) * sizeof(uint32_t));
  memcpy(cursor, ind, (np + 1) * sizeof(uint32_t));
  uint32_t *elsup = (uint32_t *)malloc((size_t)ind[np] * sizeof(uint32_t) + 1);
  for (size_t e = 0; e < nelem; ++e)
    for (uint32_t k = 0; k < nnoel; ++k) elsup[cursor[elem[e * nnoel + k]]++] = (uint32_t)e;
  free(cursor);
  *ind_out = ind;
  *elsup_out = elsup;
}

size_t orc_psup_count(const uint32_t *elem, size_t nelem, uint32_t nnoel, size_t np,
                      uint32_t *psup_ind) {
  uint32_t *eind, *elsup;
  orc_elsup(elem, nelem, nnoel, np, &eind, &elsup);
  uint32_t *mark = (uint32_t *)malloc(np * sizeof(uint32_t));
  for (size_t p = 0; p < np; ++p) mark[p] = ORC_UNSET;
  psup_ind[0] = 0;
  for (size_t p = 0; p < np; ++p) {
    uint32_t cnt = 0;
    mark[p] = (uint32_t)p;
    for (uint32_t q = eind[p]; q < eind[p + 1]; ++q) {
      const uint32_t e = elsup[q];
      for (uint32_t k = 0; k < nnoel; ++k) {
        const uint32_t n = elem[(size_t)e * nnoel + k];
        if (mark[n] != p) { mark[n] = (uint32_t)p; ++cnt; }
      }
    }
    psup_ind[p + 1] = psup_ind[p] + cnt;
  }
  free(mark);
  free(eind);
  free(elsup);
  return psup_ind[np];
}

void orc_psup_fill(const uint32_t *elem, size_t nelem, uint32_t nnoel, size_t np,
                   const uint32_t *psup_ind, uint32_t *psup) {
  uint32_t *eind, *elsup;
  orc_elsup(elem, nelem, nnoel, np, &eind, &elsup);
  uint32_t *mark = (uint32_t *)malloc(np * sizeof(uint32_t));
  for (size_t p = 0; p < np; ++p) mark[p] = ORC_UNSET;
  for (size_t p = 0; p < np; ++p) {
    uint32_t w = psup_ind[p];
    mark[p] = (uint32_t)p;
    for (uint32_t q = eind[p]; q < eind[p + 1]; ++q) {
      const uint32_t e = elsup[q];
      for (uint32_t k = 0; k < nnoel; ++k) {
        const uint32_t n = elem[(size_t)e * nnoel + k];
        if (mark[n] != p) { mark[n] = (uint32_t)p; psup[w++] = n; }
      }
    }
    /* ascending order inside the row (jagarray.cpp:72-92) */
    for (uint32_t a = psup_ind[p] + 1; a < psup_ind[p + 1]; ++a) {
      const uint32_t v = psup[a];
      uint32_t b = a;
      while (b > psup_ind[p] && psup[b - 1] > v) { psup[b] = psup[b - 1]; --b; }
      psup[b] = v;
    }
  }
  free(mark);
  free(eind);
  free(elsup);
}

/* ---------------------------------------------------------------------- */
/* y = alpha*K*x + beta*y, include/delfem2/ls_block_sparse.cpp:215-223 (y is */
/* scaled by beta first, even for beta == 0, so a NaN in y survives) and    */
/* the 3x3 kernel at 103-133 (off-diagonal blocks, then the diagonal).       */
void orc_bsr_matvec(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                    const double *vcrs, const double *vdia,
                    double *y, double alpha, const double *x, double beta) {
  for (size_t i = 0; i < (size_t)nblk * 3; ++i) y[i] *= beta;
  for (uint32_t i = 0; i < nblk; ++i) {
    double *yi = y + (size_t)i * 3;
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) {
      const double *a = vcrs + (size_t)s * 9;
      const double *xj = x + (size_t)col[s] * 3;
      for (int r = 0; r < 3; ++r)
        yi[r] += alpha * (a[r * 3 + 0] * xj[0] + a[r * 3 + 1] * xj[1] + a[r * 3 + 2] * xj[2]);
    }
    const double *d = vdia + (size_t)i * 9;
    const double *xi = x + (size_t)i * 3;
    for (int r = 0; r < 3; ++r)
      yi[r] += alpha * (d[r * 3 + 0] * xi[0] + d[r * 3 + 1] * xi[1] + d[r * 3 + 2] * xi[2]);
  }
}

/* CMatrixSparse<float>::MatVec, the same loops in single precision         */
/* (explicit float instantiation at ls_block_sparse.cpp:274-282).           */
void orc_bsr_matvec_f32(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                        const float *vcrs, const float *vdia,
                        float *y, float alpha, const float *x, float beta) {
  for (size_t i = 0; i < (size_t)nblk * 3; ++i) y[i] *= beta;
  for (uint32_t i = 0; i < nblk; ++i) {
    float *yi = y + (size_t)i * 3;
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) {
      const float *a = vcrs + (size_t)s * 9;
      const float *xj = x + (size_t)col[s] * 3;
      for (int r = 0; r < 3; ++r)
        yi[r] += alpha * (a[r * 3 + 0] * xj[0] + a[r * 3 + 1] * xj[1] + a[r * 3 + 2] * xj[2]);
    }
    const float *d = vdia + (size_t)i * 9;
    const float *xi = x + (size_t)i * 3;
    for (int r = 0; r < 3; ++r)
      yi[r] += alpha * (d[r * 3 + 0] * xi[0] + d[r * 3 + 1] * xi[1] + d[r * 3 + 2] * xi[2]);
  }
}

/* ---------------------------------------------------------------------- */
/* Merge<nno,nno,3,3,double>, include/delfem2/ls_block_sparse.h:260-310:    */
/* for each element row, mark the row's columns with their slots in          */
/* merge_buffer, add the (irow,jcol) 3x3 block to the marked slot, or, when  */
/* both nodes are the same block, the (irow,irow) block to the diagonal (as */
/* the reference does; it differs only for an element that repeats a node), */
/* then reset the marks. Returns 0, or 1 on a missing slot (the reference    */
/* returns false there).                                                     */
int orc_merge(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
              double *vcrs, double *vdia, uint32_t nnoel, const uint32_t *nodes,
              const double *emat, uint32_t *merge_buffer) {
  (void)nblk;
  for (uint32_t a = 0; a < nnoel; ++a) {
    const uint32_t i = nodes[a];
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) merge_buffer[col[s]] = s;
    for (uint32_t b = 0; b < nnoel; ++b) {
      const uint32_t j = nodes[b];
      const double *src = emat + ((size_t)a * nnoel + (i == j ? a : b)) * 9;
      double *dst;
      if (i == j) {
        dst = vdia + (size_t)i * 9;
      } else {
        if (merge_buffer[j] == ORC_UNSET) return 1;
        dst = vcrs + (size_t)merge_buffer[j] * 9;
      }
      for (int k = 0; k < 9; ++k) dst[k] += src[k];
    }
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) merge_buffer[col[s]] = ORC_UNSET;
  }
  return 0;
}

/* SetFixedBC = Dia(1) + Row + Col, include/delfem2/ls_block_sparse.h:147-151 */
/* and ls_block_sparse.cpp:397-472: for every fixed DOF zero its row and     */
/* column (keeping the matrix symmetric) and put 1 on the diagonal.          */
void orc_set_fixed_bc(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      double *vcrs, double *vdia, const int *bc) {
  for (uint32_t i = 0; i < nblk; ++i) {
    double *d = vdia + (size_t)i * 9;
    for (int a = 0; a < 3; ++a) {
      if (bc[(size_t)i * 3 + a] == 0) continue;
      for (int b = 0; b < 3; ++b) { d[a * 3 + b] = 0.0; d[b * 3 + a] = 0.0; }
      d[a * 3 + a] = 1.0;
    }
  }
  for (uint32_t i = 0; i < nblk; ++i)
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s)
      for (int a = 0; a < 3; ++a) {
        if (bc[(size_t)i * 3 + a] == 0) continue;
        for (int b = 0; b < 3; ++b) vcrs[(size_t)s * 9 + a * 3 + b] = 0.0;
      }
  for (uint32_t i = 0; i < nblk; ++i)
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) {
      const uint32_t j = col[s];
      for (int b = 0; b < 3; ++b) {
        if (bc[(size_t)j * 3 + b] == 0) continue;
        for (int a = 0; a < 3; ++a) vcrs[(size_t)s * 9 + a * 3 + b] = 0.0;
      }
    }
}

/* setRHS_Zero, include/delfem2/vecxitrsol.cpp:286-296 (offset 0). */
void orc_rhs_zero(double *b, const int *bc, size_t ndof) {
  for (size_t i = 0; i < ndof; ++i)
    if (bc[i] != 0) b[i] = 0.0;
}

/* ---------------------------------------------------------------------- */
/* Linear tet element: TetVolume3D include/delfem2/femutil.cpp:202-212,     */
/* TetDlDx femutil.cpp:215-258 (gradients of the barycentric coordinates),  */
/* AddEmat_LinearSolid3<4> include/delfem2/fem_solidlinear.cpp:55-79:       */
/*   K_e[i][j][a][b] = vol*(lambda dN_i[a] dN_j[b] + myu dN_j[a] dN_i[b]    */
/*                          + myu (dN_i . dN_j) delta_ab)                    */
static double orc_tet_volume(const double *p0, const double *p1, const double *p2,
                             const double *p3) {
  const double ax = p1[0] - p0[0], ay = p1[1] - p0[1], az = p1[2] - p0[2];
  const double bx = p2[0] - p0[0], by = p2[1] - p0[1], bz = p2[2] - p0[2];
  const double cx = p3[0] - p0[0], cy = p3[1] - p0[1], cz = p3[2] - p0[2];
  return (ax * (by * cz - cy * bz) - ay * (bx * cz - cx * bz) + az * (bx * cy - cx * by)) / 6.0;
}

/* gradient of barycentric coordinate k: (face opposite k) normal / (6 vol)  */
static void orc_tet_grad(const double P[4][3], double vol, double dN[4][3]) {
  const double inv6v = 1.0 / (6.0 * vol);
  for (int k = 0; k < 4; ++k) {
    /* the other three vertices, ordered so that the sign matches a 0->1->2->3 */
    /* positive orientation: N_k = 1 at P[k] and 0 on the opposite face.        */
    const double *a = P[(k + 1) % 4], *b = P[(k + 2) % 4], *c = P[(k + 3) % 4];
    const double ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2];
    const double wx = c[0] - a[0], wy = c[1] - a[1], wz = c[2] - a[2];
    const double nx = uy * wz - uz * wy, ny = uz * wx - ux * wz, nz = ux * wy - uy * wx;
    /* for odd k the cyclic triple has opposite orientation */
    const double sgn = (k % 2 == 0) ? -1.0 : 1.0;
    dN[k][0] = sgn * nx * inv6v;
    dN[k][1] = sgn * ny * inv6v;
    dN[k][2] = sgn * nz * inv6v;
  }
}

void orc_emat_tet_linear(const double P[4][3], double myu, double lambda,
                         double emat[4][4][3][3], double *vol_out) {
  const double vol = orc_tet_volume(P[0], P[1], P[2], P[3]);
  double dN[4][3];
  orc_tet_grad(P, vol, dN);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const double dd = dN[i][0] * dN[j][0] + dN[i][1] * dN[j][1] + dN[i][2] * dN[j][2];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          emat[i][j][a][b] = vol * (lambda * dN[i][a] * dN[j][b] + myu * dN[j][a] * dN[i][b] +
                                    (a == b ? myu * dd : 0.0));
    }
  if (vol_out) *vol_out = vol;
}

/* Per-tet-E assembly: the caller loop over EMat_SolidLinear_Static_Tet +   */
/* Merge that MergeLinSys_SolidLinear_Static_MeshTet3D                      */
/* (include/delfem2/fem_solidlinear.h:192-237) performs for scalar moduli.   */
/* Residual per node: body force rho*g*vol/4 (213-221) minus K_e u_e        */
/* (fem_solidlinear.cpp:430-434 with scale -1); b += residual; K += K_e.     */
/* Lame parameters from (E, nu): lambda = E nu/((1+nu)(1-2nu)),             */
/* myu = E/(2(1+nu)).                                                        */
int orc_assemble_tet_linear(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                            double *vcrs, double *vdia, double *b,
                            const double *xyz, const uint32_t *tet, size_t ntet,
                            const double *young, double nu, double rho,
                            const double g[3], const double *disp) {
  uint32_t *buf = (uint32_t *)malloc((size_t)nblk * sizeof(uint32_t));
  for (uint32_t i = 0; i < nblk; ++i) buf[i] = ORC_UNSET;
  double emat[4][4][3][3];
  int status = 0;
  for (size_t e = 0; e < ntet && status == 0; ++e) {
    const uint32_t *n = tet + e * 4;
    double P[4][3], U[4][3];
    for (int k = 0; k < 4; ++k)
      for (int d = 0; d < 3; ++d) {
        P[k][d] = xyz[(size_t)n[k] * 3 + d];
        U[k][d] = disp ? disp[(size_t)n[k] * 3 + d] : 0.0;
      }
    const double E = young[e];
    const double lambda = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    const double myu = E / (2.0 * (1.0 + nu));
    double vol;
    orc_emat_tet_linear(P, myu, lambda, emat, &vol);
    for (int i = 0; i < 4; ++i) {
      double res[3];
      for (int a = 0; a < 3; ++a) res[a] = vol * rho * g[a] * 0.25;
      for (int j = 0; j < 4; ++j)
        for (int a = 0; a < 3; ++a)
          res[a] -= emat[i][j][a][0] * U[j][0] + emat[i][j][a][1] * U[j][1] + emat[i][j][a][2] * U[j][2];
      for (int a = 0; a < 3; ++a) b[(size_t)n[i] * 3 + a] += res[a];
    }
    status = orc_merge(nblk, row_start, col, vcrs, vdia, 4, n, &emat[0][0][0][0], buf);
  }
  free(buf);
  return status;
}

/* Adjoint element term dL/dE_e = -lam_e^T (dK_e/dE_e) u_e. K_e is linear in */
/* E (lambda and myu both scale with E), so dK_e/dE_e = K_e / E_e.           */
void orc_tet_dLdE(const double *xyz, const uint32_t *tet, size_t ntet,
                  const double *young, double nu, const double *u,
                  const double *lam, double *dLdE) {
  double emat[4][4][3][3];
  const double lam1 = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double myu1 = 1.0 / (2.0 * (1.0 + nu));
  (void)young;
  for (size_t e = 0; e < ntet; ++e) {
    const uint32_t *n = tet + e * 4;
    double P[4][3];
    for (int k = 0; k < 4; ++k)
      for (int d = 0; d < 3; ++d) P[k][d] = xyz[(size_t)n[k] * 3 + d];
    orc_emat_tet_linear(P, myu1, lam1, emat, NULL);
    double s = 0.0;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        for (int a = 0; a < 3; ++a)
          for (int c = 0; c < 3; ++c)
            s += lam[(size_t)n[i] * 3 + a] * emat[i][j][a][c] * u[(size_t)n[j] * 3 + c];
    dLdE[e] = -s;
  }
}

/* ---------------------------------------------------------------------- */
/* SetPattern0, include/delfem2/ls_ilu_block_sparse.cpp:1057-1090: copy the */
/* pattern, sort each row ascending, dia_ind[i] = first slot with col > i   */
/* (row end if none).                                                        */
void orc_ilu_pattern0(uint32_t nblk, const uint32_t *row_start, const uint32_t *col_in,
                      uint32_t *col_out, uint32_t *dia_ind) {
  memcpy(col_out, col_in, (size_t)row_start[nblk] * sizeof(uint32_t));
  for (uint32_t i = 0; i < nblk; ++i) {
    for (uint32_t a = row_start[i] + 1; a < row_start[i + 1]; ++a) {
      const uint32_t v = col_out[a];
      uint32_t b = a;
      while (b > row_start[i] && col_out[b - 1] > v) { col_out[b] = col_out[b - 1]; --b; }
      col_out[b] = v;
    }
    dia_ind[i] = row_start[i + 1];
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s)
      if (col_out[s] > i) { dia_ind[i] = s; break; }
  }
}

/* CopyValue, ls_ilu_block_sparse.cpp:1009-1047: zero the factor storage,  */
/* scatter each matrix block into the ILU slot with the same column, copy   */
/* the diagonal.                                                            */
void orc_ilu_copy_value(uint32_t nblk, const uint32_t *row_start, const uint32_t *col_ilu,
                        double *ilu_vcrs, double *ilu_vdia,
                        const uint32_t *col_mat, const double *mat_vcrs,
                        const double *mat_vdia) {
  memset(ilu_vcrs, 0, (size_t)row_start[nblk] * 9 * sizeof(double));
  int64_t *slot_of = (int64_t *)malloc((size_t)nblk * sizeof(int64_t));
  for (uint32_t i = 0; i < nblk; ++i) slot_of[i] = -1;
  for (uint32_t i = 0; i < nblk; ++i) {
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) slot_of[col_ilu[s]] = s;
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) {
      const int64_t t = slot_of[col_mat[s]];
      if (t < 0) continue;
      memcpy(ilu_vcrs + (size_t)t * 9, mat_vcrs + (size_t)s * 9, 9 * sizeof(double));
    }
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) slot_of[col_ilu[s]] = -1;
  }
  free(slot_of);
  memcpy(ilu_vdia, mat_vdia, (size_t)nblk * 9 * sizeof(double));
}

/* 3x3 determinant and adjugate inverse (the cofactor formula used by       */
/* ls_ilu_block_sparse.cpp:84-103).                                          */
static double orc_det3(const double *m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

static void orc_inv3(double *m) {
  const double t[9] = {m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8]};
  const double s = 1.0 / orc_det3(t);
  m[0] = s * (t[4] * t[8] - t[5] * t[7]);
  m[1] = s * (t[2] * t[7] - t[1] * t[8]);
  m[2] = s * (t[1] * t[5] - t[2] * t[4]);
  m[3] = s * (t[5] * t[6] - t[3] * t[8]);
  m[4] = s * (t[0] * t[8] - t[2] * t[6]);
  m[5] = s * (t[2] * t[3] - t[0] * t[5]);
  m[6] = s * (t[3] * t[7] - t[4] * t[6]);
  m[7] = s * (t[1] * t[6] - t[0] * t[7]);
  m[8] = s * (t[0] * t[4] - t[1] * t[3]);
}

/* Decompose (double, 3x3 branch), ls_ilu_block_sparse.cpp:152-160,286-356: */
/* rows in ascending order; for every k < i in row i (ascending) and every  */
/* j > k in row k: A_ij -= A_ik A_kj when (i,j) is in the pattern (A_ii when */
/* j == i). Then D_i <- inverse(D_i) unless |det| <= 1e-30 (counted as a    */
/* singular pivot and left as is; more than 10 stops with failure), then    */
/* U_ij <- D_i^-1 U_ij. Returns 0 on success, 1 on failure.                  */
int orc_ilu_decompose(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      const uint32_t *dia_ind, double *vcrs, double *vdia,
                      int *n_singular) {
  int64_t *slot_of = (int64_t *)malloc((size_t)nblk * sizeof(int64_t));
  for (uint32_t i = 0; i < nblk; ++i) slot_of[i] = -1;
  int nsing = 0, status = 0;
  for (uint32_t i = 0; i < nblk && status == 0; ++i) {
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) slot_of[col[s]] = s;
    for (uint32_t sk = row_start[i]; sk < dia_ind[i]; ++sk) {
      const uint32_t k = col[sk];
      const double *aik = vcrs + (size_t)sk * 9;
      for (uint32_t sj = dia_ind[k]; sj < row_start[k + 1]; ++sj) {
        const uint32_t j = col[sj];
        double *aij;
        if (j == i) {
          aij = vdia + (size_t)i * 9;
        } else {
          if (slot_of[j] < 0) continue;
          aij = vcrs + (size_t)slot_of[j] * 9;
        }
        const double *akj = vcrs + (size_t)sj * 9;
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c)
            aij[r * 3 + c] -= aik[r * 3 + 0] * akj[0 * 3 + c] + aik[r * 3 + 1] * akj[1 * 3 + c] +
                              aik[r * 3 + 2] * akj[2 * 3 + c];
      }
    }
    double *dii = vdia + (size_t)i * 9;
    if (fabs(orc_det3(dii)) > 1.0e-30) {
      orc_inv3(dii);
    } else {
      ++nsing;
      if (nsing > 10) status = 1;
    }
    if (status == 0) {
      for (uint32_t s = dia_ind[i]; s < row_start[i + 1]; ++s) {
        double *u = vcrs + (size_t)s * 9;
        const double t[9] = {u[0], u[1], u[2], u[3], u[4], u[5], u[6], u[7], u[8]};
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c)
            u[r * 3 + c] = dii[r * 3 + 0] * t[0 * 3 + c] + dii[r * 3 + 1] * t[1 * 3 + c] +
                           dii[r * 3 + 2] * t[2 * 3 + c];
      }
    }
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) slot_of[col[s]] = -1;
  }
  free(slot_of);
  if (n_singular) *n_singular = nsing;
  return status;
}

/* ForwardSubstitution 3x3, ls_ilu_block_sparse.cpp:544-573:                */
/* v_i <- D_i^-1 (v_i - sum_{j<i} L_ij v_j), ascending rows, in place.      */
void orc_ilu_forward(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                     const uint32_t *dia_ind, const double *vcrs, const double *vdia,
                     double *vec) {
  for (uint32_t i = 0; i < nblk; ++i) {
    double t[3] = {vec[(size_t)i * 3], vec[(size_t)i * 3 + 1], vec[(size_t)i * 3 + 2]};
    for (uint32_t s = row_start[i]; s < dia_ind[i]; ++s) {
      const double *a = vcrs + (size_t)s * 9;
      const double *vj = vec + (size_t)col[s] * 3;
      for (int r = 0; r < 3; ++r) t[r] -= a[r * 3] * vj[0] + a[r * 3 + 1] * vj[1] + a[r * 3 + 2] * vj[2];
    }
    const double *d = vdia + (size_t)i * 9;
    for (int r = 0; r < 3; ++r)
      vec[(size_t)i * 3 + r] = d[r * 3] * t[0] + d[r * 3 + 1] * t[1] + d[r * 3 + 2] * t[2];
  }
}

/* BackwardSubstitution 3x3, ls_ilu_block_sparse.cpp:721-749:               */
/* v_i <- v_i - sum_{j>i} U'_ij v_j, descending rows, in place.             */
void orc_ilu_backward(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      const uint32_t *dia_ind, const double *vcrs, double *vec) {
  for (uint32_t ii = nblk; ii-- > 0;) {
    double t[3] = {vec[(size_t)ii * 3], vec[(size_t)ii * 3 + 1], vec[(size_t)ii * 3 + 2]};
    for (uint32_t s = dia_ind[ii]; s < row_start[ii + 1]; ++s) {
      const double *a = vcrs + (size_t)s * 9;
      const double *vj = vec + (size_t)col[s] * 3;
      for (int r = 0; r < 3; ++r) t[r] -= a[r * 3] * vj[0] + a[r * 3 + 1] * vj[1] + a[r * 3 + 2] * vj[2];
    }
    for (int r = 0; r < 3; ++r) vec[(size_t)ii * 3 + r] = t[r];
  }
}

/* Level sets of the triangular sweeps (no reference counterpart: the       */
/* reference sweeps rows serially). Forward: level(i) = 0 when row i has no */
/* column j < i, else 1 + max level(j) over its columns j < i. Backward:    */
/* the same over columns j > i. `order` lists the rows by (level, row id)   */
/* ascending; level_start[l] is the first position of level l. Returns the  */
/* number of levels.                                                         */
uint32_t orc_ilu_levels(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                        const uint32_t *dia_ind, int backward, uint32_t *level,
                        uint32_t *order, uint32_t *level_start) {
  uint32_t nlev = 0;
  for (uint32_t n = 0; n < nblk; ++n) {
    const uint32_t i = backward ? nblk - 1 - n : n;
    const uint32_t s0 = backward ? dia_ind[i] : row_start[i];
    const uint32_t s1 = backward ? row_start[i + 1] : dia_ind[i];
    uint32_t lv = 0;
    for (uint32_t s = s0; s < s1; ++s) {
      const uint32_t j = col[s];
      if (j == i) continue;
      if (level[j] + 1 > lv) lv = level[j] + 1;
    }
    level[i] = lv;
    if (lv + 1 > nlev) nlev = lv + 1;
  }
  for (uint32_t l = 0; l <= nlev; ++l) level_start[l] = 0;
  for (uint32_t i = 0; i < nblk; ++i) level_start[level[i] + 1] += 1;
  for (uint32_t l = 0; l < nlev; ++l) level_start[l + 1] += level_start[l];
  uint32_t *cursor = (uint32_t *)malloc(((size_t)nlev + 1) * sizeof(uint32_t));
  memcpy(cursor, level_start, ((size_t)nlev + 1) * sizeof(uint32_t));
  for (uint32_t i = 0; i < nblk; ++i) order[cursor[level[i]]++] = i;
  free(cursor);
  return nlev;
}

/* ---------------------------------------------------------------------- */
double orc_dot(const double *a, const double *b, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* Solve_PCG, include/delfem2/lsitrsol.h:80-148 with the vector primitives  */
/* of include/delfem2/view_vectorx.h:61-109. x starts at 0; history holds   */
/* absolute residual norms [|r0|, |r1|, ...]; stops when                     */
/* sqrt(|r|^2/|r0|^2) < tol; early return when |r0|^2 < 1e-30; one extra    */
/* final entry when max_iter is exhausted. r is overwritten with the final   */
/* residual. Returns the history length (entries past hist_cap are counted  */
/* but not stored).                                                          */
uint32_t orc_solve_pcg_k(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                         const double *vcrs, const double *vdia, const uint32_t *ilu_row_start,
                         const uint32_t *ilu_col, const uint32_t *dia_ind,
                         const double *ilu_vcrs, const double *ilu_vdia,
                         double *r, double *x, double tol, uint32_t max_iter,
                         double *hist, uint32_t hist_cap) {
  const size_t n = (size_t)nblk * 3;
  uint32_t nh = 0;
#define ORC_PUSH(v)                          \
  do {                                       \
    if (nh < hist_cap) hist[nh] = (v);       \
    ++nh;                                    \
  } while (0)
  for (size_t k = 0; k < n; ++k) x[k] = 0.0;
  const double sq0 = orc_dot(r, r, n);
  ORC_PUSH(sqrt(sq0));
  if (sq0 < 1.0e-30) return nh;
  const double inv_sq0 = 1.0 / sq0;
  double *Pr = (double *)malloc(n * sizeof(double));
  double *p = (double *)malloc(n * sizeof(double));
  memcpy(Pr, r, n * sizeof(double));
  orc_ilu_forward(nblk, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia, Pr);
  orc_ilu_backward(nblk, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, Pr);
  memcpy(p, Pr, n * sizeof(double));
  double rPr = orc_dot(r, Pr, n);
  int converged = 0;
  for (uint32_t it = 0; it < max_iter; ++it) {
    double *Ap = Pr; /* the reference reuses Pr's storage for Ap */
    orc_bsr_matvec(nblk, row_start, col, vcrs, vdia, Ap, 1.0, p, 0.0);
    const double pAp = orc_dot(p, Ap, n);
    const double alpha = rPr / pAp;
    for (size_t k = 0; k < n; ++k) r[k] += -alpha * Ap[k];
    for (size_t k = 0; k < n; ++k) x[k] += alpha * p[k];
    const double sq = orc_dot(r, r, n);
    ORC_PUSH(sqrt(sq));
    if (sqrt(sq * inv_sq0) < tol) { converged = 1; break; }
    memcpy(Pr, r, n * sizeof(double));
    orc_ilu_forward(nblk, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia, Pr);
    orc_ilu_backward(nblk, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, Pr);
    const double rPr1 = orc_dot(r, Pr, n);
    const double beta = rPr1 / rPr;
    rPr = rPr1;
    for (size_t k = 0; k < n; ++k) p[k] = beta * p[k] + Pr[k];
  }
  if (!converged) ORC_PUSH(sqrt(orc_dot(r, r, n)));
#undef ORC_PUSH
  free(Pr);
  free(p);
  return nh;
}

/* Solve_PCG with the ILU(0) factors (the ILU shares the matrix's row offsets). */
uint32_t orc_solve_pcg(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                       const double *vcrs, const double *vdia,
                       const uint32_t *ilu_col, const uint32_t *dia_ind,
                       const double *ilu_vcrs, const double *ilu_vdia,
                       double *r, double *x, double tol, uint32_t max_iter,
                       double *hist, uint32_t hist_cap) {
  return orc_solve_pcg_k(nblk, row_start, col, vcrs, vdia, row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia, r, x,
                         tol, max_iter, hist, hist_cap);
}

/* Solve_CG, include/delfem2/lsitrsol.h:35-74: history holds the relative   */
/* ratio sqrt(|r|^2/|r0|^2) per iteration (no initial or final extra entry). */
uint32_t orc_solve_cg(uint32_t nblk, const uint32_t *row_start, const uint32_t *col,
                      const double *vcrs, const double *vdia, double *r, double *x,
                      double tol, uint32_t max_iter, double *hist, uint32_t hist_cap) {
  const size_t n = (size_t)nblk * 3;
  uint32_t nh = 0;
  for (size_t k = 0; k < n; ++k) x[k] = 0.0;
  double sq = orc_dot(r, r, n);
  if (sq < 1.0e-30) return 0;
  const double inv_sq0 = 1.0 / sq;
  double *p = (double *)malloc(n * sizeof(double));
  double *Ap = (double *)malloc(n * sizeof(double));
  memcpy(p, r, n * sizeof(double));
  for (uint32_t it = 0; it < max_iter; ++it) {
    orc_bsr_matvec(nblk, row_start, col, vcrs, vdia, Ap, 1.0, p, 0.0);
    const double alpha = sq / orc_dot(p, Ap, n);
    for (size_t k = 0; k < n; ++k) x[k] += alpha * p[k];
    for (size_t k = 0; k < n; ++k) r[k] += -alpha * Ap[k];
    const double sq1 = orc_dot(r, r, n);
    const double ratio = sqrt(sq1 * inv_sq0);
    if (nh < hist_cap) hist[nh] = ratio;
    ++nh;
    if (ratio < tol) break;
    const double beta = sq1 / sq;
    sq = sq1;
    for (size_t k = 0; k < n; ++k) p[k] = beta * p[k] + r[k];
  }
  free(p);
  free(Ap);
  return nh;
}

/* ====================================================================== */
/* Cloth (implicit, backward Euler).                                       */

/* SetClothShape_Square, include/delfem2/cloth_internal.h:333-397 (mesh     */
/* part): (ndiv+1)^2 nodes (ix major), two triangles per cell, and the four-*/
/* node bending stencils: one per cell diagonal, then the y-direction and   */
/* the x-direction interior edges.                                           */
void orc_cloth_square(uint32_t ndiv, double size, double *xyz0, uint32_t *tri, uint32_t *quad) {
  const double h = size / ndiv;
  const uint32_t m = ndiv + 1;
  size_t k = 0;
  for (uint32_t ix = 0; ix <= ndiv; ++ix)
    for (uint32_t iy = 0; iy <= ndiv; ++iy) {
      xyz0[k++] = ix * h;
      xyz0[k++] = iy * h;
      xyz0[k++] = 0.0;
    }
#define ORC_ID(x, y) ((x) * m + (y))
  size_t t = 0;
  for (uint32_t ix = 0; ix < ndiv; ++ix)
    for (uint32_t iy = 0; iy < ndiv; ++iy) {
      tri[t++] = ORC_ID(ix, iy);
      tri[t++] = ORC_ID(ix + 1, iy);
      tri[t++] = ORC_ID(ix, iy + 1);
      tri[t++] = ORC_ID(ix + 1, iy + 1);
      tri[t++] = ORC_ID(ix, iy + 1);
      tri[t++] = ORC_ID(ix + 1, iy);
    }
  size_t q = 0;
  for (uint32_t ix = 0; ix < ndiv; ++ix)
    for (uint32_t iy = 0; iy < ndiv; ++iy) {
      quad[q++] = ORC_ID(ix, iy);
      quad[q++] = ORC_ID(ix + 1, iy + 1);
      quad[q++] = ORC_ID(ix + 1, iy);
      quad[q++] = ORC_ID(ix, iy + 1);
    }
  for (uint32_t ix = 0; ix < ndiv; ++ix)
    for (uint32_t iy = 0; iy + 1 < ndiv; ++iy) {
      quad[q++] = ORC_ID(ix + 1, iy);
      quad[q++] = ORC_ID(ix, iy + 2);
      quad[q++] = ORC_ID(ix + 1, iy + 1);
      quad[q++] = ORC_ID(ix, iy + 1);
    }
  for (uint32_t ix = 0; ix + 1 < ndiv; ++ix)
    for (uint32_t iy = 0; iy < ndiv; ++iy) {
      quad[q++] = ORC_ID(ix, iy + 1);
      quad[q++] = ORC_ID(ix + 2, iy);
      quad[q++] = ORC_ID(ix + 1, iy);
      quad[q++] = ORC_ID(ix + 1, iy + 1);
    }
#undef ORC_ID
}

static void orc_cross(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
static double orc_dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* MakePositiveDefinite_Sim22, include/delfem2/fem_stvk.cpp:211-264, on the  */
/* symmetric 2x2 [[s0,s2],[s2,s1]] with eigenvalues b-e <= b+e: kept when    */
/* b-e > 1e-20, zeroed when b+e < 0, else l*t t^T with l = b+e and t the     */
/* normalised longer row of (S - l I) (zero if both rows are < 1e-10 long). */
/* Note t is orthogonal to the eigenvector of l: the reference's rank-1      */
/* result is kept as is for parity.                                          */
void orc_make_pd_sim22(const double s2[3], double s3[3]) {
  const double b = 0.5 * (s2[0] + s2[1]);
  const double e = sqrt(0.25 * (s2[0] - s2[1]) * (s2[0] - s2[1]) + s2[2] * s2[2]);
  if (b - e > 1.0e-20) {
    s3[0] = s2[0];
    s3[1] = s2[1];
    s3[2] = s2[2];
    return;
  }
  if (b + e < 0) {
    s3[0] = s3[1] = s3[2] = 0.0;
    return;
  }
  const double l = b + e;
  double t0[2] = {s2[0] - l, s2[2]}, t1[2] = {s2[2], s2[1] - l};
  const double q0 = t0[0] * t0[0] + t0[1] * t0[1], q1 = t1[0] * t1[0] + t1[1] * t1[1];
  const double *t = q0 > q1 ? t0 : t1;
  const double qq = q0 > q1 ? q0 : q1;
  if (qq < 1.0e-20) {
    s3[0] = s3[1] = s3[2] = 0.0;
    return;
  }
  const double inv = 1.0 / sqrt(qq);
  const double u0 = t[0] * inv, u1 = t[1] * inv;
  s3[0] = l * u0 * u0;
  s3[1] = l * u1 * u1;
  s3[2] = l * u0 * u1;
}

/* WdWddW_CST, include/delfem2/fem_stvk.cpp:267-374: St.Venant-Kirchhoff    */
/* constant-strain triangle. Covariant rest edges G0, G1 and contravariant   */
/* G^0, G^1; Green strain E = (E00, E11, 2E01); S = C E with the plane       */
/* constitutive matrix in the contravariant metric; W = A/2 E.S;             */
/* dW[a][i] = A sum_p S_p B_p(a,i) with B_0 = g0_i dN_a0, B_1 = g1_i dN_a1,   */
/* B_2 = g0_i dN_a1 + g1_i dN_a0; ddW = A B^T C B + A (S+ : dN dN) I where  */
/* S+ is S made positive definite (orc_make_pd_sim22).                       */
void orc_wdwddw_cst(const double C[3][3], const double c[3][3], double lambda, double myu, double *W,
                    double dW[3][3], double ddW[3][3][3][3]) {
  double G0[3], G1[3], n[3];
  for (int d = 0; d < 3; ++d) {
    G0[d] = C[1][d] - C[0][d];
    G1[d] = C[2][d] - C[0][d];
  }
  orc_cross(G0, G1, n);
  const double nlen = sqrt(orc_dot3(n, n));
  const double area = 0.5 * nlen;
  for (int d = 0; d < 3; ++d) n[d] /= nlen;
  double Gu0[3], Gu1[3];
  orc_cross(G1, n, Gu0);
  orc_cross(n, G0, Gu1);
  const double s0 = 1.0 / orc_dot3(Gu0, G0), s1 = 1.0 / orc_dot3(Gu1, G1);
  for (int d = 0; d < 3; ++d) {
    Gu0[d] *= s0;
    Gu1[d] *= s1;
  }
  double g0[3], g1[3];
  for (int d = 0; d < 3; ++d) {
    g0[d] = c[1][d] - c[0][d];
    g1[d] = c[2][d] - c[0][d];
  }
  const double E[3] = {0.5 * (orc_dot3(g0, g0) - orc_dot3(G0, G0)), 0.5 * (orc_dot3(g1, g1) - orc_dot3(G1, G1)),
                       orc_dot3(g0, g1) - orc_dot3(G0, G1)};
  const double m00 = orc_dot3(Gu0, Gu0), m11 = orc_dot3(Gu1, Gu1), m01 = orc_dot3(Gu1, Gu0);
  const double Cm[3][3] = {{lambda * m00 * m00 + 2 * myu * m00 * m00, lambda * m00 * m11 + 2 * myu * m01 * m01,
                            lambda * m00 * m01 + 2 * myu * m00 * m01},
                           {lambda * m11 * m00 + 2 * myu * m01 * m01, lambda * m11 * m11 + 2 * myu * m11 * m11,
                            lambda * m11 * m01 + 2 * myu * m01 * m11},
                           {lambda * m01 * m00 + 2 * myu * m00 * m01, lambda * m01 * m11 + 2 * myu * m01 * m11,
                            lambda * m01 * m01 + myu * (m00 * m11 + m01 * m01)}};
  double S[3];
  for (int p = 0; p < 3; ++p) S[p] = Cm[p][0] * E[0] + Cm[p][1] * E[1] + Cm[p][2] * E[2];
  *W = 0.5 * area * (E[0] * S[0] + E[1] * S[1] + E[2] * S[2]);
  static const double dN[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};
  double B[3][3][3]; /* B[p][a][i] */
  for (int a = 0; a < 3; ++a)
    for (int i = 0; i < 3; ++i) {
      B[0][a][i] = g0[i] * dN[a][0];
      B[1][a][i] = g1[i] * dN[a][1];
      B[2][a][i] = g0[i] * dN[a][1] + g1[i] * dN[a][0];
      dW[a][i] = area * (S[0] * B[0][a][i] + S[1] * B[1][a][i] + S[2] * B[2][a][i]);
    }
  double Sp[3];
  orc_make_pd_sim22(S, Sp);
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double v = 0.0;
          for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) v += B[p][a][i] * Cm[p][q] * B[q][b][j];
          ddW[a][b][i][j] = area * v;
        }
      const double g = area * (Sp[0] * dN[a][0] * dN[b][0] + Sp[2] * (dN[a][0] * dN[b][1] + dN[a][1] * dN[b][0]) +
                               Sp[1] * dN[a][1] * dN[b][1]);
      for (int i = 0; i < 3; ++i) ddW[a][b][i][i] += g;
    }
}

static double orc_tri_area(const double *a, const double *b, const double *c) {
  double u[3], w[3], n[3];
  for (int d = 0; d < 3; ++d) {
    u[d] = b[d] - a[d];
    w[d] = c[d] - a[d];
  }
  orc_cross(u, w, n);
  return 0.5 * sqrt(orc_dot3(n, n));
}

/* WdWddW_Bend, include/delfem2/fem_quadratic_bending.cpp:49-107: quadratic  */
/* bending of the hinge (C2,C3) shared by triangles (C0,C2,C3), (C1,C3,C2):  */
/* cotangent weights K, ddW[a][b] = K_a K_b stiff/((A0+A1) L^2) I (constant), */
/* dW = ddW c, W = dW . c.                                                    */
void orc_wdwddw_bend(const double C[4][3], const double c[4][3], double stiff, double *W, double dW[4][3],
                     double ddW[4][4][3][3]) {
  const double A0 = orc_tri_area(C[0], C[2], C[3]), A1 = orc_tri_area(C[1], C[3], C[2]);
  double e23[3], e02[3], e03[3], e12[3], e13[3];
  for (int d = 0; d < 3; ++d) {
    e23[d] = C[3][d] - C[2][d];
    e02[d] = C[2][d] - C[0][d];
    e03[d] = C[3][d] - C[0][d];
    e12[d] = C[2][d] - C[1][d];
    e13[d] = C[3][d] - C[1][d];
  }
  const double L = sqrt(orc_dot3(e23, e23));
  const double H0 = 2.0 * A0 / L, H1 = 2.0 * A1 / L;
  const double c023 = -orc_dot3(e02, e23) / H0, c032 = orc_dot3(e03, e23) / H0;
  const double c123 = -orc_dot3(e12, e23) / H1, c132 = orc_dot3(e13, e23) / H1;
  const double k = stiff / ((A0 + A1) * L * L);
  const double K[4] = {-c023 - c032, -c123 - c132, c032 + c132, c023 + c123};
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) ddW[a][b][i][j] = (i == j) ? K[a] * K[b] * k : 0.0;
  *W = 0.0;
  for (int a = 0; a < 4; ++a)
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int b = 0; b < 4; ++b) s += K[a] * K[b] * k * c[b][i];
      dW[a][i] = s;
      *W += s * c[a][i];
    }
}

/* MergeLinSys_Cloth, include/delfem2/femcloth.h:48-114, with the membrane    */
/* moduli per triangle (lambda, myu from E_t and nu): adds the CST and bending */
/* Hessians into K and their gradients into dW; returns the energy (or NaN on */
/* a missing slot).                                                           */
double orc_cloth_assemble(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                          double *vdia, double *dW, const double *xyz0, const double *xyz, const uint32_t *tri,
                          size_t ntri, const uint32_t *quad, size_t nquad, const double *young_tri, double nu,
                          double stiff_bend) {
  uint32_t *buf = (uint32_t *)malloc((size_t)nblk * sizeof(uint32_t));
  for (uint32_t i = 0; i < nblk; ++i) buf[i] = ORC_UNSET;
  double W = 0.0;
  for (size_t t = 0; t < ntri; ++t) {
    const uint32_t *n = tri + t * 3;
    double C[3][3], c[3][3], w, dw[3][3], ddw[3][3][3][3];
    for (int a = 0; a < 3; ++a)
      for (int d = 0; d < 3; ++d) {
        C[a][d] = xyz0[(size_t)n[a] * 3 + d];
        c[a][d] = xyz[(size_t)n[a] * 3 + d];
      }
    const double E = young_tri[t];
    orc_wdwddw_cst(C, c, E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), E / (2.0 * (1.0 + nu)), &w, dw, ddw);
    W += w;
    for (int a = 0; a < 3; ++a)
      for (int d = 0; d < 3; ++d) dW[(size_t)n[a] * 3 + d] += dw[a][d];
    if (orc_merge(nblk, row_start, col, vcrs, vdia, 3, n, &ddw[0][0][0][0], buf)) W = NAN;
  }
  for (size_t q = 0; q < nquad; ++q) {
    const uint32_t *n = quad + q * 4;
    double C[4][3], c[4][3], w, dw[4][3], ddw[4][4][3][3];
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) {
        C[a][d] = xyz0[(size_t)n[a] * 3 + d];
        c[a][d] = xyz[(size_t)n[a] * 3 + d];
      }
    orc_wdwddw_bend(C, c, stiff_bend, &w, dw, ddw);
    W += w;
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) dW[(size_t)n[a] * 3 + d] += dw[a][d];
    if (orc_merge(nblk, row_start, col, vcrs, vdia, 4, n, &ddw[0][0][0][0], buf)) W = NAN;
  }
  free(buf);
  return W;
}

/* One backward-Euler step, the sequence of StepTime_InternalDynamicsILU     */
/* (include/delfem2/cloth_internal.h:179-269) with the gravity term of       */
/* AddWdW_Gravity (76-92) and the caller's tolerance and iteration limit:    */
/*   A = M/dt^2 + ddW(x), b = -(dW(x) - M g) + M v/dt, clamp, ILU(0)-PCG;     */
/*   free DOFs: x += dx, v = dx/dt. Returns the PCG history length.           */
uint32_t orc_cloth_step(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *xyz, double *uvw,
                        const double *xyz0, const int *bc, const uint32_t *tri, size_t ntri, const uint32_t *quad,
                        size_t nquad, const double *young_tri, double nu, double stiff_bend, const double g[3],
                        double mass, double dt, double tol, uint32_t max_iter) {
  const size_t nnz = row_start[nblk], n = (size_t)nblk * 3;
  double *vcrs = (double *)calloc(nnz * 9 + 1, sizeof(double));
  double *vdia = (double *)calloc((size_t)nblk * 9, sizeof(double));
  double *b = (double *)calloc(n, sizeof(double));
  orc_cloth_assemble(nblk, row_start, col, vcrs, vdia, b, xyz0, xyz, tri, ntri, quad, nquad, young_tri, nu,
                     stiff_bend);
  for (uint32_t i = 0; i < nblk; ++i)
    for (int d = 0; d < 3; ++d) b[(size_t)i * 3 + d] -= mass * g[d];
  for (size_t k = 0; k < n; ++k) b[k] = -b[k] + mass * uvw[k] / dt;
  for (uint32_t i = 0; i < nblk; ++i)
    for (int d = 0; d < 3; ++d) vdia[(size_t)i * 9 + d * 4] += mass / (dt * dt);
  orc_set_fixed_bc(nblk, row_start, col, vcrs, vdia, bc);
  orc_rhs_zero(b, bc, n);
  uint32_t *icol = (uint32_t *)malloc((nnz + 1) * sizeof(uint32_t));
  uint32_t *dia = (uint32_t *)malloc((size_t)nblk * sizeof(uint32_t));
  double *ivcrs = (double *)malloc((nnz * 9 + 1) * sizeof(double));
  double *ivdia = (double *)malloc((size_t)nblk * 9 * sizeof(double));
  orc_ilu_pattern0(nblk, row_start, col, icol, dia);
  orc_ilu_copy_value(nblk, row_start, icol, ivcrs, ivdia, col, vcrs, vdia);
  int ns = 0;
  orc_ilu_decompose(nblk, row_start, icol, dia, ivcrs, ivdia, &ns);
  double *dx = (double *)calloc(n, sizeof(double));
  double *hist = (double *)malloc(((size_t)max_iter + 2) * sizeof(double));
  const uint32_t nh = orc_solve_pcg(nblk, row_start, col, vcrs, vdia, icol, dia, ivcrs, ivdia, b, dx, tol, max_iter,
                                    hist, max_iter + 2);
  for (size_t k = 0; k < n; ++k) {
    if (bc[k] != 0) continue;
    xyz[k] += dx[k];
    uvw[k] = dx[k] / dt;
  }
  free(vcrs);
  free(vdia);
  free(b);
  free(icol);
  free(dia);
  free(ivcrs);
  free(ivdia);
  free(dx);
  free(hist);
  return nh;
}

/* ---- cloth adjoint (no reference counterpart; checker for the device's) ---- */

/* Jacobian J[k][l] = d s3_k / d s2_l of orc_make_pd_sim22, branch by branch:  */
/* identity, zero, or the derivative of l u u^T (l = b + e, u = t/|t|, t the   */
/* chosen row of S - l I; the branch choice is locally constant).              */
void orc_pd_sim22_jac(const double s2[3], double J[3][3]) {
  for (int k = 0; k < 3; ++k)
    for (int l = 0; l < 3; ++l) J[k][l] = 0.0;
  const double b = 0.5 * (s2[0] + s2[1]);
  const double e = sqrt(0.25 * (s2[0] - s2[1]) * (s2[0] - s2[1]) + s2[2] * s2[2]);
  if (b - e > 1.0e-20) {
    for (int k = 0; k < 3; ++k) J[k][k] = 1.0;
    return;
  }
  if (b + e < 0) return;
  const double lam = b + e;
  double t0[2] = {s2[0] - lam, s2[2]}, t1[2] = {s2[2], s2[1] - lam};
  const double q0 = t0[0] * t0[0] + t0[1] * t0[1], q1 = t1[0] * t1[0] + t1[1] * t1[1];
  const int first = q0 > q1;
  const double qq = first ? q0 : q1;
  if (qq < 1.0e-20) return;
  /* dl/ds */
  const double dl[3] = {0.5 + 0.25 * (s2[0] - s2[1]) / e, 0.5 - 0.25 * (s2[0] - s2[1]) / e, s2[2] / e};
  /* dt/ds (2 x 3) */
  double dt[2][3];
  for (int l = 0; l < 3; ++l) {
    if (first) {
      dt[0][l] = (l == 0) - dl[l];
      dt[1][l] = (l == 2);
    } else {
      dt[0][l] = (l == 2);
      dt[1][l] = (l == 1) - dl[l];
    }
  }
  const double *t = first ? t0 : t1;
  const double r = sqrt(qq);
  const double u[2] = {t[0] / r, t[1] / r};
  for (int l = 0; l < 3; ++l) {
    /* du = (I - u u^T) dt / r */
    const double ud = u[0] * dt[0][l] + u[1] * dt[1][l];
    const double du[2] = {(dt[0][l] - u[0] * ud) / r, (dt[1][l] - u[1] * ud) / r};
    J[0][l] = dl[l] * u[0] * u[0] + lam * 2.0 * u[0] * du[0];
    J[1][l] = dl[l] * u[1] * u[1] + lam * 2.0 * u[1] * du[1];
    J[2][l] = dl[l] * u[0] * u[1] + lam * (du[0] * u[1] + u[0] * du[1]);
  }
}

/* Per triangle (per-triangle E), with mu the adjoint solve and dx the step  */
/* increment:                                                                */
/*   xbar += -H_true mu - grad_c (mu^T ddW(c) dx),                           */
/*   Ebar_t += -(mu.dW_t + mu^T ddW_t dx) / E_t;                              */
/* per quad: xbar += -H_bend mu. H_true is ddW with the raw stress S in the  */
/* geometric term instead of S+. Written in node space with explicit B       */
/* matrices (dB/dc is constant: dB_p(a,i)/dc(b,j) = delta_ij w_p(a,b)).      */
void orc_cloth_adjoint_terms(const double *xyz0, const double *xyz, const uint32_t *tri, size_t ntri,
                             const uint32_t *quad, size_t nquad, const double *young_tri, double nu,
                             double stiff_bend, const double *mu, const double *dx, double *xbar, double *Ebar) {
  static const double dN[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};
  for (size_t t = 0; t < ntri; ++t) {
    const uint32_t *n = tri + t * 3;
    double C[3][3], c[3][3], M[3][3], D[3][3];
    for (int a = 0; a < 3; ++a)
      for (int d = 0; d < 3; ++d) {
        C[a][d] = xyz0[(size_t)n[a] * 3 + d];
        c[a][d] = xyz[(size_t)n[a] * 3 + d];
        M[a][d] = mu[(size_t)n[a] * 3 + d];
        D[a][d] = dx[(size_t)n[a] * 3 + d];
      }
    const double E = young_tri[t];
    const double lambda = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), myu = E / (2.0 * (1.0 + nu));
    /* W, dW, ddW at c give S (through dW is awkward): recompute the pieces. */
    double G0[3], G1[3], nr[3];
    for (int d = 0; d < 3; ++d) {
      G0[d] = C[1][d] - C[0][d];
      G1[d] = C[2][d] - C[0][d];
    }
    orc_cross(G0, G1, nr);
    const double nlen = sqrt(orc_dot3(nr, nr));
    const double area = 0.5 * nlen;
    for (int d = 0; d < 3; ++d) nr[d] /= nlen;
    double Gu0[3], Gu1[3];
    orc_cross(G1, nr, Gu0);
    orc_cross(nr, G0, Gu1);
    const double s0 = 1.0 / orc_dot3(Gu0, G0), s1 = 1.0 / orc_dot3(Gu1, G1);
    for (int d = 0; d < 3; ++d) {
      Gu0[d] *= s0;
      Gu1[d] *= s1;
    }
    double g0[3], g1[3];
    for (int d = 0; d < 3; ++d) {
      g0[d] = c[1][d] - c[0][d];
      g1[d] = c[2][d] - c[0][d];
    }
    const double Es[3] = {0.5 * (orc_dot3(g0, g0) - orc_dot3(G0, G0)),
                          0.5 * (orc_dot3(g1, g1) - orc_dot3(G1, G1)), orc_dot3(g0, g1) - orc_dot3(G0, G1)};
    const double m00 = orc_dot3(Gu0, Gu0), m11 = orc_dot3(Gu1, Gu1), m01 = orc_dot3(Gu1, Gu0);
    const double Cm[3][3] = {{lambda * m00 * m00 + 2 * myu * m00 * m00, lambda * m00 * m11 + 2 * myu * m01 * m01,
                              lambda * m00 * m01 + 2 * myu * m00 * m01},
                             {lambda * m11 * m00 + 2 * myu * m01 * m01, lambda * m11 * m11 + 2 * myu * m11 * m11,
                              lambda * m11 * m01 + 2 * myu * m01 * m11},
                             {lambda * m01 * m00 + 2 * myu * m00 * m01, lambda * m01 * m11 + 2 * myu * m01 * m11,
                              lambda * m01 * m01 + myu * (m00 * m11 + m01 * m01)}};
    double S[3], Sp[3], J[3][3];
    for (int p = 0; p < 3; ++p) S[p] = Cm[p][0] * Es[0] + Cm[p][1] * Es[1] + Cm[p][2] * Es[2];
    orc_make_pd_sim22(S, Sp);
    orc_pd_sim22_jac(S, J);
    double B[3][3][3], w[3][3][3]; /* B[p][a][i]; w[p][a][b] = dB_p(a,.)/dc(b,.) */
    for (int a = 0; a < 3; ++a) {
      for (int i = 0; i < 3; ++i) {
        B[0][a][i] = g0[i] * dN[a][0];
        B[1][a][i] = g1[i] * dN[a][1];
        B[2][a][i] = g0[i] * dN[a][1] + g1[i] * dN[a][0];
      }
      for (int b = 0; b < 3; ++b) {
        w[0][a][b] = dN[a][0] * dN[b][0];
        w[1][a][b] = dN[a][1] * dN[b][1];
        w[2][a][b] = dN[a][1] * dN[b][0] + dN[a][0] * dN[b][1];
      }
    }
    double Bm[3] = {0, 0, 0}, Bd[3] = {0, 0, 0}; /* B mu, B dx */
    for (int p = 0; p < 3; ++p)
      for (int a = 0; a < 3; ++a)
        for (int i = 0; i < 3; ++i) {
          Bm[p] += B[p][a][i] * M[a][i];
          Bd[p] += B[p][a][i] * D[a][i];
        }
    double CBm[3], CBd[3];
    for (int p = 0; p < 3; ++p) {
      CBm[p] = Cm[p][0] * Bm[0] + Cm[p][1] * Bm[1] + Cm[p][2] * Bm[2];
      CBd[p] = Cm[p][0] * Bd[0] + Cm[p][1] * Bd[1] + Cm[p][2] * Bd[2];
    }
    /* Q_p = sum_ab w_p(a,b) mu_a . dx_b, so mu^T (S+ : dN dN) dx = S+ . Q */
    double Q[3] = {0, 0, 0};
    for (int p = 0; p < 3; ++p)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) Q[p] += w[p][a][b] * orc_dot3(M[a], D[b]);
    double JtQ[3];
    for (int l = 0; l < 3; ++l) JtQ[l] = J[0][l] * Q[0] + J[1][l] * Q[1] + J[2][l] * Q[2];
    for (int b = 0; b < 3; ++b)
      for (int j = 0; j < 3; ++j) {
        /* H_true mu at (b,j) */
        double h = 0.0;
        for (int p = 0; p < 3; ++p) h += B[p][b][j] * CBm[p];
        for (int a = 0; a < 3; ++a) h += (S[0] * w[0][b][a] + S[1] * w[1][b][a] + S[2] * w[2][b][a]) * M[a][j];
        /* d/dc(b,j) of Bm.Cm.Bd + S+.Q */
        double dBm[3], dBd[3], dS[3];
        for (int p = 0; p < 3; ++p) {
          dBm[p] = 0.0;
          dBd[p] = 0.0;
          for (int a = 0; a < 3; ++a) {
            dBm[p] += w[p][a][b] * M[a][j];
            dBd[p] += w[p][a][b] * D[a][j];
          }
          dS[p] = 0.0;
        }
        for (int p = 0; p < 3; ++p)
          for (int q = 0; q < 3; ++q) dS[p] += Cm[p][q] * B[q][b][j]; /* dS/dc(b,j) = Cm dE/dc = Cm B(.,b,j) */
        double gphi = 0.0;
        for (int p = 0; p < 3; ++p) gphi += dBm[p] * CBd[p] + CBm[p] * dBd[p] + JtQ[p] * dS[p];
        xbar[(size_t)n[b] * 3 + j] -= area * (h + gphi);
      }
    const double muW = area * (S[0] * Bm[0] + S[1] * Bm[1] + S[2] * Bm[2]);
    const double phi = area * (Bm[0] * CBd[0] + Bm[1] * CBd[1] + Bm[2] * CBd[2] + Sp[0] * Q[0] + Sp[1] * Q[1] +
                               Sp[2] * Q[2]);
    Ebar[t] -= (muW + phi) / E;
  }
  for (size_t q = 0; q < nquad; ++q) {
    const uint32_t *n = quad + q * 4;
    double C[4][3], c[4][3], w, dw[4][3], ddw[4][4][3][3];
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) {
        C[a][d] = xyz0[(size_t)n[a] * 3 + d];
        c[a][d] = xyz[(size_t)n[a] * 3 + d];
      }
    orc_wdwddw_bend(C, c, stiff_bend, &w, dw, ddw);
    for (int a = 0; a < 4; ++a)
      for (int i = 0; i < 3; ++i) {
        double h = 0.0;
        for (int b = 0; b < 4; ++b)
          for (int j = 0; j < 3; ++j) h += ddw[a][b][i][j] * mu[(size_t)n[b] * 3 + j];
        xbar[(size_t)n[a] * 3 + i] -= h;
      }
  }
}

/* ---- ILU(k) --------------------------------------------------------------- */

/* Initialize_ILUk(m, lev_fill), include/delfem2/ls_ilu_block_sparse.cpp:849-999: */
/* level-of-fill symbolic factorisation, row by row. Row i starts as the      */
/* sorted matrix row (level 0); for each k < i in it (ascending) with         */
/* lev(i,k) + 1 <= lev_fill, each j in row k's upper part with               */
/* lev(k,j) + 1 <= lev_fill and j != i that row i lacks is inserted with      */
/* level max(lev(i,k), lev(k,j)) + 1 (existing entries keep their level).     */
/* lev_fill == -1 takes every fill. Writes row_start_out (nblk+1) and, when   */
/* cap is large enough, col_out and dia_ind; returns the pattern's size.      */
size_t orc_ilu_pattern_k(uint32_t nblk, const uint32_t *row_start, const uint32_t *col_in, int lev_fill,
                         uint32_t *row_start_out, uint32_t *col_out, size_t cap, uint32_t *dia_ind) {
  /* rows kept as arrays of (col, lev), sorted by col */
  size_t tot = 0, acap = (size_t)row_start[nblk] * 2 + 16;
  uint32_t *acol = (uint32_t *)malloc(acap * sizeof(uint32_t));
  uint32_t *alev = (uint32_t *)malloc(acap * sizeof(uint32_t));
  uint32_t *rs = (uint32_t *)malloc(((size_t)nblk + 1) * sizeof(uint32_t));
  uint32_t *dia = (uint32_t *)malloc(((size_t)nblk + 1) * sizeof(uint32_t));
  size_t wcap = 64;
  uint32_t *wc = (uint32_t *)malloc(wcap * sizeof(uint32_t)), *wl = (uint32_t *)malloc(wcap * sizeof(uint32_t));
  rs[0] = 0;
  for (uint32_t i = 0; i < nblk; ++i) {
    /* working row: sorted copy of the matrix row, level 0 */
    size_t n = row_start[i + 1] - row_start[i];
    if (n + 1 > wcap) {
      wcap = 2 * (n + 1);
      wc = (uint32_t *)realloc(wc, wcap * sizeof(uint32_t));
      wl = (uint32_t *)realloc(wl, wcap * sizeof(uint32_t));
    }
    for (size_t t = 0; t < n; ++t) {
      const uint32_t v = col_in[row_start[i] + t];
      size_t b = t;
      while (b > 0 && wc[b - 1] > v) {
        wc[b] = wc[b - 1];
        --b;
      }
      wc[b] = v;
      wl[t] = 0;
    }
    /* walk k ascending over the (growing) row while k < i */
    for (size_t kk = 0; kk < n; ++kk) {
      const uint32_t k = wc[kk], lik = wl[kk];
      if (lev_fill != -1 && (int)lik + 1 > lev_fill) continue;
      if (k >= i) break;
      size_t pos = kk; /* fills of this k are inserted after kk, in column order */
      for (uint32_t s = dia[k]; s < rs[k + 1]; ++s) {
        const uint32_t lkj = alev[s];
        if (lev_fill != -1 && (int)lkj + 1 > lev_fill) continue;
        const uint32_t j = acol[s];
        if (j == i) continue;
        while (pos + 1 < n && wc[pos + 1] < j) ++pos;
        if (pos + 1 < n && wc[pos + 1] == j) continue; /* present: level unchanged */
        if (n + 1 > wcap) {
          wcap *= 2;
          wc = (uint32_t *)realloc(wc, wcap * sizeof(uint32_t));
          wl = (uint32_t *)realloc(wl, wcap * sizeof(uint32_t));
        }
        memmove(wc + pos + 2, wc + pos + 1, (n - pos - 1) * sizeof(uint32_t));
        memmove(wl + pos + 2, wl + pos + 1, (n - pos - 1) * sizeof(uint32_t));
        wc[pos + 1] = j;
        wl[pos + 1] = (lik > lkj ? lik : lkj) + 1;
        ++n;
        ++pos;
      }
    }
    if (tot + n > acap) {
      while (tot + n > acap) acap *= 2;
      acol = (uint32_t *)realloc(acol, acap * sizeof(uint32_t));
      alev = (uint32_t *)realloc(alev, acap * sizeof(uint32_t));
    }
    memcpy(acol + tot, wc, n * sizeof(uint32_t));
    memcpy(alev + tot, wl, n * sizeof(uint32_t));
    dia[i] = (uint32_t)(tot + n);
    for (size_t t = 0; t < n; ++t)
      if (wc[t] > i) {
        dia[i] = (uint32_t)(tot + t);
        break;
      }
    tot += n;
    rs[i + 1] = (uint32_t)tot;
  }
  memcpy(row_start_out, rs, ((size_t)nblk + 1) * sizeof(uint32_t));
  if (col_out && cap >= tot) {
    memcpy(col_out, acol, tot * sizeof(uint32_t));
    memcpy(dia_ind, dia, (size_t)nblk * sizeof(uint32_t));
  }
  free(acol);
  free(alev);
  free(rs);
  free(dia);
  free(wc);
  free(wl);
  return tot;
}

/* CopyValue (ls_ilu_block_sparse.cpp:1009-1047) for an ILU pattern with its */
/* own row offsets (fill-in): zero, scatter each matrix block into the slot  */
/* with the same column, copy the diagonal. lev_fill names the pattern's     */
/* fill level (the pattern itself is given).                                 */
void orc_ilu_copy_value_k(uint32_t nblk, const uint32_t *mrow_start, const uint32_t *col_mat,
                          const double *mat_vcrs, const double *mat_vdia, int lev_fill,
                          const uint32_t *irow_start, const uint32_t *col_ilu, double *ilu_vcrs,
                          double *ilu_vdia) {
  (void)lev_fill;
  memset(ilu_vcrs, 0, (size_t)irow_start[nblk] * 9 * sizeof(double));
  int64_t *slot_of = (int64_t *)malloc((size_t)nblk * sizeof(int64_t));
  for (uint32_t i = 0; i < nblk; ++i) slot_of[i] = -1;
  for (uint32_t i = 0; i < nblk; ++i) {
    for (uint32_t s = irow_start[i]; s < irow_start[i + 1]; ++s) slot_of[col_ilu[s]] = s;
    for (uint32_t s = mrow_start[i]; s < mrow_start[i + 1]; ++s) {
      const int64_t t = slot_of[col_mat[s]];
      if (t >= 0) memcpy(ilu_vcrs + (size_t)t * 9, mat_vcrs + (size_t)s * 9, 9 * sizeof(double));
    }
    for (uint32_t s = irow_start[i]; s < irow_start[i + 1]; ++s) slot_of[col_ilu[s]] = -1;
  }
  free(slot_of);
  memcpy(ilu_vdia, mat_vdia, (size_t)nblk * 9 * sizeof(double));
}

/* ---- Solve_PBiCGStab ------------------------------------------------------- */

/* Solve_PBiCGStab, include/delfem2/vecxitrsol.h:350-437, with the ILU(0)    */
/* preconditioner: x = 0; |r0|^2 < 1e-60 returns [|r0|]; r0* = r, p = r; for */
/* iitr = 1 .. max_niter-1: Mp = M^-1 p, alpha = (r,r0*)/(A Mp, r0*),        */
/* s = r - alpha A Mp, Ms = M^-1 s, omega = (s, A Ms)/(A Ms, A Ms),          */
/* x += alpha Mp + omega Ms, r = s - omega A Ms, push |r|/|r0| (stop below   */
/* tol), beta = (r,r0*) alpha / ((r,r0*)_old omega), p = beta p + r -        */
/* beta omega A Mp. The history holds RELATIVE residuals, one per iteration. */
uint32_t orc_solve_pbicgstab(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, const double *vcrs,
                             const double *vdia, const uint32_t *ilu_row_start, const uint32_t *ilu_col,
                             const uint32_t *dia_ind, const double *ilu_vcrs, const double *ilu_vdia, double *r,
                             double *x, double tol, uint32_t max_iter, double *hist, uint32_t hist_cap) {
  const size_t n = (size_t)nblk * 3;
  uint32_t nh = 0;
  for (size_t k = 0; k < n; ++k) x[k] = 0.0;
  const double sq0 = orc_dot(r, r, n);
  if (sq0 < 1.0e-60) {
    if (hist_cap) hist[0] = sqrt(sq0);
    return 1;
  }
  const double inv0 = 1.0 / sq0;
  /* zero-initialised like the reference's std::vector buffers: MatVec scales  */
  /* y by beta = 0 first, which keeps a NaN an uninitialised y might hold     */
  double *r0 = (double *)calloc(n, sizeof(double)), *p = (double *)calloc(n, sizeof(double));
  double *s = (double *)calloc(n, sizeof(double)), *Mp = (double *)calloc(n, sizeof(double));
  double *AMp = (double *)calloc(n, sizeof(double)), *Ms = (double *)calloc(n, sizeof(double));
  double *AMs = (double *)calloc(n, sizeof(double));
  memcpy(r0, r, n * sizeof(double));
  memcpy(p, r, n * sizeof(double));
  for (uint32_t it = 1; it < max_iter; ++it) {
    memcpy(Mp, p, n * sizeof(double));
    orc_ilu_forward(nblk, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia, Mp);
    orc_ilu_backward(nblk, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, Mp);
    const double r_r2 = orc_dot(r, r0, n);
    orc_bsr_matvec(nblk, row_start, col, vcrs, vdia, AMp, 1.0, Mp, 0.0);
    const double alpha = r_r2 / orc_dot(AMp, r0, n);
    for (size_t k = 0; k < n; ++k) s[k] = r[k] - alpha * AMp[k];
    memcpy(Ms, s, n * sizeof(double));
    orc_ilu_forward(nblk, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia, Ms);
    orc_ilu_backward(nblk, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, Ms);
    orc_bsr_matvec(nblk, row_start, col, vcrs, vdia, AMs, 1.0, Ms, 0.0);
    const double omega = orc_dot(s, AMs, n) / orc_dot(AMs, AMs, n);
    for (size_t k = 0; k < n; ++k) x[k] += alpha * Mp[k];
    for (size_t k = 0; k < n; ++k) x[k] += omega * Ms[k];
    for (size_t k = 0; k < n; ++k) r[k] = s[k] - omega * AMs[k];
    const double ratio = sqrt(orc_dot(r, r, n) * inv0);
    if (nh < hist_cap) hist[nh] = ratio;
    ++nh;
    if (ratio < tol) break;
    const double beta = orc_dot(r, r0, n) * alpha / (r_r2 * omega);
    for (size_t k = 0; k < n; ++k) p[k] = beta * p[k] + r[k] - beta * omega * AMp[k];
  }
  free(r0);
  free(p);
  free(s);
  free(Mp);
  free(AMp);
  free(Ms);
  free(AMs);
  return nh;
}

/* ====================================================================== */
/* Scalar (ndim 1) and 2x2 (ndim 2) blocks. Every function below takes     */
/* ndim in {1, 2, 3}; ndim 3 runs the 3x3 functions above. Values are      */
/* row-major ndim x ndim blocks, vectors ndim entries per block row.       */

/* y = alpha*A*x + beta*y, include/delfem2/ls_block_sparse.cpp:213-224 (y   */
/* scaled by beta first) with MatVec_MatSparseCRS_Blk11 (59-78) and          */
/* MatVec_MatSparseCRS_Blk22 (80-101), in their expression order.            */
void orc_nd_matvec(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                   const double *vcrs, const double *vdia, double *y, double alpha, const double *x,
                   double beta) {
  if (ndim == 3) {
    orc_bsr_matvec(nblk, row_start, col, vcrs, vdia, y, alpha, x, beta);
    return;
  }
  for (size_t i = 0; i < (size_t)nblk * ndim; ++i) y[i] *= beta;
  if (ndim == 1) {
    for (uint32_t i = 0; i < nblk; ++i) {
      for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) y[i] += alpha * vcrs[s] * x[col[s]];
      y[i] += alpha * vdia[i] * x[i];
    }
    return;
  }
  for (uint32_t i = 0; i < nblk; ++i) {
    double *yi = y + (size_t)i * 2;
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) {
      const double *a = vcrs + (size_t)s * 4, *xj = x + (size_t)col[s] * 2;
      yi[0] += alpha * (a[0] * xj[0] + a[1] * xj[1]);
      yi[1] += alpha * (a[2] * xj[0] + a[3] * xj[1]);
    }
    const double *d = vdia + (size_t)i * 4, *xi = x + (size_t)i * 2;
    yi[0] += alpha * (d[0] * xi[0] + d[1] * xi[1]);
    yi[1] += alpha * (d[2] * xi[0] + d[3] * xi[1]);
  }
}

/* Mearge / Merge<nrow,ncol,ndimrow,ndimcol> and Merge<nrow,ncol>,           */
/* include/delfem2/ls_block_sparse.h:209-358, with the same diagonal rule as */
/* orc_merge: a (irow, jcol) pair on one block adds the (irow, irow) block.  */
int orc_nd_merge(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                 double *vdia, uint32_t nnoel, const uint32_t *nodes, const double *emat, uint32_t *merge_buffer) {
  (void)nblk;
  const size_t bb = (size_t)ndim * ndim;
  for (uint32_t a = 0; a < nnoel; ++a) {
    const uint32_t i = nodes[a];
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) merge_buffer[col[s]] = s;
    for (uint32_t b = 0; b < nnoel; ++b) {
      const uint32_t j = nodes[b];
      double *dst;
      if (i == j) {
        dst = vdia + (size_t)i * bb;
      } else {
        if (merge_buffer[j] == ORC_UNSET) return 1;
        dst = vcrs + (size_t)merge_buffer[j] * bb;
      }
      const double *src = emat + ((size_t)a * nnoel + (i == j ? a : b)) * bb;
      for (size_t k = 0; k < bb; ++k) dst[k] += src[k];
    }
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) merge_buffer[col[s]] = ORC_UNSET;
  }
  return 0;
}

/* SetFixedBC (Dia(1), Row, Col), include/delfem2/ls_block_sparse.cpp:397-472 */
/* for any block size.                                                        */
void orc_nd_set_fixed_bc(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                         double *vcrs, double *vdia, const int *bc) {
  const size_t bb = (size_t)ndim * ndim;
  for (uint32_t i = 0; i < nblk; ++i) {
    double *d = vdia + (size_t)i * bb;
    for (uint32_t a = 0; a < ndim; ++a) {
      if (bc[(size_t)i * ndim + a] == 0) continue;
      for (uint32_t b = 0; b < ndim; ++b) { d[a * ndim + b] = 0.0; d[b * ndim + a] = 0.0; }
      d[a * ndim + a] = 1.0;
    }
  }
  for (uint32_t i = 0; i < nblk; ++i)
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s)
      for (uint32_t a = 0; a < ndim; ++a) {
        if (bc[(size_t)i * ndim + a] == 0) continue;
        for (uint32_t b = 0; b < ndim; ++b) vcrs[(size_t)s * bb + a * ndim + b] = 0.0;
      }
  for (uint32_t i = 0; i < nblk; ++i)
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) {
      const uint32_t j = col[s];
      for (uint32_t b = 0; b < ndim; ++b) {
        if (bc[(size_t)j * ndim + b] == 0) continue;
        for (uint32_t a = 0; a < ndim; ++a) vcrs[(size_t)s * bb + a * ndim + b] = 0.0;
      }
    }
}

/* CopyValue, ls_ilu_block_sparse.cpp:1009-1047, any block size, for an ILU  */
/* pattern with its own row offsets (lev_fill names the pattern's fill       */
/* level; the pattern itself is given).                                       */
void orc_nd_ilu_copy_value(uint32_t nblk, uint32_t ndim, const uint32_t *mrow_start, const uint32_t *col_mat,
                           const double *mat_vcrs, const double *mat_vdia, int lev_fill,
                           const uint32_t *irow_start, const uint32_t *col_ilu, double *ilu_vcrs,
                           double *ilu_vdia) {
  (void)lev_fill;
  const size_t bb = (size_t)ndim * ndim;
  memset(ilu_vcrs, 0, (size_t)irow_start[nblk] * bb * sizeof(double));
  int64_t *slot_of = (int64_t *)malloc((size_t)nblk * sizeof(int64_t) + 1);
  for (uint32_t i = 0; i < nblk; ++i) slot_of[i] = -1;
  for (uint32_t i = 0; i < nblk; ++i) {
    for (uint32_t s = irow_start[i]; s < irow_start[i + 1]; ++s) slot_of[col_ilu[s]] = s;
    for (uint32_t s = mrow_start[i]; s < mrow_start[i + 1]; ++s) {
      const int64_t t = slot_of[col_mat[s]];
      if (t >= 0) memcpy(ilu_vcrs + (size_t)t * bb, mat_vcrs + (size_t)s * bb, bb * sizeof(double));
    }
    for (uint32_t s = irow_start[i]; s < irow_start[i + 1]; ++s) slot_of[col_ilu[s]] = -1;
  }
  free(slot_of);
  memcpy(ilu_vdia, mat_vdia, (size_t)nblk * bb * sizeof(double));
}

/* Decompose, ls_ilu_block_sparse.cpp:168-213 (ndim 1) and 214-285 (ndim 2): */
/* as orc_ilu_decompose with A_ij -= A_ik A_kj on 1x1 / 2x2 blocks; the      */
/* pivot is inverted when |d| (ndim 1) or |det| (ndim 2) exceeds 1e-30,      */
/* else counted and left (more than 10 stop with failure); then             */
/* U_ij <- D_i^-1 U_ij.                                                      */
int orc_nd_ilu_decompose(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                         const uint32_t *dia_ind, double *vcrs, double *vdia, int *n_singular) {
  if (ndim == 3) return orc_ilu_decompose(nblk, row_start, col, dia_ind, vcrs, vdia, n_singular);
  const size_t bb = (size_t)ndim * ndim;
  int64_t *slot_of = (int64_t *)malloc((size_t)nblk * sizeof(int64_t) + 1);
  for (uint32_t i = 0; i < nblk; ++i) slot_of[i] = -1;
  int nsing = 0, status = 0;
  for (uint32_t i = 0; i < nblk && status == 0; ++i) {
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) slot_of[col[s]] = s;
    for (uint32_t sk = row_start[i]; sk < dia_ind[i]; ++sk) {
      const uint32_t k = col[sk];
      const double *aik = vcrs + (size_t)sk * bb;
      for (uint32_t sj = dia_ind[k]; sj < row_start[k + 1]; ++sj) {
        const uint32_t j = col[sj];
        double *aij;
        if (j != i) {
          if (slot_of[j] < 0) continue;
          aij = vcrs + (size_t)slot_of[j] * bb;
        } else {
          aij = vdia + (size_t)i * bb;
        }
        const double *akj = vcrs + (size_t)sj * bb;
        if (ndim == 1) {
          aij[0] -= aik[0] * akj[0];
        } else {
          aij[0] -= aik[0] * akj[0] + aik[1] * akj[2];
          aij[1] -= aik[0] * akj[1] + aik[1] * akj[3];
          aij[2] -= aik[2] * akj[0] + aik[3] * akj[2];
          aij[3] -= aik[2] * akj[1] + aik[3] * akj[3];
        }
      }
    }
    double *dii = vdia + (size_t)i * bb;
    if (ndim == 1) {
      if (fabs(dii[0]) > 1.0e-30) {
        dii[0] = 1.0 / dii[0];
      } else if (++nsing > 10) {
        status = 1;
      }
    } else {
      const double det = dii[0] * dii[3] - dii[1] * dii[2];
      if (fabs(det) > 1.0e-30) {
        const double inv_det = 1.0 / det, d0 = dii[0];
        dii[0] = inv_det * dii[3];
        dii[1] = -inv_det * dii[1];
        dii[2] = -inv_det * dii[2];
        dii[3] = inv_det * d0;
      } else if (++nsing > 10) {
        status = 1;
      }
    }
    if (status == 0) {
      for (uint32_t s = dia_ind[i]; s < row_start[i + 1]; ++s) {
        double *u = vcrs + (size_t)s * bb;
        if (ndim == 1) {
          u[0] = u[0] * dii[0];
        } else {
          const double t[4] = {u[0], u[1], u[2], u[3]};
          u[0] = dii[0] * t[0] + dii[1] * t[2];
          u[1] = dii[0] * t[1] + dii[1] * t[3];
          u[2] = dii[2] * t[0] + dii[3] * t[2];
          u[3] = dii[2] * t[1] + dii[3] * t[3];
        }
      }
    }
    for (uint32_t s = row_start[i]; s < row_start[i + 1]; ++s) slot_of[col[s]] = -1;
  }
  free(slot_of);
  if (n_singular) *n_singular = nsing;
  return status;
}

/* ForwardSubstitution, ls_ilu_block_sparse.cpp:502-543 (ndim 1 and 2), in  */
/* place: v_i <- D_i^-1 (v_i - sum_{j<i} L_ij v_j), ascending rows.          */
void orc_nd_ilu_forward(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                        const uint32_t *dia_ind, const double *vcrs, const double *vdia, double *vec) {
  if (ndim == 3) {
    orc_ilu_forward(nblk, row_start, col, dia_ind, vcrs, vdia, vec);
    return;
  }
  for (uint32_t i = 0; i < nblk; ++i) {
    if (ndim == 1) {
      double t = vec[i];
      for (uint32_t s = row_start[i]; s < dia_ind[i]; ++s) t -= vcrs[s] * vec[col[s]];
      vec[i] = vdia[i] * t;
    } else {
      double t0 = vec[(size_t)i * 2], t1 = vec[(size_t)i * 2 + 1];
      for (uint32_t s = row_start[i]; s < dia_ind[i]; ++s) {
        const double *a = vcrs + (size_t)s * 4;
        const double v0 = vec[(size_t)col[s] * 2], v1 = vec[(size_t)col[s] * 2 + 1];
        t0 -= a[0] * v0 + a[1] * v1;
        t1 -= a[2] * v0 + a[3] * v1;
      }
      const double *d = vdia + (size_t)i * 4;
      vec[(size_t)i * 2] = d[0] * t0 + d[1] * t1;
      vec[(size_t)i * 2 + 1] = d[2] * t0 + d[3] * t1;
    }
  }
}

/* BackwardSubstitution, ls_ilu_block_sparse.cpp:680-720 (ndim 1 and 2), in */
/* place: v_i <- v_i - sum_{j>i} U'_ij v_j, descending rows.                 */
void orc_nd_ilu_backward(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                         const uint32_t *dia_ind, const double *vcrs, double *vec) {
  if (ndim == 3) {
    orc_ilu_backward(nblk, row_start, col, dia_ind, vcrs, vec);
    return;
  }
  for (uint32_t ii = nblk; ii-- > 0;) {
    if (ndim == 1) {
      double t = vec[ii];
      for (uint32_t s = dia_ind[ii]; s < row_start[ii + 1]; ++s) t -= vcrs[s] * vec[col[s]];
      vec[ii] = t;
    } else {
      double t0 = vec[(size_t)ii * 2], t1 = vec[(size_t)ii * 2 + 1];
      for (uint32_t s = dia_ind[ii]; s < row_start[ii + 1]; ++s) {
        const double *a = vcrs + (size_t)s * 4;
        const double v0 = vec[(size_t)col[s] * 2], v1 = vec[(size_t)col[s] * 2 + 1];
        t0 -= a[0] * v0 + a[1] * v1;
        t1 -= a[2] * v0 + a[3] * v1;
      }
      vec[(size_t)ii * 2] = t0;
      vec[(size_t)ii * 2 + 1] = t1;
    }
  }
}

/* Solve_PCG (lsitrsol.h:80-148, the semantics of orc_solve_pcg_k) for any  */
/* block size.                                                               */
uint32_t orc_nd_solve_pcg(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                          const double *vcrs, const double *vdia, const uint32_t *ilu_row_start,
                          const uint32_t *ilu_col, const uint32_t *dia_ind, const double *ilu_vcrs,
                          const double *ilu_vdia, double *r, double *x, double tol, uint32_t max_iter,
                          double *hist, uint32_t hist_cap) {
  const size_t n = (size_t)nblk * ndim;
  uint32_t nh = 0;
#define ORC_PUSH(v)                    \
  do {                                 \
    if (nh < hist_cap) hist[nh] = (v); \
    ++nh;                              \
  } while (0)
  for (size_t k = 0; k < n; ++k) x[k] = 0.0;
  const double sq0 = orc_dot(r, r, n);
  ORC_PUSH(sqrt(sq0));
  if (sq0 < 1.0e-30) return nh;
  const double inv_sq0 = 1.0 / sq0;
  double *Pr = (double *)malloc(n * sizeof(double) + 1);
  double *p = (double *)malloc(n * sizeof(double) + 1);
  memcpy(Pr, r, n * sizeof(double));
  orc_nd_ilu_forward(nblk, ndim, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia, Pr);
  orc_nd_ilu_backward(nblk, ndim, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, Pr);
  memcpy(p, Pr, n * sizeof(double));
  double rPr = orc_dot(r, Pr, n);
  int converged = 0;
  for (uint32_t it = 0; it < max_iter; ++it) {
    double *Ap = Pr;
    orc_nd_matvec(nblk, ndim, row_start, col, vcrs, vdia, Ap, 1.0, p, 0.0);
    const double alpha = rPr / orc_dot(p, Ap, n);
    for (size_t k = 0; k < n; ++k) r[k] += -alpha * Ap[k];
    for (size_t k = 0; k < n; ++k) x[k] += alpha * p[k];
    const double sq = orc_dot(r, r, n);
    ORC_PUSH(sqrt(sq));
    if (sqrt(sq * inv_sq0) < tol) { converged = 1; break; }
    memcpy(Pr, r, n * sizeof(double));
    orc_nd_ilu_forward(nblk, ndim, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia, Pr);
    orc_nd_ilu_backward(nblk, ndim, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, Pr);
    const double rPr1 = orc_dot(r, Pr, n);
    const double beta = rPr1 / rPr;
    rPr = rPr1;
    for (size_t k = 0; k < n; ++k) p[k] = beta * p[k] + Pr[k];
  }
  if (!converged) ORC_PUSH(sqrt(orc_dot(r, r, n)));
#undef ORC_PUSH
  free(Pr);
  free(p);
  return nh;
}

/* Solve_PBiCGStab (vecxitrsol.h:350-437, the semantics of                  */
/* orc_solve_pbicgstab) for any block size.                                 */
uint32_t orc_nd_solve_pbicgstab(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col,
                                const double *vcrs, const double *vdia, const uint32_t *ilu_row_start,
                                const uint32_t *ilu_col, const uint32_t *dia_ind, const double *ilu_vcrs,
                                const double *ilu_vdia, double *r, double *x, double tol, uint32_t max_iter,
                                double *hist, uint32_t hist_cap) {
  const size_t n = (size_t)nblk * ndim;
  uint32_t nh = 0;
  for (size_t k = 0; k < n; ++k) x[k] = 0.0;
  const double sq0 = orc_dot(r, r, n);
  if (sq0 < 1.0e-60) {
    if (hist_cap) hist[0] = sqrt(sq0);
    return 1;
  }
  const double inv0 = 1.0 / sq0;
  double *r0 = (double *)calloc(n + 1, sizeof(double)), *p = (double *)calloc(n + 1, sizeof(double));
  double *s = (double *)calloc(n + 1, sizeof(double)), *Mp = (double *)calloc(n + 1, sizeof(double));
  double *AMp = (double *)calloc(n + 1, sizeof(double)), *Ms = (double *)calloc(n + 1, sizeof(double));
  double *AMs = (double *)calloc(n + 1, sizeof(double));
  memcpy(r0, r, n * sizeof(double));
  memcpy(p, r, n * sizeof(double));
  for (uint32_t it = 1; it < max_iter; ++it) {
    memcpy(Mp, p, n * sizeof(double));
    orc_nd_ilu_forward(nblk, ndim, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia, Mp);
    orc_nd_ilu_backward(nblk, ndim, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, Mp);
    const double r_r2 = orc_dot(r, r0, n);
    orc_nd_matvec(nblk, ndim, row_start, col, vcrs, vdia, AMp, 1.0, Mp, 0.0);
    const double alpha = r_r2 / orc_dot(AMp, r0, n);
    for (size_t k = 0; k < n; ++k) s[k] = r[k] - alpha * AMp[k];
    memcpy(Ms, s, n * sizeof(double));
    orc_nd_ilu_forward(nblk, ndim, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, ilu_vdia, Ms);
    orc_nd_ilu_backward(nblk, ndim, ilu_row_start, ilu_col, dia_ind, ilu_vcrs, Ms);
    orc_nd_matvec(nblk, ndim, row_start, col, vcrs, vdia, AMs, 1.0, Ms, 0.0);
    const double omega = orc_dot(s, AMs, n) / orc_dot(AMs, AMs, n);
    for (size_t k = 0; k < n; ++k) x[k] += alpha * Mp[k];
    for (size_t k = 0; k < n; ++k) x[k] += omega * Ms[k];
    for (size_t k = 0; k < n; ++k) r[k] = s[k] - omega * AMs[k];
    const double ratio = sqrt(orc_dot(r, r, n) * inv0);
    if (nh < hist_cap) hist[nh] = ratio;
    ++nh;
    if (ratio < tol) break;
    const double beta = orc_dot(r, r0, n) * alpha / (r_r2 * omega);
    for (size_t k = 0; k < n; ++k) p[k] = beta * p[k] + r[k] - beta * omega * AMp[k];
  }
  free(r0);
  free(p);
  free(s);
  free(Mp);
  free(AMp);
  free(Ms);
  free(AMs);
  return nh;
}

/* ---- scalar and 2-D element assembly ----------------------------------- */

/* EMat_Poisson_Tet3D, include/delfem2/fem_poisson.cpp:163-194:              */
/*   K_e[i][j] = alpha vol (dN_i . dN_j),                                   */
/*   r_e[i] = source vol / 4 - sum_j K_e[i][j] value_j.                      */
void orc_emat_poisson_tet(const double P[4][3], double alpha, double source, const double value[4],
                          double emat[4][4], double eres[4]) {
  const double vol = orc_tet_volume(P[0], P[1], P[2], P[3]);
  double dN[4][3];
  orc_tet_grad(P, vol, dN);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      emat[i][j] = alpha * vol * (dN[i][0] * dN[j][0] + dN[i][1] * dN[j][1] + dN[i][2] * dN[j][2]);
  for (int i = 0; i < 4; ++i) eres[i] = source * vol * 0.25;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) eres[i] -= emat[i][j] * value[j];
}

/* MergeLinSys_Poission_MeshTet3D, include/delfem2/fem_poisson.h:128-162:   */
/* per tet b[node] += r_e and Merge<4,4> of K_e (scalar blocks). Returns 0,  */
/* or 1 when an element block is missing from the pattern.                   */
int orc_assemble_poisson_tet(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                             double *vdia, double *b, double alpha, double source, const double *xyz,
                             const uint32_t *tet, size_t ntet, const double *val) {
  uint32_t *buf = (uint32_t *)malloc((size_t)nblk * sizeof(uint32_t) + 1);
  for (uint32_t i = 0; i < nblk; ++i) buf[i] = ORC_UNSET;
  int status = 0;
  for (size_t e = 0; e < ntet && status == 0; ++e) {
    const uint32_t *ip = tet + e * 4;
    double P[4][3], value[4], emat[4][4], eres[4];
    for (int a = 0; a < 4; ++a) {
      for (int k = 0; k < 3; ++k) P[a][k] = xyz[(size_t)ip[a] * 3 + k];
      value[a] = val ? val[ip[a]] : 0.0;
    }
    orc_emat_poisson_tet(P, alpha, source, value, emat, eres);
    for (int a = 0; a < 4; ++a) b[ip[a]] += eres[a];
    status = orc_nd_merge(nblk, 1, row_start, col, vcrs, vdia, 4, ip, &emat[0][0], buf);
  }
  free(buf);
  return status;
}

/* TriArea2D (femutil.cpp:16-21) and TriDlDx (femutil.cpp:177-197).         */
static double orc_tri_area2(const double *p0, const double *p1, const double *p2) {
  return 0.5 * ((p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1]));
}

static void orc_tri_dldx2(const double P[3][2], double area, double dldx[3][2]) {
  const double t = 0.5 / area;
  dldx[0][0] = t * (P[1][1] - P[2][1]);
  dldx[1][0] = t * (P[2][1] - P[0][1]);
  dldx[2][0] = t * (P[0][1] - P[1][1]);
  dldx[0][1] = t * (P[2][0] - P[1][0]);
  dldx[1][1] = t * (P[0][0] - P[2][0]);
  dldx[2][1] = t * (P[1][0] - P[0][0]);
}

/* EMat_Poisson_Tri2D, include/delfem2/fem_poisson.cpp:15-46:                */
/*   K_e[i][j] = alpha area (dN_i . dN_j), r_e[i] = source area / 3 - K_e v. */
void orc_emat_poisson_tri2(const double P[3][2], double alpha, double source, const double value[3],
                           double emat[3][3], double eres[3]) {
  const double area = orc_tri_area2(P[0], P[1], P[2]);
  double d[3][2];
  orc_tri_dldx2(P, area, d);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) emat[i][j] = alpha * area * (d[i][0] * d[j][0] + d[i][1] * d[j][1]);
  for (int i = 0; i < 3; ++i) eres[i] = source * area * 0.33333333333333333;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) eres[i] -= emat[i][j] * value[j];
}

/* EMat_SolidStaticLinear_Tri2D, include/delfem2/fem_solidlinear.cpp:89-124  */
/* with SetEmat_LinearSolid2<3> (fem_solidlinear.cpp:35-53):                  */
/*   K_e[i][j] = area (lambda dN_i dN_j^T + myu dN_j dN_i^T                   */
/*                     + myu (dN_i . dN_j) I),                                */
/*   r_e[i] = area rho g / 3 - sum_j K_e[i][j] u_j.                           */
void orc_emat_solid_tri2(const double P[3][2], double myu, double lambda, double rho, double gx, double gy,
                         const double disp[3][2], double emat[3][3][2][2], double eres[3][2]) {
  const double area = orc_tri_area2(P[0], P[1], P[2]);
  double d[3][2];
  orc_tri_dldx2(P, area, d);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      emat[i][j][0][0] = area * (lambda + myu) * d[i][0] * d[j][0];
      emat[i][j][0][1] = area * (lambda * d[i][0] * d[j][1] + myu * d[j][0] * d[i][1]);
      emat[i][j][1][0] = area * (lambda * d[i][1] * d[j][0] + myu * d[j][1] * d[i][0]);
      emat[i][j][1][1] = area * (lambda + myu) * d[i][1] * d[j][1];
      const double t = area * myu * (d[i][1] * d[j][1] + d[i][0] * d[j][0]);
      emat[i][j][0][0] += t;
      emat[i][j][1][1] += t;
    }
  for (int i = 0; i < 3; ++i) {
    eres[i][0] = area * rho * gx * 0.33333333333333333;
    eres[i][1] = area * rho * gy * 0.33333333333333333;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      eres[i][0] -= emat[i][j][0][0] * disp[j][0] + emat[i][j][0][1] * disp[j][1];
      eres[i][1] -= emat[i][j][1][0] * disp[j][0] + emat[i][j][1][1] * disp[j][1];
    }
}

/* MergeLinSys_Poission_MeshTri2D (fem_poisson.h:92-127, ndim 1) and         */
/* MergeLinSys_SolidLinear_Static_MeshTri2D (fem_solidlinear.h:155-187,      */
/* ndim 2): per triangle b += r_e and Merge<3,3(,2,2)> of K_e. `val` is the  */
/* nodal value (ndim 1) or displacement (ndim 2), or NULL for zero. Returns  */
/* 0, or 1 when an element block is missing from the pattern.                */
int orc_assemble_tri2(uint32_t nblk, uint32_t ndim, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                      double *vdia, double *b, const double *param, const double *xy, const uint32_t *tri,
                      size_t ntri, const double *val) {
  uint32_t *buf = (uint32_t *)malloc((size_t)nblk * sizeof(uint32_t) + 1);
  for (uint32_t i = 0; i < nblk; ++i) buf[i] = ORC_UNSET;
  int status = 0;
  for (size_t e = 0; e < ntri && status == 0; ++e) {
    const uint32_t *ip = tri + e * 3;
    double P[3][2];
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 2; ++k) P[a][k] = xy[(size_t)ip[a] * 2 + k];
    if (ndim == 1) { /* param: alpha, source */
      double value[3], emat[3][3], eres[3];
      for (int a = 0; a < 3; ++a) value[a] = val ? val[ip[a]] : 0.0;
      orc_emat_poisson_tri2(P, param[0], param[1], value, emat, eres);
      for (int a = 0; a < 3; ++a) b[ip[a]] += eres[a];
      status = orc_nd_merge(nblk, 1, row_start, col, vcrs, vdia, 3, ip, &emat[0][0], buf);
    } else { /* param: myu, lambda, rho, gx, gy */
      double disp[3][2], emat[3][3][2][2], eres[3][2];
      for (int a = 0; a < 3; ++a)
        for (int k = 0; k < 2; ++k) disp[a][k] = val ? val[(size_t)ip[a] * 2 + k] : 0.0;
      orc_emat_solid_tri2(P, param[0], param[1], param[2], param[3], param[4], disp, emat, eres);
      for (int a = 0; a < 3; ++a) {
        b[(size_t)ip[a] * 2] += eres[a][0];
        b[(size_t)ip[a] * 2 + 1] += eres[a][1];
      }
      status = orc_nd_merge(nblk, 2, row_start, col, vcrs, vdia, 3, ip, &emat[0][0][0][0], buf);
    }
  }
  free(buf);
  return status;
}

/* ---- dynamic linear tets (3x3 blocks) ----------------------------------- */

/* MergeLinSys_SolidLinear_BEuler_MeshTet3D, include/delfem2/fem_solidlinear.h: */
/* 381-443, and, with rot (np 3x3 row-major rotations) not NULL,              */
/* MergeLinSys_SolidStiffwarp_BEuler_MeshTet3D (445-530). Per tet: K_e of     */
/* SetEmat_LinearSolid3<4>; stiffness warping makes K_ij <- R_i K_ij R_i^T;   */
/* r_i = vol rho g / 4 - sum_j K_ij w_j with w_j = u_j + dt v_j (warped:      */
/* w_j = P_j + u_j + dt v_j - R_i P_j); then K_ii += rho vol / (4 dt^2) I,    */
/* b_i += r_i / dt and Merge<4,4,3,3>. Returns 0, or 1 on a missing slot.      */
int orc_assemble_tet_beuler(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                            double *vdia, double *b, double myu, double lambda, double rho, const double g[3],
                            double dt, const double *xyz, const uint32_t *tet, size_t ntet, const double *disp,
                            const double *velo, const double *rot) {
  uint32_t *buf = (uint32_t *)malloc((size_t)nblk * sizeof(uint32_t) + 1);
  for (uint32_t i = 0; i < nblk; ++i) buf[i] = ORC_UNSET;
  int status = 0;
  for (size_t e = 0; e < ntet && status == 0; ++e) {
    const uint32_t *n = tet + e * 4;
    double P[4][3], u[4][3], v[4][3], emat[4][4][3][3], vol;
    for (int k = 0; k < 4; ++k)
      for (int d = 0; d < 3; ++d) {
        P[k][d] = xyz[(size_t)n[k] * 3 + d];
        u[k][d] = disp[(size_t)n[k] * 3 + d];
        v[k][d] = velo[(size_t)n[k] * 3 + d];
      }
    orc_emat_tet_linear(P, myu, lambda, emat, &vol);
    if (rot) { /* MatMatTrans3 then MatMat3 (femutil.cpp:96-116): R_i K_ij R_i^T */
      for (int i = 0; i < 4; ++i) {
        const double *R = rot + (size_t)n[i] * 9;
        for (int j = 0; j < 4; ++j) {
          double t[3][3];
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
              t[r][c] = emat[i][j][r][0] * R[c * 3 + 0] + emat[i][j][r][1] * R[c * 3 + 1] +
                        emat[i][j][r][2] * R[c * 3 + 2];
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
              emat[i][j][r][c] = R[r * 3 + 0] * t[0][c] + R[r * 3 + 1] * t[1][c] + R[r * 3 + 2] * t[2][c];
        }
      }
    }
    double res[4][3];
    for (int i = 0; i < 4; ++i) {
      const double *R = rot ? rot + (size_t)n[i] * 9 : NULL;
      for (int a = 0; a < 3; ++a) res[i][a] = vol * rho * g[a] * 0.25;
      for (int j = 0; j < 4; ++j) {
        double w[3];
        if (R) {
          for (int d = 0; d < 3; ++d) {
            const double pj1 = R[d * 3 + 0] * P[j][0] + R[d * 3 + 1] * P[j][1] + R[d * 3 + 2] * P[j][2];
            w[d] = P[j][d] + u[j][d] + dt * v[j][d] - pj1;
          }
        } else {
          for (int d = 0; d < 3; ++d) w[d] = u[j][d] + dt * v[j][d];
        }
        for (int a = 0; a < 3; ++a) {
          res[i][a] -= emat[i][j][a][0] * w[0];
          res[i][a] -= emat[i][j][a][1] * w[1];
          res[i][a] -= emat[i][j][a][2] * w[2];
        }
      }
    }
    const double m = rho * vol * 0.25 / (dt * dt);
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) emat[i][i][a][a] += m;
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) b[(size_t)n[i] * 3 + a] += res[i][a] / dt;
    status = orc_merge(nblk, row_start, col, vcrs, vdia, 4, n, &emat[0][0][0][0], buf);
  }
  free(buf);
  return status;
}

/* MergeLinSys_SolidLinear_NewmarkBeta_MeshTet3D, include/delfem2/           */
/* fem_solidlinear.h:331-379, with EMat_SolidLinear_NewmarkBeta_MeshTet3D     */
/* (fem_solidlinear.cpp:437-488, is_initial_iter true): K_e of                */
/* SetEmat_LinearSolid3<4>, consistent mass M_ij = rho vol / 20 (1 + d_ij) I  */
/* (femutil.cpp:260-280); E_e = M + beta dt^2 K; r = vol rho g / 4 - K u -    */
/* M a - dt K v - dt^2/2 K a (AddEmatEvecScale3, femutil.h:252-268, in that  */
/* order); b += r and Merge<4,4,3,3> of E_e. gamma is unused, as in the       */
/* reference. Returns 0, or 1 on a missing slot.                              */
int orc_assemble_tet_newmark(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs,
                             double *vdia, double *b, double myu, double lambda, double rho, const double g[3],
                             double dt, double gamma, double beta, const double *xyz, const uint32_t *tet,
                             size_t ntet, const double *disp, const double *velo, const double *acc) {
  (void)gamma;
  uint32_t *buf = (uint32_t *)malloc((size_t)nblk * sizeof(uint32_t) + 1);
  for (uint32_t i = 0; i < nblk; ++i) buf[i] = ORC_UNSET;
  int status = 0;
  for (size_t e = 0; e < ntet && status == 0; ++e) {
    const uint32_t *n = tet + e * 4;
    double P[4][3], U[3][4][3], eK[4][4][3][3], eM[4][4][3][3], emat[4][4][3][3], vol;
    const double *src[3] = {disp, velo, acc};
    for (int k = 0; k < 4; ++k)
      for (int d = 0; d < 3; ++d) {
        P[k][d] = xyz[(size_t)n[k] * 3 + d];
        for (int q = 0; q < 3; ++q) U[q][k][d] = src[q][(size_t)n[k] * 3 + d];
      }
    orc_emat_tet_linear(P, myu, lambda, eK, &vol);
    const double mw = rho * vol * 0.05;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) eM[i][j][r][c] = (r == c) ? mw + (i == j ? mw : 0.0) : 0.0;
    const double bdt2 = beta * dt * dt;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) emat[i][j][r][c] = eM[i][j][r][c] + bdt2 * eK[i][j][r][c];
    double res[4][3];
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) res[i][a] = vol * rho * g[a] * 0.25;
    /* (matrix, vector, scale) in the reference's order */
    const double (*mats[4])[4][3][3] = {eK, eM, eK, eK};
    const int vecs[4] = {0, 2, 1, 2};
    const double scales[4] = {-1.0, -1.0, -dt, -0.5 * dt * dt};
    for (int t = 0; t < 4; ++t)
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
          for (int a = 0; a < 3; ++a) {
            const double(*Mt)[3] = mats[t][i][j];
            const double *x = U[vecs[t]][j];
            res[i][a] += scales[t] * (Mt[a][0] * x[0] + Mt[a][1] * x[1] + Mt[a][2] * x[2]);
          }
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) b[(size_t)n[i] * 3 + a] += res[i][a];
    status = orc_merge(nblk, row_start, col, vcrs, vdia, 4, n, &emat[0][0][0][0], buf);
  }
  free(buf);
  return status;
}

/* ---- trilinear hexahedra (Q1, 3x3 blocks) ----------------------------- */

/* Three-point Gauss-Legendre rule as the reference tabulates it (include/  */
/* delfem2/quadrature.h:28-31, in that order, to 15 digits): the Q1 element */
/* asks for table block iGauss = 2, which is the three-point rule.           */
static const double kOrcGauss3[3][2] = {
    {+0.000000000000000, 0.888888888888889}, {-0.774596669241483, 0.555555555555556},
    {+0.774596669241483, 0.555555555555556}};

/* ShapeFunc_Hex8 + HexVox, include/delfem2/femutil.cpp:118-170, 372-421:   */
/* shape values an[8], physical gradients dndx[8][3] and det(dx/dr) at the  */
/* reference point (r0, r1, r2); node k sits at the corner                  */
/* ((k+1)&2 ? + : -, k&2 ? + : -, k&4 ? + : -).                               */
static void orc_hex8_shape(double r0, double r1, double r2, const double P[8][3], double *detjac,
                           double dndx[8][3], double an[8]) {
  static const double sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
                      sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
  double dndr[8][3];
  for (int k = 0; k < 8; ++k) {
    const double a = 1.0 + sx[k] * r0, b = 1.0 + sy[k] * r1, c = 1.0 + sz[k] * r2;
    an[k] = 0.125 * a * b * c;
    dndr[k][0] = sx[k] * 0.125 * b * c;
    dndr[k][1] = sy[k] * 0.125 * a * c;
    dndr[k][2] = sz[k] * 0.125 * a * b;
  }
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int k = 0; k < 8; ++k)
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) J[r][c] += P[k][r] * dndr[k][c];
  const double det = J[0][0] * J[1][1] * J[2][2] + J[1][0] * J[2][1] * J[0][2] + J[2][0] * J[0][1] * J[1][2] -
                     J[0][0] * J[2][1] * J[1][2] - J[1][0] * J[0][1] * J[2][2] - J[2][0] * J[1][1] * J[0][2];
  const double s = 1.0 / det;
  double Ji[3][3];
  Ji[0][0] = s * (J[1][1] * J[2][2] - J[1][2] * J[2][1]);
  Ji[0][1] = s * (J[0][2] * J[2][1] - J[0][1] * J[2][2]);
  Ji[0][2] = s * (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
  Ji[1][0] = s * (J[1][2] * J[2][0] - J[1][0] * J[2][2]);
  Ji[1][1] = s * (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
  Ji[1][2] = s * (J[0][2] * J[1][0] - J[0][0] * J[1][2]);
  Ji[2][0] = s * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  Ji[2][1] = s * (J[0][1] * J[2][0] - J[0][0] * J[2][1]);
  Ji[2][2] = s * (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
  for (int k = 0; k < 8; ++k)
    for (int c = 0; c < 3; ++c)
      dndx[k][c] = dndr[k][0] * Ji[0][c] + dndr[k][1] * Ji[1][c] + dndr[k][2] * Ji[2][c];
  *detjac = det;
}

/* elemMatRes_LinearSolidGravity3_Static_Q1, include/delfem2/               */
/* fem_solidlinear.cpp:238-281: 3x3x3 Gauss points (r0 outer, r2 inner);    */
/* at each, w = det J w0 w1 w2; K += AddEmat_LinearSolid3<8>(w) (55-79) and */
/* r_i += w rho g N_i; then r -= K u.                                        */
void orc_emat_hex_q1(const double P[8][3], double myu, double lambda, double rho, const double g[3],
                     const double disp[8][3], double emat[8][8][3][3], double eres[8][3]) {
  memset(emat, 0, sizeof(double) * 8 * 8 * 9);
  memset(eres, 0, sizeof(double) * 8 * 3);
  for (int i0 = 0; i0 < 3; ++i0)
    for (int i1 = 0; i1 < 3; ++i1)
      for (int i2 = 0; i2 < 3; ++i2) {
        double det, dn[8][3], an[8];
        orc_hex8_shape(kOrcGauss3[i0][0], kOrcGauss3[i1][0], kOrcGauss3[i2][0], P, &det, dn, an);
        const double w = det * kOrcGauss3[i0][1] * kOrcGauss3[i1][1] * kOrcGauss3[i2][1];
        for (int i = 0; i < 8; ++i)
          for (int j = 0; j < 8; ++j) {
            for (int r = 0; r < 3; ++r)
              for (int c = 0; c < 3; ++c)
                emat[i][j][r][c] += w * (lambda * dn[i][r] * dn[j][c] + myu * dn[j][r] * dn[i][c]);
            const double dd = dn[i][0] * dn[j][0] + dn[i][1] * dn[j][1] + dn[i][2] * dn[j][2];
            for (int r = 0; r < 3; ++r) emat[i][j][r][r] += w * myu * dd;
          }
        for (int i = 0; i < 8; ++i)
          for (int r = 0; r < 3; ++r) eres[i][r] += w * rho * g[r] * an[i];
      }
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 8; ++j)
      for (int r = 0; r < 3; ++r)
        eres[i][r] += -1.0 * (emat[i][j][r][0] * disp[j][0] + emat[i][j][r][1] * disp[j][1] +
                              emat[i][j][r][2] * disp[j][2]);
}

/* The element loop of MergeLinSys_LinearSolid3D_Static_Q1                   */
/* (include/delfem2/fem_solidlinear.h:239-276) without its own zeroing of K */
/* and b: per hex b += r_e and Merge<8,8,3,3> of K_e. disp may be NULL.       */
/* Returns 0, or 1 on a missing slot.                                        */
int orc_assemble_hex_q1(uint32_t nblk, const uint32_t *row_start, const uint32_t *col, double *vcrs, double *vdia,
                        double *b, double myu, double lambda, double rho, const double g[3], const double *xyz,
                        const uint32_t *hex, size_t nhex, const double *disp) {
  uint32_t *buf = (uint32_t *)malloc((size_t)nblk * sizeof(uint32_t) + 1);
  for (uint32_t i = 0; i < nblk; ++i) buf[i] = ORC_UNSET;
  int status = 0;
  static double emat[8][8][3][3];
  for (size_t e = 0; e < nhex && status == 0; ++e) {
    const uint32_t *n = hex + e * 8;
    double P[8][3], U[8][3], eres[8][3];
    for (int k = 0; k < 8; ++k)
      for (int d = 0; d < 3; ++d) {
        P[k][d] = xyz[(size_t)n[k] * 3 + d];
        U[k][d] = disp ? disp[(size_t)n[k] * 3 + d] : 0.0;
      }
    orc_emat_hex_q1(P, myu, lambda, rho, g, U, emat, eres);
    for (int k = 0; k < 8; ++k)
      for (int d = 0; d < 3; ++d) b[(size_t)n[k] * 3 + d] += eres[k][d];
    status = orc_merge(nblk, row_start, col, vcrs, vdia, 8, n, &emat[0][0][0][0], buf);
  }
  free(buf);
  return status;
}

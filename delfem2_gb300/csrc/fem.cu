// Linear tets on the device: colour-scheduled, atomic-free assembly of the
// elasticity K and b (3x3 blocks, per-tet Young's modulus), the adjoint element
// term dL/dE, and the scalar Poisson K and b (1x1 blocks).
//
// Layout: tet[4*ntet] node ids, slot[16*ntet] with slot[16e + 4a + b] the
// val_crs_ slot of block (tet[e][a], tet[e][b]) (0xffffffff on the diagonal),
// by_color = tets grouped by colour. Within one colour no two tets share a
// node, so each thread (tet, node a) owns block row a of its tet exclusively.
#include <cstring>

#include "common.cuh"

namespace dfm2g {

constexpr unsigned kDiagSlot = 0xFFFFFFFFu;

// Volume and barycentric-coordinate gradients of a tet (the quantities of
// TetVolume3D / TetDlDx, include/delfem2/femutil.cpp:202-258): dN_k is the
// normal of the face opposite vertex k, scaled by 1/(6 vol), pointing to k.
__device__ __forceinline__ double tet_geometry(const double P[4][3], double dN[4][3]) {
  const double ax = P[1][0] - P[0][0], ay = P[1][1] - P[0][1], az = P[1][2] - P[0][2];
  const double bx = P[2][0] - P[0][0], by = P[2][1] - P[0][1], bz = P[2][2] - P[0][2];
  const double cx = P[3][0] - P[0][0], cy = P[3][1] - P[0][1], cz = P[3][2] - P[0][2];
  const double vol = (ax * (by * cz - cy * bz) - ay * (bx * cz - cx * bz) + az * (bx * cy - cx * by)) / 6.0;
  const double inv6v = 1.0 / (6.0 * vol);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double *a = P[(k + 1) & 3], *b = P[(k + 2) & 3], *c = P[(k + 3) & 3];
    const double ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2];
    const double wx = c[0] - a[0], wy = c[1] - a[1], wz = c[2] - a[2];
    const double s = ((k & 1) ? 1.0 : -1.0) * inv6v;
    dN[k][0] = s * (uy * wz - uz * wy);
    dN[k][1] = s * (uz * wx - ux * wz);
    dN[k][2] = s * (ux * wy - uy * wx);
  }
  return vol;
}

// One thread per (tet of this colour, local node a): block row a of K_e,
// K_e[a][b][r][c] = vol (lambda dN_a[r] dN_b[c] + myu dN_b[r] dN_a[c]
//                        + myu (dN_a . dN_b) delta_rc)
// (AddEmat_LinearSolid3, include/delfem2/fem_solidlinear.cpp:55-79), added into
// the diagonal block or the mapped slot; b_i += rho g vol/4 - sum_b K_ab u_b.
__global__ void __launch_bounds__(128) k_tet_assemble(unsigned n, const unsigned *__restrict__ list,
                                                      const unsigned *__restrict__ tet,
                                                      const unsigned *__restrict__ slot,
                                                      const double *__restrict__ xyz, const double *__restrict__ young,
                                                      double nu, double rho, double gx, double gy, double gz,
                                                      const double *__restrict__ disp, double *vcrs, double *vdia,
                                                      double *rhs) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * 4u) return;
  const unsigned e = list[t >> 2], a = t & 3u;
  unsigned nd[4];
  double P[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    nd[k] = tet[(size_t)e * 4 + k];
#pragma unroll
    for (int d = 0; d < 3; ++d) P[k][d] = xyz[(size_t)nd[k] * 3 + d];
  }
  double dN[4][3];
  const double vol = tet_geometry(P, dN);
  const double E = young[e];
  const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double myu = E / (2.0 * (1.0 + nu));
  const unsigned i = nd[a];
  double res[3] = {vol * rho * gx * 0.25, vol * rho * gy * 0.25, vol * rho * gz * 0.25};
  double da[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) da[d] = (a == 0) ? dN[0][d] : (a == 1) ? dN[1][d] : (a == 2) ? dN[2][d] : dN[3][d];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const double dd = da[0] * dN[b][0] + da[1] * dN[b][1] + da[2] * dN[b][2];
    double k[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        k[r * 3 + c] = vol * (lam * da[r] * dN[b][c] + myu * dN[b][r] * da[c] + (r == c ? myu * dd : 0.0));
    if (disp) {
      const double *u = disp + (size_t)nd[b] * 3;
#pragma unroll
      for (int r = 0; r < 3; ++r) res[r] -= k[r * 3 + 0] * u[0] + k[r * 3 + 1] * u[1] + k[r * 3 + 2] * u[2];
    }
    const unsigned s = slot[(size_t)e * 16 + a * 4 + b];
    double *dst = (s == kDiagSlot) ? vdia + (size_t)i * 9 : vcrs + (size_t)s * 9;
#pragma unroll
    for (int q = 0; q < 9; ++q) dst[q] += k[q];
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) rhs[(size_t)i * 3 + r] += res[r];
}

// One thread per (tet of this colour, local node a): row a of the scalar
// element matrix of EMat_Poisson_Tet3D (include/delfem2/fem_poisson.cpp:
// 163-194), K_e[a][b] = alpha vol (dN_a . dN_b), added to the diagonal (the
// (a, a) entry when both nodes are one block, as the reference's Merge does)
// or to the mapped slot; b_i += source vol / 4 - sum_b K_ab val_b.
__global__ void __launch_bounds__(128) k_tet_poisson(unsigned n, const unsigned *__restrict__ list,
                                                     const unsigned *__restrict__ tet,
                                                     const unsigned *__restrict__ slot,
                                                     const double *__restrict__ xyz, double alpha, double source,
                                                     const double *__restrict__ val, double *vcrs, double *vdia,
                                                     double *rhs) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * 4u) return;
  const unsigned e = list[t >> 2], a = t & 3u;
  unsigned nd[4];
  double P[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    nd[k] = tet[(size_t)e * 4 + k];
#pragma unroll
    for (int d = 0; d < 3; ++d) P[k][d] = xyz[(size_t)nd[k] * 3 + d];
  }
  double dN[4][3];
  const double vol = tet_geometry(P, dN);
  double da[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) da[d] = (a == 0) ? dN[0][d] : (a == 1) ? dN[1][d] : (a == 2) ? dN[2][d] : dN[3][d];
  const double kaa = alpha * vol * (da[0] * da[0] + da[1] * da[1] + da[2] * da[2]);
  const unsigned i = nd[a];
  double res = source * vol * 0.25;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const double k = alpha * vol * (da[0] * dN[b][0] + da[1] * dN[b][1] + da[2] * dN[b][2]);
    if (val) res -= k * val[nd[b]];
    const unsigned s = slot[(size_t)e * 16 + a * 4 + b];
    if (s == kDiagSlot)
      vdia[i] += kaa;
    else
      vcrs[s] += k;
  }
  rhs[i] += res;
}

// Row a of the dynamic linear-tet element matrices (3x3 blocks), one thread
// per (tet of this colour, local node a), K_ab as in k_tet_assemble
// (SetEmat_LinearSolid3<4>, include/delfem2/fem_solidlinear.h:128-153):
//  kBEuler: MergeLinSys_SolidLinear_BEuler_MeshTet3D (fem_solidlinear.h:
//    381-443): r_a = vol rho g/4 - sum_b K_ab (u_b + dt v_b); E_ab = K_ab +
//    rho vol/(4 dt^2) I [a == b]; b_i += r_a / dt.
//  kWarp: MergeLinSys_SolidStiffwarp_BEuler_MeshTet3D (445-530): the same
//    with K_ab <- R_a K_ab R_a^T and u_b + dt v_b <- P_b + u_b + dt v_b -
//    R_a P_b (R_a = rot of node i, row-major).
//  kNewmark: MergeLinSys_SolidLinear_NewmarkBeta_MeshTet3D (331-379, with
//    EMat_SolidLinear_NewmarkBeta_MeshTet3D, fem_solidlinear.cpp:437-488,
//    first iteration): M_ab = rho vol/20 (1 + [a == b]) I, E_ab = M_ab +
//    beta dt^2 K_ab, r_a = vol rho g/4 - K u - M acc - dt K v - dt^2/2 K acc
//    (summed in that order); b_i += r_a.
// E_ab goes to the diagonal (the (a, a) block when both nodes are one block,
// as the reference's Merge does) or to the mapped slot.
enum { kBEuler = 0, kWarp = 1, kNewmark = 2 };

template <int MODE>
__global__ void __launch_bounds__(128) k_tet_dynamic(unsigned n, const unsigned *__restrict__ list,
                                                     const unsigned *__restrict__ tet,
                                                     const unsigned *__restrict__ slot,
                                                     const double *__restrict__ xyz, double myu, double lam,
                                                     double rho, double gx, double gy, double gz, double dt,
                                                     double beta, const double *__restrict__ disp,
                                                     const double *__restrict__ velo,
                                                     const double *__restrict__ acc_or_rot, double *vcrs,
                                                     double *vdia, double *rhs) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * 4u) return;
  const unsigned e = list[t >> 2], a = t & 3u;
  unsigned nd[4];
  double P[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    nd[k] = tet[(size_t)e * 4 + k];
#pragma unroll
    for (int d = 0; d < 3; ++d) P[k][d] = xyz[(size_t)nd[k] * 3 + d];
  }
  double dN[4][3];
  const double vol = tet_geometry(P, dN);
  double da[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) da[d] = (a == 0) ? dN[0][d] : (a == 1) ? dN[1][d] : (a == 2) ? dN[2][d] : dN[3][d];
  const unsigned i = nd[a];
  double R[9];
  if constexpr (MODE == kWarp) {
#pragma unroll
    for (int q = 0; q < 9; ++q) R[q] = acc_or_rot[(size_t)i * 9 + q];
  }
  // K_ab (warped for kWarp)
  auto kblock = [&](int b, double k[9]) {
    const double dd = da[0] * dN[b][0] + da[1] * dN[b][1] + da[2] * dN[b][2];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        k[r * 3 + c] = vol * (lam * da[r] * dN[b][c] + myu * dN[b][r] * da[c] + (r == c ? myu * dd : 0.0));
    if constexpr (MODE == kWarp) {
      double tmp[9];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          tmp[r * 3 + c] = k[r * 3 + 0] * R[c * 3 + 0] + k[r * 3 + 1] * R[c * 3 + 1] + k[r * 3 + 2] * R[c * 3 + 2];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          k[r * 3 + c] = R[r * 3 + 0] * tmp[0 * 3 + c] + R[r * 3 + 1] * tmp[1 * 3 + c] + R[r * 3 + 2] * tmp[2 * 3 + c];
    }
  };
  // E_ab, the block that is merged
  const double mass = (MODE == kNewmark) ? rho * vol * 0.05 : rho * vol * 0.25 / (dt * dt);
  auto eblock = [&](int b, double k[9]) {
    kblock(b, k);
    if constexpr (MODE == kNewmark) {
      const double bdt2 = beta * dt * dt;
      const double m = (b == (int)a) ? mass + mass : mass;
#pragma unroll
      for (int q = 0; q < 9; ++q) k[q] = ((q % 4 == 0) ? m : 0.0) + bdt2 * k[q];
    } else {
      if (b == (int)a) {
        k[0] += mass;
        k[4] += mass;
        k[8] += mass;
      }
    }
  };
  double res[3] = {vol * rho * gx * 0.25, vol * rho * gy * 0.25, vol * rho * gz * 0.25};
  if constexpr (MODE == kNewmark) {
    // (matrix, vector, scale): (K, u, -1), (M, acc, -1), (K, v, -dt), (K, acc, -dt^2/2)
#pragma unroll
    for (int pass = 0; pass < 4; ++pass) {
      const double *vec = pass == 0 ? disp : (pass == 2 ? velo : acc_or_rot);
      const double sc = pass == 2 ? -dt : (pass == 3 ? -0.5 * dt * dt : -1.0);
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const double *x = vec + (size_t)nd[b] * 3;
        if (pass == 1) {
          const double m = (b == (int)a) ? mass + mass : mass;
#pragma unroll
          for (int r = 0; r < 3; ++r) res[r] += sc * (m * x[r]);
        } else {
          double k[9];
          kblock(b, k);
#pragma unroll
          for (int r = 0; r < 3; ++r) res[r] += sc * (k[r * 3 + 0] * x[0] + k[r * 3 + 1] * x[1] + k[r * 3 + 2] * x[2]);
        }
      }
    }
  } else {
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      double k[9], w[3];
      kblock(b, k);
      const double *u = disp + (size_t)nd[b] * 3, *v = velo + (size_t)nd[b] * 3;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if constexpr (MODE == kWarp)
          w[d] = P[b][d] + u[d] + dt * v[d] - (R[d * 3 + 0] * P[b][0] + R[d * 3 + 1] * P[b][1] + R[d * 3 + 2] * P[b][2]);
        else
          w[d] = u[d] + dt * v[d];
      }
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        res[r] -= k[r * 3 + 0] * w[0];
        res[r] -= k[r * 3 + 1] * w[1];
        res[r] -= k[r * 3 + 2] * w[2];
      }
    }
  }
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const unsigned s = slot[(size_t)e * 16 + a * 4 + b];
    double k[9];
    eblock(s == kDiagSlot ? (int)a : b, k);
    double *dst = (s == kDiagSlot) ? vdia + (size_t)i * 9 : vcrs + (size_t)s * 9;
#pragma unroll
    for (int q = 0; q < 9; ++q) dst[q] += k[q];
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) rhs[(size_t)i * 3 + r] += (MODE == kNewmark) ? res[r] : res[r] / dt;
}

// dL/dE_e = -lam_e^T (K_e / E_e) u_e with G(v)[r][c] = sum_k v_k[r] dN_k[c]:
// lam^T K_e u = vol (lambda1 tr(GL) tr(GU) + myu1 (tr(GL GU) + GL:GU)),
// lambda1 = nu/((1+nu)(1-2nu)), myu1 = 1/(2(1+nu)) (the moduli at E = 1).
__global__ void k_tet_dLdE(size_t ntet, const unsigned *__restrict__ tet, const double *__restrict__ xyz, double nu,
                           const double *__restrict__ u, const double *__restrict__ lamv, double *__restrict__ out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < ntet; e += (size_t)gridDim.x * blockDim.x) {
    unsigned nd[4];
    double P[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      nd[k] = tet[e * 4 + k];
#pragma unroll
      for (int d = 0; d < 3; ++d) P[k][d] = xyz[(size_t)nd[k] * 3 + d];
    }
    double dN[4][3];
    const double vol = tet_geometry(P, dN);
    double GL[3][3] = {{0}}, GU[3][3] = {{0}};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const double *lk = lamv + (size_t)nd[k] * 3, *uk = u + (size_t)nd[k] * 3;
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          GL[r][c] += lk[r] * dN[k][c];
          GU[r][c] += uk[r] * dN[k][c];
        }
    }
    const double lam1 = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    const double myu1 = 1.0 / (2.0 * (1.0 + nu));
    double tr_prod = 0.0, frob = 0.0;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        tr_prod += GL[r][c] * GU[c][r];
        frob += GL[r][c] * GU[r][c];
      }
    const double trL = GL[0][0] + GL[1][1] + GL[2][2], trU = GU[0][0] + GU[1][1] + GU[2][2];
    out[e] = -vol * (lam1 * trL * trU + myu1 * (tr_prod + frob));
  }
}

}  // namespace dfm2g

using namespace dfm2g;

extern "C" {

int dfm2g_tetmesh_create(dfm2g_tetmesh *out, dfm2g_bsr m, const double *xyz, size_t np, const unsigned *tet,
                         size_t ntet) try {
  if (!out) return fail(DFM2G_ERR_ARG, "tetmesh_create: null out");
  if (!m || !m->has_pattern) return fail(DFM2G_ERR_STATE, "tetmesh_create: matrix has no pattern");
  if (m->ndim == 2) return fail(DFM2G_ERR_UNSUPPORTED, "tetmesh_create: 2x2 blocks (tets take 1x1 or 3x3)");
  if (np != m->nblk) return fail(DFM2G_ERR_ARG, "tetmesh_create: np (%zu) != matrix blocks (%u)", np, m->nblk);
  if ((ntet && !tet) || (np && !xyz)) return fail(DFM2G_ERR_ARG, "tetmesh_create: null mesh array");
  if (ntet > 0xFFFFFFFFull / 16) return fail(DFM2G_ERR_ARG, "tetmesh_create: too many tets");
  DFM2G_TRY(ensure_context());
  auto *t = new dfm2g_tetmesh_s();
  t->np = np;
  t->ntet = ntet;
  t->nblk = m->nblk;
  t->bsr = m;
  t->pattern_version = m->pattern_version;
  std::vector<unsigned> by_color;
  int s = color_elements(tet, ntet, 4, np, by_color, t->color_start);
  if (s == DFM2G_OK) s = t->xyz.resize(np * 3 + 1);
  if (s == DFM2G_OK) s = t->tet.resize(ntet * 4 + 1);
  if (s == DFM2G_OK) s = t->slot.resize(ntet * 16 + 1);
  if (s == DFM2G_OK) s = t->by_color.resize(ntet + 1);
  if (s == DFM2G_OK && np &&
      cudaMemcpyAsync(t->xyz.p, xyz, sizeof(double) * np * 3, cudaMemcpyHostToDevice, stream()) != cudaSuccess)
    s = fail(DFM2G_ERR_CUDA, "tetmesh_create: copy xyz");
  if (s == DFM2G_OK && ntet &&
      (cudaMemcpyAsync(t->tet.p, tet, sizeof(unsigned) * ntet * 4, cudaMemcpyHostToDevice, stream()) != cudaSuccess ||
       cudaMemcpyAsync(t->by_color.p, by_color.data(), sizeof(unsigned) * ntet, cudaMemcpyHostToDevice, stream()) !=
           cudaSuccess))
    s = fail(DFM2G_ERR_CUDA, "tetmesh_create: copy tets");
  if (s == DFM2G_OK) s = build_slot_map(t->tet.p, ntet, 4, m, t->slot.p);
  if (s != DFM2G_OK) {
    delete t;
    return s;
  }
  *out = t;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_tetmesh_destroy(dfm2g_tetmesh t) try {
  if (t) {
    cudaStreamSynchronize(stream());
    delete t;
  }
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_tetmesh_info(dfm2g_tetmesh t, unsigned *ncolor, size_t *ntet) try {
  if (!t) return fail(DFM2G_ERR_ARG, "null tetmesh");
  if (ncolor) *ncolor = t->color_start.empty() ? 0 : (unsigned)t->color_start.size() - 1;
  if (ntet) *ntet = t->ntet;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_tetmesh_assemble_linear(dfm2g_tetmesh t, dfm2g_bsr m, const double *young, double nu, double rho,
                                  const double *g, const double *disp, double *b, int mem) try {
  if (!t || !m) return fail(DFM2G_ERR_ARG, "assemble: null handle");
  if (m != t->bsr || m->pattern_version != t->pattern_version)
    return fail(DFM2G_ERR_STATE, "assemble: matrix pattern differs from the one the mesh was mapped to");
  DFM2G_TRY(require_3x3(m, "tetmesh_assemble_linear"));
  if (!young || !g || !b) return fail(DFM2G_ERR_ARG, "assemble: null argument");
  VecArg<double> ay, ad, ab;
  DFM2G_TRY(ay.in(young, t->ntet, mem, true));
  if (disp) DFM2G_TRY(ad.in(disp, t->np * 3, mem, true));
  DFM2G_TRY(ab.in(b, t->np * 3, mem, true));
  for (size_t c = 0; c + 1 < t->color_start.size(); ++c) {
    const unsigned n = t->color_start[c + 1] - t->color_start[c];
    k_tet_assemble<<<blocks_for((size_t)n * 4, 128), 128, 0, stream()>>>(
        n, t->by_color.p + t->color_start[c], t->tet.p, t->slot.p, t->xyz.p, ay.dev(), nu, rho, g[0], g[1], g[2],
        disp ? ad.dev() : nullptr, m->vcrs.p, m->vdia.p, ab.dev());
  }
  DFM2G_LAUNCH_CHECK();
  m->f32_valid = false;
  return ab.copy_back();
} catch (...) {
  return host_failure();
}

int dfm2g_tetmesh_assemble_poisson(dfm2g_tetmesh t, dfm2g_bsr m, double alpha, double source, const double *val,
                                   double *b, int mem) try {
  if (!t || !m) return fail(DFM2G_ERR_ARG, "assemble_poisson: null handle");
  if (m != t->bsr || m->pattern_version != t->pattern_version)
    return fail(DFM2G_ERR_STATE, "assemble_poisson: matrix pattern differs from the one the mesh was mapped to");
  if (m->ndim != 1) return fail(DFM2G_ERR_UNSUPPORTED, "assemble_poisson: needs a scalar (ndim 1) matrix");
  if (!b) return fail(DFM2G_ERR_ARG, "assemble_poisson: null b");
  VecArg<double> av, ab;
  if (val) DFM2G_TRY(av.in(val, t->np, mem, true));
  DFM2G_TRY(ab.in(b, t->np, mem, true));
  for (size_t c = 0; c + 1 < t->color_start.size(); ++c) {
    const unsigned n = t->color_start[c + 1] - t->color_start[c];
    k_tet_poisson<<<blocks_for((size_t)n * 4, 128), 128, 0, stream()>>>(
        n, t->by_color.p + t->color_start[c], t->tet.p, t->slot.p, t->xyz.p, alpha, source, val ? av.dev() : nullptr,
        m->vcrs.p, m->vdia.p, ab.dev());
  }
  note_launches((unsigned)(t->color_start.empty() ? 0 : t->color_start.size() - 1));
  DFM2G_LAUNCH_CHECK();
  m->f32_valid = false;
  return ab.copy_back();
} catch (...) {
  return host_failure();
}

static int tet_dynamic(dfm2g_tetmesh t, dfm2g_bsr m, int mode, double myu, double lambda, double rho,
                       const double *g, double dt, double beta, const double *disp, const double *velo,
                       const double *third, double *b, int mem, const char *what) {
  if (!t || !m) return fail(DFM2G_ERR_ARG, "%s: null handle", what);
  if (m != t->bsr || m->pattern_version != t->pattern_version)
    return fail(DFM2G_ERR_STATE, "%s: matrix pattern differs from the one the mesh was mapped to", what);
  DFM2G_TRY(require_3x3(m, what));
  if (!g || !b || !disp || !velo || (mode != kBEuler && !third)) return fail(DFM2G_ERR_ARG, "%s: null argument", what);
  if (!(dt > 0)) return fail(DFM2G_ERR_ARG, "%s: dt must be positive", what);
  VecArg<double> ad, av, a3, ab;
  DFM2G_TRY(ad.in(disp, t->np * 3, mem, true));
  DFM2G_TRY(av.in(velo, t->np * 3, mem, true));
  if (mode != kBEuler) DFM2G_TRY(a3.in(third, t->np * (mode == kWarp ? 9 : 3), mem, true));
  DFM2G_TRY(ab.in(b, t->np * 3, mem, true));
  for (size_t c = 0; c + 1 < t->color_start.size(); ++c) {
    const unsigned n = t->color_start[c + 1] - t->color_start[c];
    const unsigned *list = t->by_color.p + t->color_start[c];
    const unsigned grid = blocks_for((size_t)n * 4, 128);
#define DFM2G_TET_DYN(M)                                                                                            \
  k_tet_dynamic<M><<<grid, 128, 0, stream()>>>(n, list, t->tet.p, t->slot.p, t->xyz.p, myu, lambda, rho, g[0], g[1], \
                                               g[2], dt, beta, ad.dev(), av.dev(),                                  \
                                               mode == kBEuler ? nullptr : a3.dev(), m->vcrs.p, m->vdia.p, ab.dev())
    if (mode == kBEuler)
      DFM2G_TET_DYN(kBEuler);
    else if (mode == kWarp)
      DFM2G_TET_DYN(kWarp);
    else
      DFM2G_TET_DYN(kNewmark);
#undef DFM2G_TET_DYN
  }
  note_launches((unsigned)(t->color_start.empty() ? 0 : t->color_start.size() - 1));
  DFM2G_LAUNCH_CHECK();
  m->f32_valid = false;
  return ab.copy_back();
}

int dfm2g_tetmesh_assemble_beuler(dfm2g_tetmesh t, dfm2g_bsr m, double myu, double lambda, double rho,
                                  const double *g, double dt, const double *disp, const double *velo,
                                  const double *rot, double *b, int mem) try {
  return tet_dynamic(t, m, rot ? kWarp : kBEuler, myu, lambda, rho, g, dt, 0.0, disp, velo, rot, b, mem,
                     "tetmesh_assemble_beuler");
} catch (...) {
  return host_failure();
}

int dfm2g_tetmesh_assemble_newmark(dfm2g_tetmesh t, dfm2g_bsr m, double myu, double lambda, double rho,
                                   const double *g, double dt, double gamma, double beta, const double *disp,
                                   const double *velo, const double *acc, double *b, int mem) try {
  (void)gamma;  // unused by the reference's first-iteration element matrix as well
  return tet_dynamic(t, m, kNewmark, myu, lambda, rho, g, dt, beta, disp, velo, acc, b, mem,
                     "tetmesh_assemble_newmark");
} catch (...) {
  return host_failure();
}

int dfm2g_tetmesh_dLdE(dfm2g_tetmesh t, const double *young, double nu, const double *u, const double *lam,
                       double *dLdE, int mem) try {
  if (!t) return fail(DFM2G_ERR_ARG, "dLdE: null handle");
  (void)young;
  if (!u || !lam || !dLdE) return fail(DFM2G_ERR_ARG, "dLdE: null argument");
  VecArg<double> au, al, ao;
  DFM2G_TRY(au.in(u, t->np * 3, mem, true));
  DFM2G_TRY(al.in(lam, t->np * 3, mem, true));
  DFM2G_TRY(ao.in(dLdE, t->ntet, mem, false));
  if (t->ntet)
    k_tet_dLdE<<<blocks_for(t->ntet, 128, ctx().num_sms * 32), 128, 0, stream()>>>(t->ntet, t->tet.p, t->xyz.p, nu,
                                                                                  au.dev(), al.dev(), ao.dev());
  DFM2G_LAUNCH_CHECK();
  return ao.copy_back();
} catch (...) {
  return host_failure();
}

}  // extern "C"

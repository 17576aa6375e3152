// Trilinear hexahedra (Q1) on the device: colour-scheduled, atomic-free
// assembly of the static linear solid (3x3 blocks), the element loop of
// MergeLinSys_LinearSolid3D_Static_Q1 (include/delfem2/fem_solidlinear.h:
// 239-276) with elemMatRes_LinearSolidGravity3_Static_Q1
// (fem_solidlinear.cpp:238-281).
//
// Layout: xyz[3*np], hex[8*nhex] node ids (ShapeFunc_Hex8's corner order),
// slot[64*nhex] with slot[64e + 8a + b] the val_crs_ slot of block
// (hex[e][a], hex[e][b]) (0xffffffff on the diagonal), by_color = hexes
// grouped by colour (no two hexes of one colour share a node).
//
// One CTA of 128 threads takes two hexes of a colour. Per hex, 27 threads
// evaluate the 27 Gauss points (inverse Jacobian and weight) into shared
// memory; then thread (a, b) accumulates the 3x3 block K_ab over the Gauss
// points in the reference's order, leaves K_ab u_b in shared memory for the
// residual of row a, and adds K_ab to its slot.
#include "common.cuh"

struct dfm2g_hexmesh_s {
  size_t np = 0, nhex = 0;
  unsigned pattern_version = 0;
  const dfm2g_bsr_s *bsr = nullptr;
  dfm2g::DevBuf<double> xyz;
  dfm2g::DevBuf<unsigned> hex, slot, by_color;
  std::vector<unsigned> color_start;
};

namespace dfm2g {

constexpr unsigned kHexDiag = 0xFFFFFFFFu;
constexpr int kHexPerCta = 2;

// The three-point Gauss-Legendre rule as the reference tabulates it
// (include/delfem2/quadrature.h:28-31, in that order): the Q1 element asks for
// the table's block iGauss = 2, the three-point rule.
__constant__ double kGauss3[3][2] = {{+0.000000000000000, 0.888888888888889},
                                     {-0.774596669241483, 0.555555555555556},
                                     {+0.774596669241483, 0.555555555555556}};

// Corner signs of ShapeFunc_Hex8 (include/delfem2/femutil.cpp:372-421).
__device__ __forceinline__ double hx(int k) { return ((k + 1) & 2) ? 1.0 : -1.0; }
__device__ __forceinline__ double hy(int k) { return (k & 2) ? 1.0 : -1.0; }
__device__ __forceinline__ double hz(int k) { return (k & 4) ? 1.0 : -1.0; }

// dN_k/dr at (r0, r1, r2) and N_k.
__device__ __forceinline__ void hex_dndr(int k, double r0, double r1, double r2, double d[3], double *an) {
  const double a = 1.0 + hx(k) * r0, b = 1.0 + hy(k) * r1, c = 1.0 + hz(k) * r2;
  d[0] = hx(k) * 0.125 * b * c;
  d[1] = hy(k) * 0.125 * a * c;
  d[2] = hz(k) * 0.125 * a * b;
  if (an) *an = 0.125 * a * b * c;
}

__global__ void __launch_bounds__(128) k_hex_q1(unsigned n, const unsigned *__restrict__ list,
                                                const unsigned *__restrict__ hexes,
                                                const unsigned *__restrict__ slot, const double *__restrict__ xyz,
                                                double myu, double lam, double rho, double gx, double gy, double gz,
                                                const double *__restrict__ disp, double *vcrs, double *vdia,
                                                double *rhs) {
  __shared__ double sP[kHexPerCta][8][3];
  __shared__ double sJi[kHexPerCta][27][9];
  __shared__ double sW[kHexPerCta][27];
  __shared__ double sK[kHexPerCta][64][9];
  __shared__ double sKu[kHexPerCta][64][3];
  const unsigned h = threadIdx.x >> 6, t = threadIdx.x & 63;
  const unsigned q = blockIdx.x * kHexPerCta + h;  // position in this colour's list
  const bool live = q < n;
  const unsigned e = live ? list[q] : 0u;
  if (live && t < 24) sP[h][t / 3][t % 3] = xyz[(size_t)hexes[(size_t)e * 8 + t / 3] * 3 + t % 3];
  __syncthreads();
  if (live && t < 27) {  // Gauss point t = (i0, i1, i2), i2 fastest
    const int i0 = t / 9, i1 = (t / 3) % 3, i2 = t % 3;
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int k = 0; k < 8; ++k) {
      double d[3];
      hex_dndr(k, kGauss3[i0][0], kGauss3[i1][0], kGauss3[i2][0], d, nullptr);
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) J[r][c] += sP[h][k][r] * d[c];
    }
    const double det = J[0][0] * J[1][1] * J[2][2] + J[1][0] * J[2][1] * J[0][2] + J[2][0] * J[0][1] * J[1][2] -
                       J[0][0] * J[2][1] * J[1][2] - J[1][0] * J[0][1] * J[2][2] - J[2][0] * J[1][1] * J[0][2];
    const double s = 1.0 / det;
    double *Ji = sJi[h][t];
    Ji[0] = s * (J[1][1] * J[2][2] - J[1][2] * J[2][1]);
    Ji[1] = s * (J[0][2] * J[2][1] - J[0][1] * J[2][2]);
    Ji[2] = s * (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
    Ji[3] = s * (J[1][2] * J[2][0] - J[1][0] * J[2][2]);
    Ji[4] = s * (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
    Ji[5] = s * (J[0][2] * J[1][0] - J[0][0] * J[1][2]);
    Ji[6] = s * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    Ji[7] = s * (J[0][1] * J[2][0] - J[0][0] * J[2][1]);
    Ji[8] = s * (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
    sW[h][t] = det * kGauss3[i0][1] * kGauss3[i1][1] * kGauss3[i2][1];
  }
  __syncthreads();
  const int a = (int)(t >> 3), b = (int)(t & 7);
  double k9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  double res[3] = {0, 0, 0};
  if (live) {
    for (int g = 0; g < 27; ++g) {
      const double r0 = kGauss3[g / 9][0], r1 = kGauss3[(g / 3) % 3][0], r2 = kGauss3[g % 3][0];
      const double *Ji = sJi[h][g];
      const double w = sW[h][g];
      double da[3], db[3], xa[3], xb[3], ana;
      hex_dndr(a, r0, r1, r2, da, &ana);
      hex_dndr(b, r0, r1, r2, db, nullptr);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        xa[c] = da[0] * Ji[0 * 3 + c] + da[1] * Ji[1 * 3 + c] + da[2] * Ji[2 * 3 + c];
        xb[c] = db[0] * Ji[0 * 3 + c] + db[1] * Ji[1 * 3 + c] + db[2] * Ji[2 * 3 + c];
      }
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) k9[r * 3 + c] += w * (lam * xa[r] * xb[c] + myu * xb[r] * xa[c]);
      const double dd = xa[0] * xb[0] + xa[1] * xb[1] + xa[2] * xb[2];
      k9[0] += w * myu * dd;
      k9[4] += w * myu * dd;
      k9[8] += w * myu * dd;
      if (b == 0) {
        res[0] += w * rho * gx * ana;
        res[1] += w * rho * gy * ana;
        res[2] += w * rho * gz * ana;
      }
    }
#pragma unroll
    for (int q9 = 0; q9 < 9; ++q9) sK[h][t][q9] = k9[q9];
    const double *u = disp ? disp + (size_t)hexes[(size_t)e * 8 + b] * 3 : nullptr;
#pragma unroll
    for (int r = 0; r < 3; ++r)
      sKu[h][t][r] = u ? (k9[r * 3 + 0] * u[0] + k9[r * 3 + 1] * u[1] + k9[r * 3 + 2] * u[2]) : 0.0;
  }
  __syncthreads();
  if (!live) return;
  const unsigned i = hexes[(size_t)e * 8 + a];
  const unsigned s = slot[(size_t)e * 64 + t];
  const double *src = sK[h][s == kHexDiag ? a * 8 + a : t];
  double *dst = (s == kHexDiag) ? vdia + (size_t)i * 9 : vcrs + (size_t)s * 9;
#pragma unroll
  for (int q9 = 0; q9 < 9; ++q9) dst[q9] += src[q9];
  if (b == 0) {
    for (int bb = 0; bb < 8; ++bb)
#pragma unroll
      for (int r = 0; r < 3; ++r) res[r] += -1.0 * sKu[h][a * 8 + bb][r];
#pragma unroll
    for (int r = 0; r < 3; ++r) rhs[(size_t)i * 3 + r] += res[r];
  }
}

}  // namespace dfm2g

using namespace dfm2g;

extern "C" {

int dfm2g_hexmesh_create(dfm2g_hexmesh *out, dfm2g_bsr m, const double *xyz, size_t np, const unsigned *hex,
                         size_t nhex) try {
  if (!out) return fail(DFM2G_ERR_ARG, "hexmesh_create: null out");
  if (!m || !m->has_pattern) return fail(DFM2G_ERR_STATE, "hexmesh_create: matrix has no pattern");
  DFM2G_TRY(require_3x3(m, "hexmesh_create"));
  if (np != m->nblk) return fail(DFM2G_ERR_ARG, "hexmesh_create: np (%zu) != matrix blocks (%u)", np, m->nblk);
  if ((nhex && !hex) || (np && !xyz)) return fail(DFM2G_ERR_ARG, "hexmesh_create: null mesh array");
  if (nhex > 0xFFFFFFFFull / 64) return fail(DFM2G_ERR_ARG, "hexmesh_create: too many hexes");
  for (size_t e = 0; e < nhex; ++e)
    for (int a = 0; a < 8; ++a)
      for (int a0 = 0; a0 < a; ++a0)
        if (hex[e * 8 + a] == hex[e * 8 + a0])
          return fail(DFM2G_ERR_ARG, "hexmesh_create: hex %zu repeats node %u", e, hex[e * 8 + a]);
  DFM2G_TRY(ensure_context());
  auto *t = new dfm2g_hexmesh_s();
  t->np = np;
  t->nhex = nhex;
  t->bsr = m;
  t->pattern_version = m->pattern_version;
  std::vector<unsigned> by_color;
  int s = color_elements(hex, nhex, 8, np, by_color, t->color_start);
  if (s == DFM2G_OK) s = t->xyz.resize(np * 3 + 1);
  if (s == DFM2G_OK) s = t->hex.resize(nhex * 8 + 1);
  if (s == DFM2G_OK) s = t->slot.resize(nhex * 64 + 1);
  if (s == DFM2G_OK) s = t->by_color.resize(nhex + 1);
  if (s == DFM2G_OK && np &&
      cudaMemcpyAsync(t->xyz.p, xyz, sizeof(double) * np * 3, cudaMemcpyHostToDevice, stream()) != cudaSuccess)
    s = fail(DFM2G_ERR_CUDA, "hexmesh_create: copy xyz");
  if (s == DFM2G_OK && nhex &&
      (cudaMemcpyAsync(t->hex.p, hex, sizeof(unsigned) * nhex * 8, cudaMemcpyHostToDevice, stream()) != cudaSuccess ||
       cudaMemcpyAsync(t->by_color.p, by_color.data(), sizeof(unsigned) * nhex, cudaMemcpyHostToDevice, stream()) !=
           cudaSuccess))
    s = fail(DFM2G_ERR_CUDA, "hexmesh_create: copy hexes");
  if (s == DFM2G_OK) s = build_slot_map(t->hex.p, nhex, 8, m, t->slot.p);
  if (s != DFM2G_OK) {
    delete t;
    return s;
  }
  *out = t;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_hexmesh_destroy(dfm2g_hexmesh t) try {
  if (t) {
    cudaStreamSynchronize(stream());
    delete t;
  }
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_hexmesh_assemble_linear(dfm2g_hexmesh t, dfm2g_bsr m, double myu, double lambda, double rho,
                                  const double *g, const double *disp, double *b, int mem) try {
  if (!t || !m) return fail(DFM2G_ERR_ARG, "hexmesh_assemble_linear: null handle");
  if (m != t->bsr || m->pattern_version != t->pattern_version)
    return fail(DFM2G_ERR_STATE, "hexmesh_assemble_linear: matrix pattern differs from the one the mesh was mapped to");
  DFM2G_TRY(require_3x3(m, "hexmesh_assemble_linear"));
  if (!g || !b) return fail(DFM2G_ERR_ARG, "hexmesh_assemble_linear: null argument");
  VecArg<double> ad, ab;
  if (disp) DFM2G_TRY(ad.in(disp, t->np * 3, mem, true));
  DFM2G_TRY(ab.in(b, t->np * 3, mem, true));
  for (size_t c = 0; c + 1 < t->color_start.size(); ++c) {
    const unsigned n = t->color_start[c + 1] - t->color_start[c];
    k_hex_q1<<<blocks_for(n, kHexPerCta), 64 * kHexPerCta, 0, stream()>>>(
        n, t->by_color.p + t->color_start[c], t->hex.p, t->slot.p, t->xyz.p, myu, lambda, rho, g[0], g[1], g[2],
        disp ? ad.dev() : nullptr, m->vcrs.p, m->vdia.p, ab.dev());
  }
  note_launches((unsigned)(t->color_start.empty() ? 0 : t->color_start.size() - 1));
  DFM2G_LAUNCH_CHECK();
  m->f32_valid = false;
  return ab.copy_back();
} catch (...) {
  return host_failure();
}

}  // extern "C"

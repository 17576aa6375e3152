// Linear triangles in 2-D on the device: colour-scheduled, atomic-free
// assembly of the scalar Poisson system (1x1 blocks) and of the static linear
// solid (2x2 blocks).
//
// Layout: xy[2*np], tri[3*ntri] node ids, slot[9*ntri] with slot[9e + 3a + b]
// the val_crs_ slot of block (tri[e][a], tri[e][b]) (0xffffffff on the
// diagonal), by_color = triangles grouped by colour. Within one colour no two
// triangles share a node, so a thread (triangle, node a) owns block row a of
// its triangle.
#include "common.cuh"

struct dfm2g_trimesh2_s {
  size_t np = 0, ntri = 0;
  unsigned pattern_version = 0;
  const dfm2g_bsr_s *bsr = nullptr;
  dfm2g::DevBuf<double> xy;
  dfm2g::DevBuf<unsigned> tri, slot, by_color;
  std::vector<unsigned> color_start;
};

namespace dfm2g {

constexpr unsigned kDiagSlot2 = 0xFFFFFFFFu;

// TriArea2D and TriDlDx (include/delfem2/femutil.cpp:16-21, 177-197):
// signed area and the gradients of the barycentric coordinates.
__device__ __forceinline__ double tri2_geometry(const double P[3][2], double d[3][2]) {
  const double area = 0.5 * ((P[1][0] - P[0][0]) * (P[2][1] - P[0][1]) - (P[2][0] - P[0][0]) * (P[1][1] - P[0][1]));
  const double t = 0.5 / area;
  d[0][0] = t * (P[1][1] - P[2][1]);
  d[1][0] = t * (P[2][1] - P[0][1]);
  d[2][0] = t * (P[0][1] - P[1][1]);
  d[0][1] = t * (P[2][0] - P[1][0]);
  d[1][1] = t * (P[0][0] - P[2][0]);
  d[2][1] = t * (P[1][0] - P[0][0]);
  return area;
}

__device__ __forceinline__ void tri2_load(unsigned e, const unsigned *__restrict__ tri, const double *__restrict__ xy,
                                          unsigned nd[3], double P[3][2]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    nd[k] = tri[(size_t)e * 3 + k];
    P[k][0] = xy[(size_t)nd[k] * 2];
    P[k][1] = xy[(size_t)nd[k] * 2 + 1];
  }
}

// Row a of EMat_Poisson_Tri2D (include/delfem2/fem_poisson.cpp:15-46):
// K_e[a][b] = alpha area (dN_a . dN_b); b_i += source area / 3 - sum_b K_ab val_b.
// A pair (a, b) on one block adds K_aa, as the reference's Merge does.
__global__ void __launch_bounds__(128) k_tri2_poisson(unsigned n, const unsigned *__restrict__ list,
                                                      const unsigned *__restrict__ tri,
                                                      const unsigned *__restrict__ slot,
                                                      const double *__restrict__ xy, double alpha, double source,
                                                      const double *__restrict__ val, double *vcrs, double *vdia,
                                                      double *rhs) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * 3u) return;
  const unsigned e = list[t / 3u], a = t % 3u;
  unsigned nd[3];
  double P[3][2], d[3][2];
  tri2_load(e, tri, xy, nd, P);
  const double area = tri2_geometry(P, d);
  const double da0 = a == 0 ? d[0][0] : a == 1 ? d[1][0] : d[2][0];
  const double da1 = a == 0 ? d[0][1] : a == 1 ? d[1][1] : d[2][1];
  const double kaa = alpha * area * (da0 * da0 + da1 * da1);
  const unsigned i = nd[a];
  double res = source * area * 0.33333333333333333;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const double k = alpha * area * (da0 * d[b][0] + da1 * d[b][1]);
    if (val) res -= k * val[nd[b]];
    const unsigned s = slot[(size_t)e * 9 + a * 3 + b];
    if (s == kDiagSlot2)
      vdia[i] += kaa;
    else
      vcrs[s] += k;
  }
  rhs[i] += res;
}

// Block (a, b) of SetEmat_LinearSolid2<3> (include/delfem2/fem_solidlinear.cpp:
// 35-53) with w = area.
__device__ __forceinline__ void solid2_block(double lam, double myu, double w, double ax, double ay, double bx,
                                             double by, double k[4]) {
  const double diag = w * myu * (ay * by + ax * bx);
  k[0] = w * (lam + myu) * ax * bx + diag;
  k[1] = w * (lam * ax * by + myu * bx * ay);
  k[2] = w * (lam * ay * bx + myu * by * ax);
  k[3] = w * (lam + myu) * ay * by + diag;
}

// Row a of EMat_SolidStaticLinear_Tri2D (include/delfem2/fem_solidlinear.cpp:
// 89-124); b_i += area rho g / 3 - sum_b K_ab u_b.
__global__ void __launch_bounds__(128) k_tri2_solid(unsigned n, const unsigned *__restrict__ list,
                                                    const unsigned *__restrict__ tri,
                                                    const unsigned *__restrict__ slot,
                                                    const double *__restrict__ xy, double myu, double lam, double rho,
                                                    double gx, double gy, const double *__restrict__ disp,
                                                    double *vcrs, double *vdia, double *rhs) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * 3u) return;
  const unsigned e = list[t / 3u], a = t % 3u;
  unsigned nd[3];
  double P[3][2], d[3][2];
  tri2_load(e, tri, xy, nd, P);
  const double area = tri2_geometry(P, d);
  const double ax = a == 0 ? d[0][0] : a == 1 ? d[1][0] : d[2][0];
  const double ay = a == 0 ? d[0][1] : a == 1 ? d[1][1] : d[2][1];
  double kaa[4];
  solid2_block(lam, myu, area, ax, ay, ax, ay, kaa);
  const unsigned i = nd[a];
  double r0 = area * rho * gx * 0.33333333333333333, r1 = area * rho * gy * 0.33333333333333333;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    double k[4];
    solid2_block(lam, myu, area, ax, ay, d[b][0], d[b][1], k);
    if (disp) {
      const double u0 = disp[(size_t)nd[b] * 2], u1 = disp[(size_t)nd[b] * 2 + 1];
      r0 -= k[0] * u0 + k[1] * u1;
      r1 -= k[2] * u0 + k[3] * u1;
    }
    const unsigned s = slot[(size_t)e * 9 + a * 3 + b];
    double *dst = (s == kDiagSlot2) ? vdia + (size_t)i * 4 : vcrs + (size_t)s * 4;
    const double *src = (s == kDiagSlot2) ? kaa : k;
#pragma unroll
    for (int q = 0; q < 4; ++q) dst[q] += src[q];
  }
  rhs[(size_t)i * 2] += r0;
  rhs[(size_t)i * 2 + 1] += r1;
}

}  // namespace dfm2g

using namespace dfm2g;

static int check_mesh2(dfm2g_trimesh2 t, dfm2g_bsr m, unsigned ndim, const char *what) {
  if (!t || !m) return fail(DFM2G_ERR_ARG, "%s: null handle", what);
  if (m != t->bsr || m->pattern_version != t->pattern_version)
    return fail(DFM2G_ERR_STATE, "%s: matrix pattern differs from the one the mesh was mapped to", what);
  if (m->ndim != ndim) return fail(DFM2G_ERR_UNSUPPORTED, "%s: needs %ux%u blocks (matrix has ndim %u)", what, ndim,
                                   ndim, m->ndim);
  return DFM2G_OK;
}

extern "C" {

int dfm2g_trimesh2_create(dfm2g_trimesh2 *out, dfm2g_bsr m, const double *xy, size_t np, const unsigned *tri,
                          size_t ntri) try {
  if (!out) return fail(DFM2G_ERR_ARG, "trimesh2_create: null out");
  if (!m || !m->has_pattern) return fail(DFM2G_ERR_STATE, "trimesh2_create: matrix has no pattern");
  if (m->ndim == 3) return fail(DFM2G_ERR_UNSUPPORTED, "trimesh2_create: 3x3 blocks (2-D triangles take 1x1 or 2x2)");
  if (np != m->nblk) return fail(DFM2G_ERR_ARG, "trimesh2_create: np (%zu) != matrix blocks (%u)", np, m->nblk);
  if ((ntri && !tri) || (np && !xy)) return fail(DFM2G_ERR_ARG, "trimesh2_create: null mesh array");
  if (ntri > 0xFFFFFFFFull / 9) return fail(DFM2G_ERR_ARG, "trimesh2_create: too many triangles");
  DFM2G_TRY(ensure_context());
  auto *t = new dfm2g_trimesh2_s();
  t->np = np;
  t->ntri = ntri;
  t->bsr = m;
  t->pattern_version = m->pattern_version;
  std::vector<unsigned> by_color;
  int s = color_elements(tri, ntri, 3, np, by_color, t->color_start);
  if (s == DFM2G_OK) s = t->xy.resize(np * 2 + 1);
  if (s == DFM2G_OK) s = t->tri.resize(ntri * 3 + 1);
  if (s == DFM2G_OK) s = t->slot.resize(ntri * 9 + 1);
  if (s == DFM2G_OK) s = t->by_color.resize(ntri + 1);
  if (s == DFM2G_OK && np &&
      cudaMemcpyAsync(t->xy.p, xy, sizeof(double) * np * 2, cudaMemcpyHostToDevice, stream()) != cudaSuccess)
    s = fail(DFM2G_ERR_CUDA, "trimesh2_create: copy xy");
  if (s == DFM2G_OK && ntri &&
      (cudaMemcpyAsync(t->tri.p, tri, sizeof(unsigned) * ntri * 3, cudaMemcpyHostToDevice, stream()) != cudaSuccess ||
       cudaMemcpyAsync(t->by_color.p, by_color.data(), sizeof(unsigned) * ntri, cudaMemcpyHostToDevice, stream()) !=
           cudaSuccess))
    s = fail(DFM2G_ERR_CUDA, "trimesh2_create: copy triangles");
  if (s == DFM2G_OK) s = build_slot_map(t->tri.p, ntri, 3, m, t->slot.p);
  if (s != DFM2G_OK) {
    delete t;
    return s;
  }
  *out = t;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_trimesh2_destroy(dfm2g_trimesh2 t) try {
  if (t) {
    cudaStreamSynchronize(stream());
    delete t;
  }
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_trimesh2_assemble_poisson(dfm2g_trimesh2 t, dfm2g_bsr m, double alpha, double source, const double *val,
                                    double *b, int mem) try {
  DFM2G_TRY(check_mesh2(t, m, 1, "trimesh2_assemble_poisson"));
  if (!b) return fail(DFM2G_ERR_ARG, "trimesh2_assemble_poisson: null b");
  VecArg<double> av, ab;
  if (val) DFM2G_TRY(av.in(val, t->np, mem, true));
  DFM2G_TRY(ab.in(b, t->np, mem, true));
  for (size_t c = 0; c + 1 < t->color_start.size(); ++c) {
    const unsigned n = t->color_start[c + 1] - t->color_start[c];
    k_tri2_poisson<<<blocks_for((size_t)n * 3, 128), 128, 0, stream()>>>(
        n, t->by_color.p + t->color_start[c], t->tri.p, t->slot.p, t->xy.p, alpha, source, val ? av.dev() : nullptr,
        m->vcrs.p, m->vdia.p, ab.dev());
  }
  note_launches((unsigned)(t->color_start.empty() ? 0 : t->color_start.size() - 1));
  DFM2G_LAUNCH_CHECK();
  m->f32_valid = false;
  return ab.copy_back();
} catch (...) {
  return host_failure();
}

int dfm2g_trimesh2_assemble_solid_linear(dfm2g_trimesh2 t, dfm2g_bsr m, double myu, double lambda, double rho,
                                         double gx, double gy, const double *disp, double *b, int mem) try {
  DFM2G_TRY(check_mesh2(t, m, 2, "trimesh2_assemble_solid_linear"));
  if (!b) return fail(DFM2G_ERR_ARG, "trimesh2_assemble_solid_linear: null b");
  VecArg<double> ad, ab;
  if (disp) DFM2G_TRY(ad.in(disp, t->np * 2, mem, true));
  DFM2G_TRY(ab.in(b, t->np * 2, mem, true));
  for (size_t c = 0; c + 1 < t->color_start.size(); ++c) {
    const unsigned n = t->color_start[c + 1] - t->color_start[c];
    k_tri2_solid<<<blocks_for((size_t)n * 3, 128), 128, 0, stream()>>>(
        n, t->by_color.p + t->color_start[c], t->tri.p, t->slot.p, t->xy.p, myu, lambda, rho, gx, gy,
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

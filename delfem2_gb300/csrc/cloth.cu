// Implicit cloth on the device: StVK constant-strain-triangle membrane with the
// 2x2 positive-definite projection of the stress, quadratic bending over the
// quads of adjacent triangle pairs, the backward-Euler step of
// StepTime_InternalDynamicsILU (include/delfem2/cloth_internal.h:179-269), and
// its hand-written adjoint with checkpoint-and-recompute rollouts.
//
// Layout (all device): tri[3 ntri], quad[4 nquad] node ids; tri_slot[9 ntri]
// and quad_slot[16 nquad] val_crs_ slot ids (0xffffffff on the diagonal);
// tri_rest[8 ntri] = {area, m00, m11, m01, G0.G0, G1.G1, G0.G1, 0} with m the
// contravariant rest metric; quad_rest[8 nquad] = {K0..K3, 1/((A0+A1) L^2),
// 0, 0, 0} (cotangent weights of WdWddW_Bend). Elements are grouped by a
// greedy colouring (no two elements of one colour share a vertex), so a thread
// owns the block rows / vertex entries it writes: no atomics, deterministic.
//
// CST quantities per triangle, in terms of the deformed edges g0 = c1 - c0,
// g1 = c2 - c0 (fem_stvk.cpp:267-374):
//   strain  E = (E00, E11, 2 E01) = ((g0.g0 - G0.G0) / 2, (g1.g1 - G1.G1) / 2,
//           g0.g1 - G0.G1); stress S = Cm E; W = A E.S / 2;
//   dW_a    = A sum_p S_p beta_a^p with beta_a^0 = dN_a0 g0, beta_a^1 = dN_a1 g1,
//             beta_a^2 = dN_a1 g0 + dN_a0 g1, dN = {(-1,-1), (1,0), (0,1)};
//   K_ab    = A sum_pq beta_a^p Cm_pq beta_b^q^T + A (S+ : dN_a dN_b) I with S+
//             the projected stress (MakePositiveDefinite_Sim22, 211-264).
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

struct dfm2g_cloth_s {
  size_t np = 0, ntri = 0, nquad = 0;
  unsigned nblk = 0;
  unsigned pattern_version = 0;
  const dfm2g_bsr_s *bsr = nullptr;
  dfm2g::DevBuf<double> xyz0;
  dfm2g::DevBuf<unsigned> tri, quad, tri_slot, quad_slot, tri_by_color, quad_by_color;
  dfm2g::DevBuf<double> tri_rest, quad_rest;
  std::vector<unsigned> tri_color_start, quad_color_start;
  // step scratch (3 np each) and the per-element energies of merge
  dfm2g::DevBuf<double> dW, b, dx, mu, dxbar, welem, wsum;
  // rollout record for the adjoint
  struct Rollout {
    bool valid = false;
    unsigned nsteps = 0, every = 0, max_iter = 0;
    int solver = 0;
    double nu = 0, stiff = 0, g[3] = {0, 0, 0}, mass = 0, dt = 0, tol = 0;
    dfm2g::DevBuf<int> bc;
    dfm2g::DevBuf<double> young;
    dfm2g::DevBuf<double> ckpt;  // (nsteps/every + 1) x (x, v), 6 np each
    dfm2g::DevBuf<double> seg;   // (every + 1) x positions of one segment
  } ro;
};

namespace dfm2g {

namespace {

constexpr unsigned kDiagSlot = 0xFFFFFFFFu;

__device__ __forceinline__ double dot3(const double *a, const double *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
__device__ __forceinline__ void cross3(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// Rest constants of one CST (the rest-shape part of WdWddW_CST): area,
// contravariant metric (m00, m11, m01) and covariant metric (G00, G11, G01).
__global__ void k_tri_rest(size_t ntri, const unsigned *__restrict__ tri, const double *__restrict__ X,
                           double *__restrict__ rest) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < ntri; t += (size_t)gridDim.x * blockDim.x) {
    const double *P0 = X + (size_t)tri[t * 3] * 3, *P1 = X + (size_t)tri[t * 3 + 1] * 3,
                 *P2 = X + (size_t)tri[t * 3 + 2] * 3;
    double G0[3], G1[3], n[3];
    for (int d = 0; d < 3; ++d) {
      G0[d] = P1[d] - P0[d];
      G1[d] = P2[d] - P0[d];
    }
    cross3(G0, G1, n);
    const double nl = sqrt(dot3(n, n));
    for (int d = 0; d < 3; ++d) n[d] /= nl;
    double U0[3], U1[3];
    cross3(G1, n, U0);
    cross3(n, G0, U1);
    const double s0 = 1.0 / dot3(U0, G0), s1 = 1.0 / dot3(U1, G1);
    for (int d = 0; d < 3; ++d) {
      U0[d] *= s0;
      U1[d] *= s1;
    }
    double *r = rest + t * 8;
    r[0] = 0.5 * nl;
    r[1] = dot3(U0, U0);
    r[2] = dot3(U1, U1);
    r[3] = dot3(U1, U0);
    r[4] = dot3(G0, G0);
    r[5] = dot3(G1, G1);
    r[6] = dot3(G0, G1);
    r[7] = 0.0;
  }
}

__device__ __forceinline__ double tri_area(const double *a, const double *b, const double *c) {
  double u[3], w[3], n[3];
  for (int d = 0; d < 3; ++d) {
    u[d] = b[d] - a[d];
    w[d] = c[d] - a[d];
  }
  cross3(u, w, n);
  return 0.5 * sqrt(dot3(n, n));
}

// Rest constants of one bending quad (WdWddW_Bend, fem_quadratic_bending.cpp:
// 57-83): cotangent weights K of the hinge (2,3) and 1/((A0+A1) L^2).
__global__ void k_quad_rest(size_t nquad, const unsigned *__restrict__ quad, const double *__restrict__ X,
                            double *__restrict__ rest) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nquad; q += (size_t)gridDim.x * blockDim.x) {
    const double *C[4];
    for (int a = 0; a < 4; ++a) C[a] = X + (size_t)quad[q * 4 + a] * 3;
    const double A0 = tri_area(C[0], C[2], C[3]), A1 = tri_area(C[1], C[3], C[2]);
    double e23[3], e02[3], e03[3], e12[3], e13[3];
    for (int d = 0; d < 3; ++d) {
      e23[d] = C[3][d] - C[2][d];
      e02[d] = C[2][d] - C[0][d];
      e03[d] = C[3][d] - C[0][d];
      e12[d] = C[2][d] - C[1][d];
      e13[d] = C[3][d] - C[1][d];
    }
    const double L = sqrt(dot3(e23, e23));
    const double H0 = 2.0 * A0 / L, H1 = 2.0 * A1 / L;
    const double c023 = -dot3(e02, e23) / H0, c032 = dot3(e03, e23) / H0;
    const double c123 = -dot3(e12, e23) / H1, c132 = dot3(e13, e23) / H1;
    double *r = rest + q * 8;
    r[0] = -c023 - c032;
    r[1] = -c123 - c132;
    r[2] = c032 + c132;
    r[3] = c023 + c123;
    r[4] = 1.0 / ((A0 + A1) * L * L);
    r[5] = r[6] = r[7] = 0.0;
  }
}

// The projection of MakePositiveDefinite_Sim22 (fem_stvk.cpp:211-264) on the
// symmetric [[s0, s2], [s2, s1]], eigenvalues b - e <= b + e: unchanged when
// b - e > 1e-20, zero when b + e < 0, else l u u^T with l = b + e and u the
// normalised longer row of S - l I (zero when both rows are < 1e-10 long).
__device__ __forceinline__ void pd_sim22(const double s[3], double o[3]) {
  const double b = 0.5 * (s[0] + s[1]);
  const double e = sqrt(0.25 * (s[0] - s[1]) * (s[0] - s[1]) + s[2] * s[2]);
  if (b - e > 1.0e-20) {
    o[0] = s[0];
    o[1] = s[1];
    o[2] = s[2];
    return;
  }
  if (b + e < 0) {
    o[0] = o[1] = o[2] = 0.0;
    return;
  }
  const double l = b + e;
  const double t0x = s[0] - l, t0y = s[2], t1x = s[2], t1y = s[1] - l;
  const double q0 = t0x * t0x + t0y * t0y, q1 = t1x * t1x + t1y * t1y;
  const bool first = q0 > q1;
  const double qq = first ? q0 : q1;
  if (qq < 1.0e-20) {
    o[0] = o[1] = o[2] = 0.0;
    return;
  }
  const double inv = 1.0 / sqrt(qq);
  const double u0 = (first ? t0x : t1x) * inv, u1 = (first ? t0y : t1y) * inv;
  o[0] = l * u0 * u0;
  o[1] = l * u1 * u1;
  o[2] = l * u0 * u1;
}

// J^T Q for the Jacobian J = d pd_sim22(s) / ds (3x3), branch by branch: I,
// 0, or the derivative of l u u^T through l = b + e and u = t/|t| with t the
// chosen row of S - l I (the branch choice is locally constant).
__device__ __forceinline__ void pd_sim22_jt(const double s[3], const double Q[3], double o[3]) {
  const double b = 0.5 * (s[0] + s[1]), d = 0.5 * (s[0] - s[1]);
  const double e = sqrt(0.25 * (s[0] - s[1]) * (s[0] - s[1]) + s[2] * s[2]);
  o[0] = o[1] = o[2] = 0.0;
  if (b - e > 1.0e-20) {
    o[0] = Q[0];
    o[1] = Q[1];
    o[2] = Q[2];
    return;
  }
  if (b + e < 0) return;
  const double l = b + e;
  const double t0x = s[0] - l, t0y = s[2], t1x = s[2], t1y = s[1] - l;
  const double q0 = t0x * t0x + t0y * t0y, q1 = t1x * t1x + t1y * t1y;
  const bool first = q0 > q1;
  const double qq = first ? q0 : q1;
  if (qq < 1.0e-20) return;  // also covers e == 0 (then t == 0)
  const double gl[3] = {0.5 + 0.5 * d / e, 0.5 - 0.5 * d / e, s[2] / e};
  double dt[2][3];
  for (int k = 0; k < 3; ++k) {
    if (first) {
      dt[0][k] = (k == 0 ? 1.0 : 0.0) - gl[k];
      dt[1][k] = (k == 2 ? 1.0 : 0.0);
    } else {
      dt[0][k] = (k == 2 ? 1.0 : 0.0);
      dt[1][k] = (k == 1 ? 1.0 : 0.0) - gl[k];
    }
  }
  const double r = sqrt(qq);
  const double u0 = (first ? t0x : t1x) / r, u1 = (first ? t0y : t1y) / r;
  for (int k = 0; k < 3; ++k) {
    const double ut = u0 * dt[0][k] + u1 * dt[1][k];
    const double du0 = (dt[0][k] - u0 * ut) / r, du1 = (dt[1][k] - u1 * ut) / r;
    const double j0 = gl[k] * u0 * u0 + 2.0 * l * u0 * du0;
    const double j1 = gl[k] * u1 * u1 + 2.0 * l * u1 * du1;
    const double j2 = gl[k] * u0 * u1 + l * (u1 * du0 + u0 * du1);
    o[k] = Q[0] * j0 + Q[1] * j1 + Q[2] * j2;
  }
}

// Per-triangle state at the current positions: moduli, deformed edges,
// constitutive matrix (symmetric, fem_stvk.cpp:320-339) and stress.
struct CstState {
  double A, g0[3], g1[3], Cm[3][3], E[3], S[3];
};

__device__ __forceinline__ void cst_state(const double *__restrict__ rest, const double *c0, const double *c1,
                                          const double *c2, double lam, double myu, CstState &st) {
  st.A = rest[0];
  const double m00 = rest[1], m11 = rest[2], m01 = rest[3];
  for (int d = 0; d < 3; ++d) {
    st.g0[d] = c1[d] - c0[d];
    st.g1[d] = c2[d] - c0[d];
  }
  st.E[0] = 0.5 * (dot3(st.g0, st.g0) - rest[4]);
  st.E[1] = 0.5 * (dot3(st.g1, st.g1) - rest[5]);
  st.E[2] = dot3(st.g0, st.g1) - rest[6];
  const double l2 = lam + 2.0 * myu;
  st.Cm[0][0] = l2 * m00 * m00;
  st.Cm[1][1] = l2 * m11 * m11;
  st.Cm[0][1] = st.Cm[1][0] = lam * m00 * m11 + 2.0 * myu * m01 * m01;
  st.Cm[0][2] = st.Cm[2][0] = l2 * m00 * m01;
  st.Cm[1][2] = st.Cm[2][1] = l2 * m11 * m01;
  st.Cm[2][2] = lam * m01 * m01 + myu * (m00 * m11 + m01 * m01);
  for (int p = 0; p < 3; ++p) st.S[p] = st.Cm[p][0] * st.E[0] + st.Cm[p][1] * st.E[1] + st.Cm[p][2] * st.E[2];
}

__constant__ double kDN[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};

__device__ __forceinline__ void cst_beta(const CstState &st, int a, double beta[3][3]) {
  const double n0 = kDN[a][0], n1 = kDN[a][1];
  for (int d = 0; d < 3; ++d) {
    beta[0][d] = n0 * st.g0[d];
    beta[1][d] = n1 * st.g1[d];
    beta[2][d] = n1 * st.g0[d] + n0 * st.g1[d];
  }
}

__device__ __forceinline__ void lame(double E, double nu, double &lam, double &myu) {
  lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  myu = E / (2.0 * (1.0 + nu));
}

// One thread per (triangle of this colour, local vertex a): block row a of the
// projected Hessian added into K, dW_a added into dW, the element energy
// (a == 0) into welem[t] when welem is given.
__global__ void __launch_bounds__(128) k_tri_assemble(unsigned n, const unsigned *__restrict__ list,
                                                      const unsigned *__restrict__ tri,
                                                      const unsigned *__restrict__ slot,
                                                      const double *__restrict__ rest, const double *__restrict__ x,
                                                      const double *__restrict__ young, double nu, double *vcrs,
                                                      double *vdia, double *dW, double *welem) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n * 3u) return;
  const unsigned t = list[tid / 3], a = tid % 3;
  const unsigned nd[3] = {tri[(size_t)t * 3], tri[(size_t)t * 3 + 1], tri[(size_t)t * 3 + 2]};
  double lam, myu;
  lame(young[t], nu, lam, myu);
  CstState st;
  cst_state(rest + (size_t)t * 8, x + (size_t)nd[0] * 3, x + (size_t)nd[1] * 3, x + (size_t)nd[2] * 3, lam, myu,
            st);
  double Sp[3];
  pd_sim22(st.S, Sp);
  double ba[3][3], ga[3][3];
  cst_beta(st, a, ba);
  for (int q = 0; q < 3; ++q)
    for (int d = 0; d < 3; ++d) ga[q][d] = st.Cm[q][0] * ba[0][d] + st.Cm[q][1] * ba[1][d] + st.Cm[q][2] * ba[2][d];
  const unsigned i = nd[a];
  for (int bn = 0; bn < 3; ++bn) {
    double bb[3][3];
    cst_beta(st, bn, bb);
    const double G = st.A * (Sp[0] * kDN[a][0] * kDN[bn][0] +
                             Sp[2] * (kDN[a][0] * kDN[bn][1] + kDN[a][1] * kDN[bn][0]) +
                             Sp[1] * kDN[a][1] * kDN[bn][1]);
    const unsigned s = slot[(size_t)t * 9 + a * 3 + bn];
    double *dst = (s == kDiagSlot) ? vdia + (size_t)i * 9 : vcrs + (size_t)s * 9;
    for (int r = 0; r < 3; ++r)
      for (int cc = 0; cc < 3; ++cc) {
        const double v = st.A * (ga[0][r] * bb[0][cc] + ga[1][r] * bb[1][cc] + ga[2][r] * bb[2][cc]);
        dst[r * 3 + cc] += v + (r == cc ? G : 0.0);
      }
  }
  for (int d = 0; d < 3; ++d)
    dW[(size_t)i * 3 + d] += st.A * (st.S[0] * ba[0][d] + st.S[1] * ba[1][d] + st.S[2] * ba[2][d]);
  if (welem && a == 0) welem[t] = 0.5 * st.A * (st.E[0] * st.S[0] + st.E[1] * st.S[1] + st.E[2] * st.S[2]);
}

// One thread per (quad of this colour, local vertex a): K_ab += s K_a K_b I,
// dW_a += s K_a sum_b K_b c_b with s = stiff / ((A0+A1) L^2); the reported
// energy is c.dW (fem_quadratic_bending.cpp:96-106).
__global__ void __launch_bounds__(128) k_quad_assemble(unsigned n, const unsigned *__restrict__ list,
                                                       const unsigned *__restrict__ quad,
                                                       const unsigned *__restrict__ slot,
                                                       const double *__restrict__ rest,
                                                       const double *__restrict__ x, double stiff, double *vcrs,
                                                       double *vdia, double *dW, double *welem) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n * 4u) return;
  const unsigned q = list[tid >> 2], a = tid & 3u;
  const double *r = rest + (size_t)q * 8;
  const double s = stiff * r[4];
  double y[3] = {0, 0, 0};
  unsigned nd[4];
  for (int b = 0; b < 4; ++b) {
    nd[b] = quad[(size_t)q * 4 + b];
    for (int d = 0; d < 3; ++d) y[d] += r[b] * x[(size_t)nd[b] * 3 + d];
  }
  const double Ka = r[a];
  const unsigned i = nd[a];
  for (int b = 0; b < 4; ++b) {
    const unsigned sl = slot[(size_t)q * 16 + a * 4 + b];
    double *dst = (sl == kDiagSlot) ? vdia + (size_t)i * 9 : vcrs + (size_t)sl * 9;
    const double v = s * Ka * r[b];
    dst[0] += v;
    dst[4] += v;
    dst[8] += v;
  }
  for (int d = 0; d < 3; ++d) dW[(size_t)i * 3 + d] += s * Ka * y[d];
  if (welem && a == 0) welem[q] = s * dot3(y, y);
}

// Fixed-order sum of n values by one block (energies of merge).
__global__ void k_sum_one_block(size_t n, const double *__restrict__ v, double *out) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) acc += v[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (unsigned w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out += sh[0];
}

// b = -(dW - m g) + m v / dt (zero at fixed DOFs); K_dia += m / dt^2 I
// (cloth_internal.h:76-92, 225-237). b may be null (the adjoint only needs A).
__global__ void k_cloth_rhs(unsigned np, const double *__restrict__ dW, const double *__restrict__ v,
                            const int *__restrict__ bc, double mass, double dt, double gx, double gy, double gz,
                            double *__restrict__ b, double *__restrict__ vdia) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const double m_dt2 = mass / (dt * dt);
    vdia[(size_t)i * 9 + 0] += m_dt2;
    vdia[(size_t)i * 9 + 4] += m_dt2;
    vdia[(size_t)i * 9 + 8] += m_dt2;
    if (b) {
      const double g[3] = {gx, gy, gz};
      for (int d = 0; d < 3; ++d) {
        const size_t k = (size_t)i * 3 + d;
        b[k] = bc[k] != 0 ? 0.0 : -(dW[k] - mass * g[d]) + mass * v[k] / dt;
      }
    }
  }
}

// Free DOFs: x += dx, v = dx / dt (cloth_internal.h:259-268).
__global__ void k_cloth_update(size_t n, const double *__restrict__ dx, const int *__restrict__ bc, double dt,
                               double *__restrict__ x, double *__restrict__ v) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    if (bc[k] != 0) continue;
    x[k] += dx[k];
    v[k] = dx[k] / dt;
  }
}

// Adjoint seed of one step: dxbar = P (xbar + vbar / dt); dx = P (x1 - x0).
__global__ void k_adj_seed(size_t n, const double *__restrict__ xbar, const double *__restrict__ vbar,
                           const int *__restrict__ bc, double dt, const double *__restrict__ x0,
                           const double *__restrict__ x1, double *__restrict__ dxbar, double *__restrict__ dx) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const bool fixed = bc[k] != 0;
    dxbar[k] = fixed ? 0.0 : xbar[k] + vbar[k] / dt;
    dx[k] = fixed ? 0.0 : x1[k] - x0[k];
  }
}

// vbar_k = m mu / dt at free DOFs (db/dv = M/dt), vbar_{k+1} kept at fixed
// DOFs (v is not updated there).
__global__ void k_adj_vbar(size_t n, const double *__restrict__ mu, const int *__restrict__ bc, double mass,
                           double dt, double *__restrict__ vbar) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    if (bc[k] == 0) vbar[k] = mass * mu[k] / dt;
}

// Adjoint terms of one triangle (thread per triangle of this colour). With
// w^0 = w_1 - w_0, w^1 = w_2 - w_0 and dE(w) = (g0.w^0, g1.w^1, g0.w^1 + g1.w^0)
// (= B w, the linearised strain):
//   H mu       = A B^T Cm dE(mu) + A (S : dN dN) mu             (unprojected)
//   phi        = mu^T A_e dx = A dE(mu).Cm dE(dx) + A S+.Q,
//                Q = (mu^0.dx^0, mu^1.dx^1, mu^0.dx^1 + mu^1.dx^0)
//   grad phi   = A [dE'(mu)^T sd + dE'(dx)^T smu] + A dE'^T Cm J^T Q
// with J = dS+/dS; all gathered on the edges (f0 on g0, f1 on g1) and sent to
// the vertices as (-f0 - f1, f0, f1). xbar -= H mu + grad phi;
// Ebar_t -= (A S.dE(mu) + phi) / E_t (S, S+ and A_e are linear in E_t).
__global__ void __launch_bounds__(128) k_tri_adjoint(unsigned n, const unsigned *__restrict__ list,
                                                     const unsigned *__restrict__ tri,
                                                     const double *__restrict__ rest,
                                                     const double *__restrict__ x, const double *__restrict__ young,
                                                     double nu, const double *__restrict__ mu,
                                                     const double *__restrict__ dx, double *__restrict__ xbar,
                                                     double *__restrict__ Ebar) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n) return;
  const unsigned t = list[tid];
  const unsigned nd[3] = {tri[(size_t)t * 3], tri[(size_t)t * 3 + 1], tri[(size_t)t * 3 + 2]};
  const double Et = young[t];
  double lam, myu;
  lame(Et, nu, lam, myu);
  CstState st;
  cst_state(rest + (size_t)t * 8, x + (size_t)nd[0] * 3, x + (size_t)nd[1] * 3, x + (size_t)nd[2] * 3, lam, myu,
            st);
  double m0[3], m1[3], d0[3], d1[3];
  for (int k = 0; k < 3; ++k) {
    const double mz = mu[(size_t)nd[0] * 3 + k], dz = dx[(size_t)nd[0] * 3 + k];
    m0[k] = mu[(size_t)nd[1] * 3 + k] - mz;
    m1[k] = mu[(size_t)nd[2] * 3 + k] - mz;
    d0[k] = dx[(size_t)nd[1] * 3 + k] - dz;
    d1[k] = dx[(size_t)nd[2] * 3 + k] - dz;
  }
  const double em[3] = {dot3(st.g0, m0), dot3(st.g1, m1), dot3(st.g0, m1) + dot3(st.g1, m0)};
  const double ed[3] = {dot3(st.g0, d0), dot3(st.g1, d1), dot3(st.g0, d1) + dot3(st.g1, d0)};
  double sm[3], sd[3];
  for (int p = 0; p < 3; ++p) {
    sm[p] = st.Cm[p][0] * em[0] + st.Cm[p][1] * em[1] + st.Cm[p][2] * em[2];
    sd[p] = st.Cm[p][0] * ed[0] + st.Cm[p][1] * ed[1] + st.Cm[p][2] * ed[2];
  }
  double Sp[3], jq[3], eta[3];
  pd_sim22(st.S, Sp);
  const double Q[3] = {dot3(m0, d0), dot3(m1, d1), dot3(m0, d1) + dot3(m1, d0)};
  pd_sim22_jt(st.S, Q, jq);
  for (int p = 0; p < 3; ++p) eta[p] = st.Cm[p][0] * jq[0] + st.Cm[p][1] * jq[1] + st.Cm[p][2] * jq[2];
  double f0[3], f1[3];
  for (int k = 0; k < 3; ++k) {
    // H mu (true Hessian)
    f0[k] = sm[0] * st.g0[k] + sm[2] * st.g1[k] + st.S[0] * m0[k] + st.S[2] * m1[k];
    f1[k] = sm[1] * st.g1[k] + sm[2] * st.g0[k] + st.S[2] * m0[k] + st.S[1] * m1[k];
    // grad of the material part of phi
    f0[k] += sd[0] * m0[k] + sd[2] * m1[k] + sm[0] * d0[k] + sm[2] * d1[k];
    f1[k] += sd[1] * m1[k] + sd[2] * m0[k] + sm[1] * d1[k] + sm[2] * d0[k];
    // grad of the geometric part of phi (through S+)
    f0[k] += eta[0] * st.g0[k] + eta[2] * st.g1[k];
    f1[k] += eta[1] * st.g1[k] + eta[2] * st.g0[k];
    f0[k] *= st.A;
    f1[k] *= st.A;
  }
  for (int k = 0; k < 3; ++k) {
    xbar[(size_t)nd[0] * 3 + k] += f0[k] + f1[k];
    xbar[(size_t)nd[1] * 3 + k] -= f0[k];
    xbar[(size_t)nd[2] * 3 + k] -= f1[k];
  }
  const double muW = st.A * (st.S[0] * em[0] + st.S[1] * em[1] + st.S[2] * em[2]);
  const double phi = st.A * (em[0] * sd[0] + em[1] * sd[1] + em[2] * sd[2] + Sp[0] * Q[0] + Sp[1] * Q[1] +
                             Sp[2] * Q[2]);
  Ebar[t] -= (muW + phi) / Et;
}

// Bending adjoint term (thread per quad of this colour): xbar_a -= s K_a sum_b
// K_b mu_b (constant Hessian, no third-derivative term, no E dependence).
__global__ void k_quad_adjoint(unsigned n, const unsigned *__restrict__ list, const unsigned *__restrict__ quad,
                               const double *__restrict__ rest, double stiff, const double *__restrict__ mu,
                               double *__restrict__ xbar) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n) return;
  const unsigned q = list[tid];
  const double *r = rest + (size_t)q * 8;
  const double s = stiff * r[4];
  unsigned nd[4];
  double y[3] = {0, 0, 0};
  for (int b = 0; b < 4; ++b) {
    nd[b] = quad[(size_t)q * 4 + b];
    for (int d = 0; d < 3; ++d) y[d] += r[b] * mu[(size_t)nd[b] * 3 + d];
  }
  for (int a = 0; a < 4; ++a)
    for (int d = 0; d < 3; ++d) xbar[(size_t)nd[a] * 3 + d] -= s * r[a] * y[d];
}

}  // namespace

// ---- host helpers -------------------------------------------------------------

static int check_cloth(dfm2g_cloth c, dfm2g_bsr m) {
  if (!c || !m) return fail(DFM2G_ERR_ARG, "cloth: null handle");
  DFM2G_TRY(require_3x3(m, "cloth"));
  if (m != c->bsr || m->pattern_version != c->pattern_version)
    return fail(DFM2G_ERR_STATE, "cloth: matrix pattern differs from the one the mesh was mapped to");
  return DFM2G_OK;
}

// K += projected Hessians, dW += gradients (device arrays); welem: energies
// per element (ntri + nquad) or null.
static int cloth_assemble(dfm2g_cloth c, dfm2g_bsr m, const double *x, const double *young, double nu,
                          double stiff, double *dW, double *welem) {
  unsigned nl = 0;
  for (size_t k = 0; k + 1 < c->tri_color_start.size(); ++k) {
    const unsigned n = c->tri_color_start[k + 1] - c->tri_color_start[k];
    k_tri_assemble<<<blocks_for((size_t)n * 3, 128), 128, 0, stream()>>>(
        n, c->tri_by_color.p + c->tri_color_start[k], c->tri.p, c->tri_slot.p, c->tri_rest.p, x, young, nu,
        m->vcrs.p, m->vdia.p, dW, welem);
    ++nl;
  }
  for (size_t k = 0; k + 1 < c->quad_color_start.size(); ++k) {
    const unsigned n = c->quad_color_start[k + 1] - c->quad_color_start[k];
    k_quad_assemble<<<blocks_for((size_t)n * 4, 128), 128, 0, stream()>>>(
        n, c->quad_by_color.p + c->quad_color_start[k], c->quad.p, c->quad_slot.p, c->quad_rest.p, x, stiff,
        m->vcrs.p, m->vdia.p, dW, welem ? welem + c->ntri : nullptr);
    ++nl;
  }
  note_launches(nl);
  DFM2G_LAUNCH_CHECK();
  m->f32_valid = false;
  return DFM2G_OK;
}

struct StepArgs {
  const int *bc;
  const double *young;
  double nu, stiff, g[3], mass, dt, tol;
  unsigned max_iter;
  int solver;
};

// A = M/dt^2 + ddW(x) clamped, factorised; b (when wanted) the step's rhs.
static int cloth_system(dfm2g_cloth c, dfm2g_bsr m, dfm2g_ilu p, const double *x, const double *v,
                        const StepArgs &a, double *b) {
  const size_t n = c->np * 3;
  DFM2G_TRY(dfm2g_bsr_set_zero(m));
  DFM2G_CUDA(cudaMemsetAsync(c->dW.p, 0, sizeof(double) * n, stream()));
  DFM2G_TRY(cloth_assemble(c, m, x, a.young, a.nu, a.stiff, c->dW.p, nullptr));
  k_cloth_rhs<<<blocks_for(c->np, 256, ctx().num_sms * 8), 256, 0, stream()>>>(
      (unsigned)c->np, c->dW.p, v, a.bc, a.mass, a.dt, a.g[0], a.g[1], a.g[2], b, m->vdia.p);
  note_launches(1);
  DFM2G_LAUNCH_CHECK();
  DFM2G_TRY(dfm2g_bsr_set_fixed_bc(m, a.bc, DFM2G_MEM_DEVICE));
  DFM2G_TRY(dfm2g_ilu_copy_value(p, m));
  int ns = 0;
  DFM2G_TRY(dfm2g_ilu_decompose(p, &ns));
  return DFM2G_OK;
}

// Solves A y = rhs (rhs kept) with the step's solver; not converging is not
// an error (the reference continues with the last iterate).
static int cloth_solve(dfm2g_bsr m, dfm2g_ilu p, double *rhs, double *y, double *scratch, const StepArgs &a,
                       dfm2g_solve_stats *st) {
  const size_t n = (size_t)m->nblk * 3;
  int s;
  if (a.solver == DFM2G_CLOTH_PCG_MIXED) {
    s = dfm2g_solve_pcg_mixed_reliable(m, p, rhs, y, a.tol, 0.1, a.max_iter, DFM2G_MEM_DEVICE, st);
  } else {
    DFM2G_CUDA(cudaMemcpyAsync(scratch, rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
    s = dfm2g_solve_pcg(m, p, scratch, y, a.tol, a.max_iter, nullptr, 0, nullptr, DFM2G_MEM_DEVICE, st);
  }
  return s == DFM2G_ERR_NOT_CONVERGED ? DFM2G_OK : s;
}

static void add_stats(dfm2g_solve_stats *acc, const dfm2g_solve_stats &s) {
  if (!acc) return;
  acc->iterations += s.iterations;
  acc->outer += s.outer;
  acc->rel_residual = std::max(acc->rel_residual, s.rel_residual);
  acc->ms += s.ms;
}

static int cloth_step_dev(dfm2g_cloth c, dfm2g_bsr m, dfm2g_ilu p, double *x, double *v, const StepArgs &a,
                          dfm2g_solve_stats *acc) {
  const size_t n = c->np * 3;
  DFM2G_TRY(cloth_system(c, m, p, x, v, a, c->b.p));
  DFM2G_CUDA(cudaMemsetAsync(c->dx.p, 0, sizeof(double) * n, stream()));
  dfm2g_solve_stats st{};
  DFM2G_TRY(cloth_solve(m, p, c->b.p, c->dx.p, c->mu.p, a, &st));
  add_stats(acc, st);
  k_cloth_update<<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(n, c->dx.p, a.bc, a.dt, x, v);
  note_launches(1);
  DFM2G_LAUNCH_CHECK();
  return DFM2G_OK;
}

static int adjoint_terms(dfm2g_cloth c, const double *x, const double *young, double nu, double stiff,
                         const double *mu, const double *dx, double *xbar, double *Ebar) {
  unsigned nl = 0;
  for (size_t k = 0; k + 1 < c->tri_color_start.size(); ++k) {
    const unsigned n = c->tri_color_start[k + 1] - c->tri_color_start[k];
    k_tri_adjoint<<<blocks_for(n, 128), 128, 0, stream()>>>(n, c->tri_by_color.p + c->tri_color_start[k], c->tri.p,
                                                            c->tri_rest.p, x, young, nu, mu, dx, xbar, Ebar);
    ++nl;
  }
  for (size_t k = 0; k + 1 < c->quad_color_start.size(); ++k) {
    const unsigned n = c->quad_color_start[k + 1] - c->quad_color_start[k];
    k_quad_adjoint<<<blocks_for(n, 128), 128, 0, stream()>>>(n, c->quad_by_color.p + c->quad_color_start[k],
                                                             c->quad.p, c->quad_rest.p, stiff, mu, xbar);
    ++nl;
  }
  note_launches(nl);
  DFM2G_LAUNCH_CHECK();
  return DFM2G_OK;
}

static int ensure_scratch(dfm2g_cloth c) {
  const size_t n = c->np * 3 + 1;
  DFM2G_TRY(c->dW.resize(n));
  DFM2G_TRY(c->b.resize(n));
  DFM2G_TRY(c->dx.resize(n));
  DFM2G_TRY(c->mu.resize(n));
  DFM2G_TRY(c->dxbar.resize(n));
  return DFM2G_OK;
}

}  // namespace dfm2g

using namespace dfm2g;

extern "C" {

int dfm2g_cloth_create(dfm2g_cloth *out, dfm2g_bsr m, const double *xyz0, size_t np, const unsigned *tri,
                       size_t ntri, const unsigned *quad, size_t nquad) try {
  if (!out) return fail(DFM2G_ERR_ARG, "cloth_create: null out");
  if (!m || !m->has_pattern) return fail(DFM2G_ERR_STATE, "cloth_create: matrix has no pattern");
  DFM2G_TRY(require_3x3(m, "cloth_create"));
  if (np != m->nblk) return fail(DFM2G_ERR_ARG, "cloth_create: np (%zu) != matrix blocks (%u)", np, m->nblk);
  if ((ntri && !tri) || (nquad && !quad) || (np && !xyz0)) return fail(DFM2G_ERR_ARG, "cloth_create: null array");
  if (ntri > 0xFFFFFFFFull / 9 || nquad > 0xFFFFFFFFull / 16) return fail(DFM2G_ERR_ARG, "cloth_create: too large");
  DFM2G_TRY(ensure_context());
  auto *c = new dfm2g_cloth_s();
  c->np = np;
  c->ntri = ntri;
  c->nquad = nquad;
  c->nblk = m->nblk;
  c->bsr = m;
  c->pattern_version = m->pattern_version;
  std::vector<unsigned> tby, qby;
  int s = color_elements(tri, ntri, 3, np, tby, c->tri_color_start);
  if (s == DFM2G_OK) s = color_elements(quad, nquad, 4, np, qby, c->quad_color_start);
  if (s == DFM2G_OK) s = c->xyz0.resize(np * 3 + 1);
  if (s == DFM2G_OK) s = c->tri.resize(ntri * 3 + 1);
  if (s == DFM2G_OK) s = c->quad.resize(nquad * 4 + 1);
  if (s == DFM2G_OK) s = c->tri_slot.resize(ntri * 9 + 1);
  if (s == DFM2G_OK) s = c->quad_slot.resize(nquad * 16 + 1);
  if (s == DFM2G_OK) s = c->tri_by_color.resize(ntri + 1);
  if (s == DFM2G_OK) s = c->quad_by_color.resize(nquad + 1);
  if (s == DFM2G_OK) s = c->tri_rest.resize(ntri * 8 + 1);
  if (s == DFM2G_OK) s = c->quad_rest.resize(nquad * 8 + 1);
  if (s == DFM2G_OK) s = ensure_scratch(c);
  auto h2d = [&](void *dst, const void *src, size_t bytes) {
    if (s == DFM2G_OK && bytes &&
        cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream()) != cudaSuccess)
      s = fail(DFM2G_ERR_CUDA, "cloth_create: copy");
  };
  h2d(c->xyz0.p, xyz0, sizeof(double) * np * 3);
  h2d(c->tri.p, tri, sizeof(unsigned) * ntri * 3);
  h2d(c->quad.p, quad, sizeof(unsigned) * nquad * 4);
  h2d(c->tri_by_color.p, tby.data(), sizeof(unsigned) * ntri);
  h2d(c->quad_by_color.p, qby.data(), sizeof(unsigned) * nquad);
  if (s == DFM2G_OK && ntri) s = build_slot_map(c->tri.p, ntri, 3, m, c->tri_slot.p);
  if (s == DFM2G_OK && nquad) s = build_slot_map(c->quad.p, nquad, 4, m, c->quad_slot.p);
  if (s == DFM2G_OK && ntri) {
    k_tri_rest<<<blocks_for(ntri, 128, ctx().num_sms * 16), 128, 0, stream()>>>(ntri, c->tri.p, c->xyz0.p,
                                                                                 c->tri_rest.p);
    if (cudaGetLastError() != cudaSuccess) s = fail(DFM2G_ERR_CUDA, "cloth_create: rest kernel");
  }
  if (s == DFM2G_OK && nquad) {
    k_quad_rest<<<blocks_for(nquad, 128, ctx().num_sms * 16), 128, 0, stream()>>>(nquad, c->quad.p, c->xyz0.p,
                                                                                   c->quad_rest.p);
    if (cudaGetLastError() != cudaSuccess) s = fail(DFM2G_ERR_CUDA, "cloth_create: rest kernel");
  }
  if (s == DFM2G_OK && cudaStreamSynchronize(stream()) != cudaSuccess) s = fail(DFM2G_ERR_CUDA, "cloth_create");
  if (s != DFM2G_OK) {
    delete c;
    return s;
  }
  *out = c;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_cloth_destroy(dfm2g_cloth c) try {
  if (c) {
    cudaStreamSynchronize(stream());
    delete c;
  }
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_cloth_info(dfm2g_cloth c, unsigned *ncolor_tri, unsigned *ncolor_quad) try {
  if (!c) return fail(DFM2G_ERR_ARG, "null cloth");
  if (ncolor_tri) *ncolor_tri = c->tri_color_start.empty() ? 0 : (unsigned)c->tri_color_start.size() - 1;
  if (ncolor_quad) *ncolor_quad = c->quad_color_start.empty() ? 0 : (unsigned)c->quad_color_start.size() - 1;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_cloth_merge(dfm2g_cloth c, dfm2g_bsr m, const double *xyz, const double *young_tri, double nu,
                      double stiff_bend, double *dW, double *W, int mem) try {
  DFM2G_TRY(check_cloth(c, m));
  if (!xyz || !dW || (c->ntri && !young_tri)) return fail(DFM2G_ERR_ARG, "cloth_merge: null argument");
  VecArg<double> ax, ay, ad;
  DFM2G_TRY(ax.in(xyz, c->np * 3, mem, true));
  DFM2G_TRY(ay.in(young_tri, c->ntri, mem, true));
  DFM2G_TRY(ad.in(dW, c->np * 3, mem, true));
  const size_t ne = c->ntri + c->nquad;
  if (W) {
    DFM2G_TRY(c->welem.resize(ne + 1));
    DFM2G_TRY(c->wsum.resize(1));
    DFM2G_CUDA(cudaMemsetAsync(c->welem.p, 0, sizeof(double) * (ne + 1), stream()));
    DFM2G_CUDA(cudaMemsetAsync(c->wsum.p, 0, sizeof(double), stream()));
  }
  DFM2G_TRY(cloth_assemble(c, m, ax.dev(), ay.dev(), nu, stiff_bend, ad.dev(), W ? c->welem.p : nullptr));
  if (W) {
    k_sum_one_block<<<1, 256, 0, stream()>>>(ne, c->welem.p, c->wsum.p);
    note_launches(1);
    DFM2G_LAUNCH_CHECK();
    DFM2G_CUDA(cudaMemcpyAsync(W, c->wsum.p, sizeof(double), cudaMemcpyDeviceToHost, stream()));
    DFM2G_CUDA(cudaStreamSynchronize(stream()));
  }
  return ad.copy_back();
} catch (...) {
  return host_failure();
}

static int step_args(dfm2g_cloth c, const int *bc, const double *young, double nu, double stiff, const double *g,
                     double mass, double dt, double tol, unsigned max_iter, int solver, StepArgs &a) {
  if (!g) return fail(DFM2G_ERR_ARG, "cloth: null gravity");
  if (!(dt > 0)) return fail(DFM2G_ERR_ARG, "cloth: dt must be > 0");
  if (solver != DFM2G_CLOTH_PCG_F64 && solver != DFM2G_CLOTH_PCG_MIXED)
    return fail(DFM2G_ERR_ARG, "cloth: unknown solver %d", solver);
  (void)c;
  a.bc = bc;
  a.young = young;
  a.nu = nu;
  a.stiff = stiff;
  for (int d = 0; d < 3; ++d) a.g[d] = g[d];
  a.mass = mass;
  a.dt = dt;
  a.tol = tol;
  a.max_iter = max_iter;
  a.solver = solver;
  return DFM2G_OK;
}

int dfm2g_cloth_step(dfm2g_cloth c, dfm2g_bsr m, dfm2g_ilu p, double *xyz, double *uvw, const int *bc,
                     const double *young_tri, double nu, double stiff_bend, const double *g, double mass, double dt,
                     double tol, unsigned max_iter, int solver, dfm2g_solve_stats *stats, int mem) try {
  DFM2G_TRY(check_cloth(c, m));
  if (!p) return fail(DFM2G_ERR_ARG, "cloth_step: null preconditioner");
  if (!xyz || !uvw || !bc || (c->ntri && !young_tri)) return fail(DFM2G_ERR_ARG, "cloth_step: null argument");
  const size_t n = c->np * 3;
  VecArg<double> ax, av, ay;
  VecArg<int> ab;
  DFM2G_TRY(ax.in(xyz, n, mem, true));
  DFM2G_TRY(av.in(uvw, n, mem, true));
  DFM2G_TRY(ab.in(bc, n, mem, true));
  DFM2G_TRY(ay.in(young_tri, c->ntri, mem, true));
  StepArgs a;
  DFM2G_TRY(step_args(c, ab.dev(), ay.dev(), nu, stiff_bend, g, mass, dt, tol, max_iter, solver, a));
  if (stats) *stats = dfm2g_solve_stats{};
  DFM2G_TRY(cloth_step_dev(c, m, p, ax.dev(), av.dev(), a, stats));
  DFM2G_TRY(ax.copy_back());
  return av.copy_back();
} catch (...) {
  return host_failure();
}

int dfm2g_cloth_adjoint_terms(dfm2g_cloth c, const double *xyz, const double *young_tri, double nu,
                              double stiff_bend, const double *mu, const double *dx, double *xbar, double *Ebar,
                              int mem) try {
  if (!c) return fail(DFM2G_ERR_ARG, "null cloth");
  if (!xyz || !mu || !dx || !xbar || !Ebar || (c->ntri && !young_tri))
    return fail(DFM2G_ERR_ARG, "cloth_adjoint_terms: null argument");
  const size_t n = c->np * 3;
  VecArg<double> ax, ay, am, ad, axb, aeb;
  DFM2G_TRY(ax.in(xyz, n, mem, true));
  DFM2G_TRY(ay.in(young_tri, c->ntri, mem, true));
  DFM2G_TRY(am.in(mu, n, mem, true));
  DFM2G_TRY(ad.in(dx, n, mem, true));
  DFM2G_TRY(axb.in(xbar, n, mem, true));
  DFM2G_TRY(aeb.in(Ebar, c->ntri, mem, true));
  DFM2G_TRY(adjoint_terms(c, ax.dev(), ay.dev(), nu, stiff_bend, am.dev(), ad.dev(), axb.dev(), aeb.dev()));
  DFM2G_TRY(axb.copy_back());
  return aeb.copy_back();
} catch (...) {
  return host_failure();
}

int dfm2g_cloth_rollout(dfm2g_cloth c, dfm2g_bsr m, dfm2g_ilu p, double *xyz, double *uvw, const int *bc,
                        const double *young_tri, double nu, double stiff_bend, const double *g, double mass,
                        double dt, double tol, unsigned max_iter, int solver, unsigned nsteps, unsigned ckpt_every,
                        dfm2g_solve_stats *stats, int mem) try {
  DFM2G_TRY(check_cloth(c, m));
  if (!p) return fail(DFM2G_ERR_ARG, "cloth_rollout: null preconditioner");
  if (!xyz || !uvw || !bc || (c->ntri && !young_tri)) return fail(DFM2G_ERR_ARG, "cloth_rollout: null argument");
  const size_t n = c->np * 3;
  auto &ro = c->ro;
  ro.valid = false;
  VecArg<double> ax, av;
  DFM2G_TRY(ax.in(xyz, n, mem, true));
  DFM2G_TRY(av.in(uvw, n, mem, true));
  // the rollout keeps its own copies of bc and E for the reverse pass
  DFM2G_TRY(ro.bc.resize(n + 1));
  DFM2G_TRY(ro.young.resize(c->ntri + 1));
  const auto kind = mem == DFM2G_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  DFM2G_CUDA(cudaMemcpyAsync(ro.bc.p, bc, sizeof(int) * n, kind, stream()));
  if (c->ntri) DFM2G_CUDA(cudaMemcpyAsync(ro.young.p, young_tri, sizeof(double) * c->ntri, kind, stream()));
  StepArgs a;
  DFM2G_TRY(step_args(c, ro.bc.p, ro.young.p, nu, stiff_bend, g, mass, dt, tol, max_iter, solver, a));
  const unsigned nck = ckpt_every ? nsteps / ckpt_every + 1 : 0;
  if (nck) DFM2G_TRY(ro.ckpt.resize((size_t)nck * 2 * n));
  if (stats) *stats = dfm2g_solve_stats{};
  for (unsigned k = 0; k < nsteps; ++k) {
    if (ckpt_every && k % ckpt_every == 0) {
      double *dst = ro.ckpt.p + (size_t)(k / ckpt_every) * 2 * n;
      DFM2G_CUDA(cudaMemcpyAsync(dst, ax.dev(), sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
      DFM2G_CUDA(cudaMemcpyAsync(dst + n, av.dev(), sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
    }
    DFM2G_TRY(cloth_step_dev(c, m, p, ax.dev(), av.dev(), a, stats));
  }
  if (ckpt_every) {
    ro.valid = true;
    ro.nsteps = nsteps;
    ro.every = ckpt_every;
    ro.max_iter = max_iter;
    ro.solver = solver;
    ro.nu = nu;
    ro.stiff = stiff_bend;
    for (int d = 0; d < 3; ++d) ro.g[d] = g[d];
    ro.mass = mass;
    ro.dt = dt;
    ro.tol = tol;
  }
  DFM2G_TRY(ax.copy_back());
  return av.copy_back();
} catch (...) {
  return host_failure();
}

int dfm2g_cloth_rollout_adjoint(dfm2g_cloth c, dfm2g_bsr m, dfm2g_ilu p, double *xbar, double *vbar, double *dLdE,
                                dfm2g_solve_stats *stats, int mem) try {
  DFM2G_TRY(check_cloth(c, m));
  if (!p) return fail(DFM2G_ERR_ARG, "cloth_rollout_adjoint: null preconditioner");
  if (!xbar || !vbar || (c->ntri && !dLdE)) return fail(DFM2G_ERR_ARG, "cloth_rollout_adjoint: null argument");
  auto &ro = c->ro;
  if (!ro.valid) return fail(DFM2G_ERR_STATE, "cloth_rollout_adjoint: no checkpointed rollout to reverse");
  const size_t n = c->np * 3;
  VecArg<double> axb, avb, ae;
  DFM2G_TRY(axb.in(xbar, n, mem, true));
  DFM2G_TRY(avb.in(vbar, n, mem, true));
  DFM2G_TRY(ae.in(dLdE, c->ntri, mem, false));
  if (c->ntri) DFM2G_CUDA(cudaMemsetAsync(ae.dev(), 0, sizeof(double) * c->ntri, stream()));
  StepArgs a;
  DFM2G_TRY(step_args(c, ro.bc.p, ro.young.p, ro.nu, ro.stiff, ro.g, ro.mass, ro.dt, ro.tol, ro.max_iter, ro.solver,
                      a));
  DFM2G_TRY(ro.seg.resize((size_t)(ro.every + 1) * n));
  DevBuf<double> vtmp;
  DFM2G_TRY(vtmp.resize(n + 1));
  if (stats) *stats = dfm2g_solve_stats{};
  const unsigned nseg = (ro.nsteps + ro.every - 1) / ro.every;
  for (unsigned sgi = nseg; sgi-- > 0;) {
    const unsigned k0 = sgi * ro.every, k1 = std::min(ro.nsteps, k0 + ro.every);
    // recompute the segment's positions from its checkpoint
    const double *ck = ro.ckpt.p + (size_t)sgi * 2 * n;
    DFM2G_CUDA(cudaMemcpyAsync(ro.seg.p, ck, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
    DFM2G_CUDA(cudaMemcpyAsync(vtmp.p, ck + n, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
    for (unsigned k = k0; k < k1; ++k) {
      double *xk = ro.seg.p + (size_t)(k - k0) * n, *xk1 = xk + n;
      DFM2G_CUDA(cudaMemcpyAsync(xk1, xk, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
      dfm2g_solve_stats st{};
      DFM2G_TRY(cloth_step_dev(c, m, p, xk1, vtmp.p, a, &st));
    }
    // reverse through the segment
    for (unsigned k = k1; k-- > k0;) {
      const double *xk = ro.seg.p + (size_t)(k - k0) * n, *xk1 = xk + n;
      DFM2G_TRY(cloth_system(c, m, p, xk, nullptr, a, nullptr));
      k_adj_seed<<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(n, axb.dev(), avb.dev(), a.bc, a.dt,
                                                                               xk, xk1, c->dxbar.p, c->dx.p);
      note_launches(1);
      DFM2G_LAUNCH_CHECK();
      DFM2G_CUDA(cudaMemsetAsync(c->mu.p, 0, sizeof(double) * n, stream()));
      dfm2g_solve_stats st{};
      DFM2G_TRY(cloth_solve(m, p, c->dxbar.p, c->mu.p, c->b.p, a, &st));
      add_stats(stats, st);
      DFM2G_TRY(adjoint_terms(c, xk, a.young, a.nu, a.stiff, c->mu.p, c->dx.p, axb.dev(), ae.dev()));
      k_adj_vbar<<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(n, c->mu.p, a.bc, a.mass, a.dt,
                                                                               avb.dev());
      note_launches(1);
      DFM2G_LAUNCH_CHECK();
    }
  }
  DFM2G_TRY(axb.copy_back());
  DFM2G_TRY(avb.copy_back());
  return ae.copy_back();
} catch (...) {
  return host_failure();
}

}  // extern "C"

// Krylov solvers on the device: Solve_PCG (FP64, the reference's exact
// semantics), Solve_CG, and the FP32-inner / FP64-refinement PCG.
//
// All scalars of the iteration (alpha, beta, (r,Pr), |r|^2, the history and
// the stop flag) live in device memory. Each reduction is deterministic: every
// block writes its partial sum and the last block to finish adds the partials
// in block order and applies the scalar update (alpha = rPr/pAp, ...). Every
// kernel of an iteration first reads the stop flag and returns if it is set,
// so the host can queue iterations in chunks and only synchronise between
// chunks.
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "nd.cuh"
#include "rowkern.cuh"
#include "spmv_tma.cuh"

namespace dfm2g {

struct IterState {
  double inv_rr0;  // 1/|r0|^2
  double rPr;      // (r, Pr) of the current iterate (CG: |r|^2)
  double alpha, beta;
  double tol;
  double rr;       // latest |r|^2
  unsigned it;     // completed iterations
  unsigned max_iter;
  int done;        // 0 running, 1 converged, 2 exhausted, 3 |r0|^2 < 1e-30, 4 non-finite
  unsigned nhist;
  unsigned hist_cap;
  int mode;        // 0 PCG (absolute history), 1 CG (relative history), 2 reliable-update PCG
  unsigned ticket[4];
  // reliable-update refinement (mode 2)
  double bnorm;    // |b|
  double delta;    // refresh the FP64 residual when |r| < delta * rmax
  double rmax;     // |r| at the last refresh
  double rtrue;    // |b - K x| at the last refresh
  int update;      // a refresh is due in this iteration
  unsigned n_updates;
  // The FP32 vectors hold scale * (FP64 quantity), with scale = 1/|r| reset at
  // every refresh, so they stay O(1/sqrt(n)) however small the residual gets
  // (unscaled, (r,z) and (p,Ap) underflow FP32 near 1e-10 on fine meshes).
  double scale;       // scale of the current FP32 segment
  double scale_next;  // scale chosen for the segment after this refresh
  double ratio;       // scale_new / scale_old, folded into the next beta (1 otherwise)
  int restart_p;      // the refreshed residual disagrees with the recursive one: p = z
};

constexpr int kThreads = 256;

// p.Ap fused into the SpMV Ap = K p (warp per block row); the last block sets
// alpha = (r, Pr) / (p, Ap).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_spmv_pAp(IterState *st, unsigned nblk,
                                                       const unsigned *__restrict__ row_start,
                                                       const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                                       const T *__restrict__ vdia, const T *__restrict__ p,
                                                       T *__restrict__ Ap, double *partials) {
  __shared__ double sh[32];
  if (st->done) return;
  const unsigned lane = threadIdx.x & 31;
  double dot = 0.0;
  spmv_rows(nblk, row_start, col, vcrs, vdia, p, [&](unsigned row, const T s[3]) {
    if (lane < 3) {
      const T v = pick3(s, lane);
      Ap[(size_t)row * 3 + lane] = v;
      dot += (double)(v * p[(size_t)row * 3 + lane]);
    }
  });
  double total;
  if (grid_sum_last(dot, partials, &st->ticket[0], sh, &total)) {
    st->alpha = st->rPr / total;
  }
}

// The same in the component layout of spmv_tma_rows_c (the default when the
// pattern has tiles).
template <typename T>
__global__ void __launch_bounds__(TileCfgC<T>::kThreads, 1)
    k_spmv_pAp_tma_c(IterState *st, const unsigned *__restrict__ tiles, unsigned ntiles,
                     const unsigned *__restrict__ row_start, const unsigned *__restrict__ col,
                     const T *__restrict__ vcrs, const T *__restrict__ vdia, const T *__restrict__ p,
                     T *__restrict__ Ap, double *partials, int *err, unsigned long long timeout_ns) {
  extern __shared__ __align__(128) unsigned char tma_smem[];
  __shared__ double sh[32];
  if (st->done) return;
  double dot = 0.0;
  spmv_tma_rows_c<T>(tiles, ntiles, row_start, col, vcrs, vdia, p, err, timeout_ns, tma_smem,
                     [&](unsigned row, unsigned a, T v) {
                       Ap[(size_t)row * 3 + a] = v;
                       dot += (double)(v * p[(size_t)row * 3 + a]);
                     });
  double total;
  if (grid_sum_last(dot, partials, &st->ticket[0], sh, &total)) {
    st->alpha = st->rPr / total;
  }
}

// The same for 1x1 and 2x2 blocks (nd.cuh).
template <typename T, int B>
__global__ void __launch_bounds__(kThreads) k_spmv_pAp_nd(IterState *st, unsigned nblk,
                                                          const unsigned *__restrict__ row_start,
                                                          const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                                          const T *__restrict__ vdia, const T *__restrict__ p,
                                                          T *__restrict__ Ap, double *partials) {
  __shared__ double sh[32];
  if (st->done) return;
  double dot = 0.0;
  nd_spmv_rows<T, B>(nblk, row_start, col, vcrs, vdia, p, [&](unsigned row, const T s[B], unsigned sub) {
    if (sub < (unsigned)B) {
      const T v = nd_pick<T, B>(s, sub);
      Ap[(size_t)row * B + sub] = v;
      dot += (double)(v * p[(size_t)row * B + sub]);
    }
  });
  double total;
  if (grid_sum_last(dot, partials, &st->ticket[0], sh, &total)) {
    st->alpha = st->rPr / total;
  }
}

template <typename T>
static int launch_spmv_pAp(dfm2g_bsr_s *m, IterState *st, const T *vcrs, const T *vdia, const T *pv, T *Ap,
                           double *partials, unsigned spmv_blocks) {
  if (m->ndim == 1) {
    k_spmv_pAp_nd<T, 1><<<spmv_blocks, kThreads, 0, stream()>>>(st, m->nblk, m->row_start.p, m->col.p, vcrs, vdia, pv,
                                                               Ap, partials);
  } else if (m->ndim == 2) {
    k_spmv_pAp_nd<T, 2><<<spmv_blocks, kThreads, 0, stream()>>>(st, m->nblk, m->row_start.p, m->col.p, vcrs, vdia, pv,
                                                               Ap, partials);
  } else if (m->tiles_ok) {
    using C = TileCfgC<T>;
    static int attr_device = -1;  // per instantiation, once per device
    if (attr_device != ctx().device) {
      DFM2G_CUDA(cudaFuncSetAttribute(k_spmv_pAp_tma_c<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)C::kSmem));
      attr_device = ctx().device;
    }
    const unsigned nt = sizeof(T) == 8 ? m->ntiles64 : m->ntiles32;
    const unsigned *tiles = sizeof(T) == 8 ? m->tiles64.p : m->tiles32.p;
    const unsigned grid = std::min(nt, (unsigned)ctx().num_sms);
    k_spmv_pAp_tma_c<T><<<grid, C::kThreads, C::kSmem, stream()>>>(st, tiles, nt, m->row_start.p, m->col.p, vcrs,
                                                                     vdia, pv, Ap, partials, m->err.p,
                                                                     kWaitTimeoutNs);
  } else {
    k_spmv_pAp<T><<<spmv_blocks, kThreads, 0, stream()>>>(st, m->nblk, m->row_start.p, m->col.p, vcrs, vdia, pv, Ap,
                                                         partials);
  }
  return DFM2G_OK;
}

// Reliable update, part 1: x64 += x32, x32 = 0 (only when a refresh is due).
__global__ void k_flush_x(const IterState *st, size_t n, double *__restrict__ x64, float *__restrict__ x32) {
  if (st->done || !st->update) return;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    x64[i] += (double)x32[i] / st->scale;
    x32[i] = 0.f;
  }
}

// End of a refresh: |b - K x64|^2 (rr) and |true - recursive residual|^2 (dd)
// summed over the grid; the last block updates the iteration state. The
// block sums of dd go to partials[gridDim.x + block] (written before
// grid_sum_last's fence); the last block adds them in block order.
__device__ __forceinline__ void refresh_tail(IterState *st, double rr, double dd, double *partials, double *sh,
                                             double *sh2) {
  dd = block_sum(dd, sh2);
  if (threadIdx.x == 0) partials[gridDim.x + blockIdx.x] = dd;
  double total;
  if (grid_sum_last(rr, partials, &st->ticket[3], sh, &total)) {
    const double rt = sqrt(total);
    double gap2 = 0.0;
    for (unsigned b2 = 0; b2 < gridDim.x; ++b2) gap2 += ld_relaxed(partials + gridDim.x + b2);
    st->restart_p = sqrt(gap2) > 0.5 * rt ? 1 : 0;
    st->rtrue = rt;
    st->update = 0;
    st->n_updates++;
    if (!isfinite(rt)) {
      st->done = 4;
    } else if (rt < st->tol * st->bnorm) {
      st->done = 1;
    } else if (st->it >= st->max_iter) {
      st->done = 2;
    } else {
      st->rmax = rt;
    }
    st->ratio = st->scale_next / st->scale;
    st->scale = st->scale_next;
  }
}

// Reliable update, part 2: r64 = b - K64 x64 in FP64, r32 = (float) r64, and
// |r64| decides convergence (|r64| < tol |b|) or the next refresh threshold.
// B = 3 runs the 3x3 row product of rowkern.cuh, B = 1, 2 that of nd.cuh.
template <int B>
__global__ void __launch_bounds__(kThreads) k_true_residual(IterState *st, unsigned nblk,
                                                            const unsigned *__restrict__ row_start,
                                                            const unsigned *__restrict__ col,
                                                            const double *__restrict__ vcrs,
                                                            const double *__restrict__ vdia,
                                                            const double *__restrict__ x64,
                                                            const double *__restrict__ b, float *__restrict__ r32,
                                                            double *partials) {
  __shared__ double sh[32];
  if (st->done || !st->update) return;
  __shared__ double sh2[32];
  const unsigned lane = threadIdx.x & 31;
  const double sc = st->scale_next, inv_old = 1.0 / st->scale;
  double rr = 0.0, dd = 0.0;
  // sub: the lane's index in the row's lanes (the warp lane for 3x3 rows)
  auto row_done = [&](unsigned row, const double s[B], unsigned sub) {
    if (sub < (unsigned)B) {
      const size_t k = (size_t)row * B + sub;
      const double r = b[k] - (B == 3 ? pick3(s, sub) : nd_pick<double, B>(s, sub));
      const double gap = r - (double)r32[k] * inv_old;  // true minus recursive residual
      r32[k] = (float)(r * sc);
      rr += r * r;
      dd += gap * gap;
    }
  };
  if constexpr (B == 3)
    spmv_rows(nblk, row_start, col, vcrs, vdia, x64, [&](unsigned row, const double s[3]) { row_done(row, s, lane); });
  else
    nd_spmv_rows<double, B>(nblk, row_start, col, vcrs, vdia, x64, row_done);
  refresh_tail(st, rr, dd, partials, sh, sh2);
}

// Both parts of the reliable update in one cooperative launch (k_flush_x,
// k_true_residual) for 3x3 patterns with SpMV tiles, only when a refresh is
// due: x64 += x32 / scale and x32 = 0 over the CTA's grid-stride share, a
// meeting of all CTAs, then r64 = b - K64 x64 through the TMA-staged
// component-layout product (spmv_tma_rows_c<double>).
__global__ void __launch_bounds__(TileCfgC<double>::kThreads, 1)
    k_refresh_tma(IterState *st, const unsigned *__restrict__ tiles, unsigned ntiles,
                  const unsigned *__restrict__ row_start, const unsigned *__restrict__ col,
                  const double *__restrict__ vcrs, const double *__restrict__ vdia, double *x64, float *x32,
                  const double *__restrict__ b, float *__restrict__ r32, size_t n, double *partials, unsigned *bar,
                  int *err, unsigned long long timeout_ns) {
  extern __shared__ __align__(128) unsigned char tma_smem[];
  __shared__ double sh[32];
  __shared__ double sh2[32];
  if (st->done || !st->update) return;
  const double sc = st->scale_next, old = st->scale, inv_old = 1.0 / st->scale;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    x64[i] += (double)x32[i] / old;
    x32[i] = 0.f;
  }
  if (!grid_barrier(bar, err, timeout_ns)) {
    if (threadIdx.x == 0) st->done = 4;
    return;
  }
  double rr = 0.0, dd = 0.0;
  spmv_tma_rows_c<double>(tiles, ntiles, row_start, col, vcrs, vdia, x64, err, timeout_ns, tma_smem,
                          [&](unsigned row, unsigned a, double v) {
                            const size_t k = (size_t)row * 3 + a;
                            const double r = b[k] - v;
                            const double gap = r - (double)r32[k] * inv_old;  // true minus recursive residual
                            r32[k] = (float)(r * sc);
                            rr += r * r;
                            dd += gap * gap;
                          });
  refresh_tail(st, rr, dd, partials, sh, sh2);
}

// Pending marker of the sync-free sweeps, as a value of type T.
template <typename T>
__device__ __forceinline__ T pending_marker() {
  if constexpr (sizeof(T) == 8)
    return __longlong_as_double(-1ll);
  else
    return __uint_as_float(0xffffffffu);
}

// r -= alpha Ap; x += alpha p over the CTA's grid-stride share of the
// vectors; returns the share of |r|^2. When fill_a and fill_b are given, both
// are set to the sweeps' pending marker element by element after Ap is read
// (Ap may alias fill_a). Four elements per thread and pass, all loads issued
// before the arithmetic.
template <typename T>
__device__ __forceinline__ double update_pass(size_t n, T *__restrict__ r, T *__restrict__ x, const T *p,
                                              const T *Ap, double alpha, T *fill_a, T *fill_b) {
  const size_t S = (size_t)gridDim.x * blockDim.x;
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double rr = 0.0;
  const T pend = pending_marker<T>();
  auto one = [&](T ri, T xi, T pi, T api, size_t k) -> double {
    double rn;
    if constexpr (sizeof(T) == 8) {
      rn = ri + (-alpha) * api;
      r[k] = rn;
      x[k] = xi + alpha * pi;
    } else {
      const float a = (float)alpha;
      const float rf = ri - a * api;
      r[k] = rf;
      x[k] = xi + a * pi;
      rn = rf;
    }
    if (fill_a) {
      fill_a[k] = pend;
      fill_b[k] = pend;
    }
    return rn;
  };
  for (; i + 3 * S < n; i += 4 * S) {
    T rv[4], xv[4], pv[4], av[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      av[u] = Ap[i + u * S];
      rv[u] = r[i + u * S];
      xv[u] = x[i + u * S];
      pv[u] = p[i + u * S];
    }
    if constexpr (sizeof(T) == 8) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const double rn = one(rv[u], xv[u], pv[u], av[u], i + u * S);
        rr += rn * rn;
      }
    } else {  // a short FP32 run, accumulated in FP64
      float acc = 0.f;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float rn = (float)one(rv[u], xv[u], pv[u], av[u], i + u * S);
        acc += rn * rn;
      }
      rr += (double)acc;
    }
  }
  for (; i < n; i += S) {
    const double rn = one(r[i], x[i], p[i], Ap[i], i);
    rr += rn * rn;
  }
  return rr;
}

// |r|^2 (total) -> history and the stop test (one thread of the grid).
__device__ __forceinline__ void update_tail(IterState *st, double total, double *hist) {
  st->rr = total;
  const unsigned it = st->it + 1;
  st->it = it;
  if (st->mode == 2) {  // reliable updates: the FP64 refresh decides convergence
    const double rn_scaled = sqrt(total);
    const double rn = rn_scaled / st->scale;
    if (st->nhist < st->hist_cap) hist[st->nhist] = rn;
    st->nhist++;
    if (!isfinite(total)) {
      st->done = 4;
    } else if (rn < st->delta * st->rmax || rn < st->tol * st->bnorm || it >= st->max_iter) {
      st->update = 1;
      st->scale_next = rn_scaled > 0.0 ? st->scale / rn_scaled : st->scale;
    }
    return;
  }
  const double ratio = sqrt(total * st->inv_rr0);
  const double entry = st->mode == 0 ? sqrt(total) : ratio;
  if (st->nhist < st->hist_cap) hist[st->nhist] = entry;
  st->nhist++;
  if (!isfinite(total)) {
    st->done = 4;
  } else if (ratio < st->tol) {
    st->done = 1;
  } else if (it >= st->max_iter) {
    if (st->mode == 0) {  // Solve_PCG appends a final |r| on exhaustion
      if (st->nhist < st->hist_cap) hist[st->nhist] = sqrt(total);
      st->nhist++;
    }
    st->done = 2;
  } else if (st->mode == 1) {  // CG: beta = |r1|^2/|r0|^2
    st->beta = total / st->rPr;
    st->rPr = total;
  }
}

// r -= alpha Ap; x += alpha p; |r|^2 -> history and the stop test
// (update_pass, update_tail).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_update(IterState *st, size_t n, T *__restrict__ r, T *__restrict__ x,
                                                     const T *p, const T *Ap, double *partials, double *hist,
                                                     T *fill_a, T *fill_b) {
  __shared__ double sh[32];
  if (st->done) return;
  const double rr = update_pass<T>(n, r, x, p, Ap, st->alpha, fill_a, fill_b);
  double total;
  if (grid_sum_last(rr, partials, &st->ticket[1], sh, &total)) update_tail(st, total, hist);
}

// The SpMV with p.Ap (component layout, k_spmv_pAp_tma_c) and the update
// (k_update) in one cooperative launch: the CTAs meet once to add the p.Ap
// partials (each CTA adds them in the same order, so every CTA has the same
// alpha), then update their grid-stride share of r and x. The |r|^2 partials
// go to partials[gridDim.x, 2 gridDim.x).
template <typename T>
__global__ void __launch_bounds__(TileCfgC<T>::kThreads, 1)
    k_spmv_update_tma_c(IterState *st, const unsigned *__restrict__ tiles, unsigned ntiles,
                        const unsigned *__restrict__ row_start, const unsigned *__restrict__ col,
                        const T *__restrict__ vcrs, const T *__restrict__ vdia, const T *p, T *Ap, T *r, T *x,
                        size_t n, double *partials, double *hist, T *fill_a, T *fill_b, unsigned *bar, int *err,
                        unsigned long long timeout_ns) {
  extern __shared__ __align__(128) unsigned char tma_smem[];
  __shared__ double sh[32];
  if (st->done) return;
  double dot = 0.0;
  spmv_tma_rows_c<T>(tiles, ntiles, row_start, col, vcrs, vdia, p, err, timeout_ns, tma_smem,
                     [&](unsigned row, unsigned a, T v) {
                       Ap[(size_t)row * 3 + a] = v;
                       dot += (double)(v * p[(size_t)row * 3 + a]);
                     });
  dot = block_sum(dot, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = dot;
  if (!grid_barrier(bar, err, timeout_ns)) {
    if (threadIdx.x == 0) st->done = 4;
    return;
  }
  const double alpha = st->rPr / sum_partials_all(partials, gridDim.x, sh);
  if (blockIdx.x == 0 && threadIdx.x == 0) st->alpha = alpha;
  const double rr = update_pass<T>(n, r, x, p, Ap, alpha, fill_a, fill_b);
  double total;
  if (grid_sum_last(rr, partials + gridDim.x, &st->ticket[1], sh, &total)) update_tail(st, total, hist);
}

// rPr1 = (r, Pr); beta = rPr1/rPr. Four elements per thread and pass.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_dot_beta(IterState *st, size_t n, const T *__restrict__ r,
                                                       const T *__restrict__ z, double *partials) {
  __shared__ double sh[32];
  if (st->done) return;
  const size_t S = (size_t)gridDim.x * blockDim.x;
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double s = 0.0;
  for (; i + 3 * S < n; i += 4 * S) {
    T a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = r[i + u * S];
      b[u] = z[i + u * S];
    }
    if constexpr (sizeof(T) == 8) {
#pragma unroll
      for (int u = 0; u < 4; ++u) s += a[u] * b[u];
    } else {  // a short FP32 run, accumulated in FP64
      float acc = 0.f;
#pragma unroll
      for (int u = 0; u < 4; ++u) acc += a[u] * b[u];
      s += (double)acc;
    }
  }
  for (; i < n; i += S) s += (double)r[i] * (double)z[i];
  double total;
  if (grid_sum_last(s, partials, &st->ticket[2], sh, &total)) {
    // after a rescale of the FP32 vectors, the old p and (r,Pr) are in the old
    // scale: p_new = z + rPr1/(rPr*ratio^2) * (ratio*p) = z + rPr1/(rPr*ratio) * p
    st->beta = st->restart_p ? 0.0 : total / (st->rPr * st->ratio);
    st->rPr = total;
    st->ratio = 1.0;
    st->restart_p = 0;
  }
}

// p = z + beta p. Four elements per thread and pass.
template <typename T>
__global__ void k_p_update(const IterState *st, size_t n, T *__restrict__ p, const T *__restrict__ z) {
  if (st->done) return;
  const T beta = (T)st->beta;
  const size_t S = (size_t)gridDim.x * blockDim.x;
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  for (; i + 3 * S < n; i += 4 * S) {
    T a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = p[i + u * S];
      b[u] = z[i + u * S];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) p[i + u * S] = beta * a[u] + b[u];
  }
  for (; i < n; i += S) p[i] = beta * p[i] + z[i];
}

// (r, z), beta and p = z + beta p in one cooperative launch (k_dot_beta and
// k_p_update): the CTAs meet once to add the dot's partials, each in the same
// order, so every CTA computes the same beta. The state the dot updates
// (rPr, ratio, restart_p) is read before the meeting and written after it.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_dot_pupdate(IterState *st, size_t n, const T *__restrict__ r,
                                                          const T *__restrict__ z, T *__restrict__ p,
                                                          double *partials, unsigned *bar, int *err,
                                                          unsigned long long timeout_ns) {
  __shared__ double sh[32];
  if (st->done) return;
  const double rPr = st->rPr, ratio = st->ratio;
  const int restart = st->restart_p;
  const size_t S = (size_t)gridDim.x * blockDim.x;
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double s = 0.0;
  for (; i + 3 * S < n; i += 4 * S) {
    T a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = r[i + u * S];
      b[u] = z[i + u * S];
    }
    if constexpr (sizeof(T) == 8) {
#pragma unroll
      for (int u = 0; u < 4; ++u) s += a[u] * b[u];
    } else {  // a short FP32 run, accumulated in FP64
      float acc = 0.f;
#pragma unroll
      for (int u = 0; u < 4; ++u) acc += a[u] * b[u];
      s += (double)acc;
    }
  }
  for (; i < n; i += S) s += (double)r[i] * (double)z[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
  if (!grid_barrier(bar, err, timeout_ns)) {
    if (threadIdx.x == 0) st->done = 4;
    return;
  }
  const double total = sum_partials_all(partials, gridDim.x, sh);
  // after a rescale of the FP32 vectors, the old p and (r,Pr) are in the old
  // scale: p_new = z + rPr1/(rPr*ratio^2) * (ratio*p) = z + rPr1/(rPr*ratio) * p
  const double beta_d = restart ? 0.0 : total / (rPr * ratio);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->beta = beta_d;
    st->rPr = total;
    st->ratio = 1.0;
    st->restart_p = 0;
  }
  const T beta = (T)beta_d;
  for (i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i + 3 * S < n; i += 4 * S) {
    T a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = p[i + u * S];
      b[u] = z[i + u * S];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) p[i + u * S] = beta * a[u] + b[u];
  }
  for (; i < n; i += S) p[i] = beta * p[i] + z[i];
}

// generic deterministic dot into a device scalar
template <typename T>
__global__ void __launch_bounds__(kThreads) k_dot(size_t n, const T *__restrict__ a, const T *__restrict__ b,
                                                  double *partials, unsigned *ticket, double *out) {
  __shared__ double sh[32];
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s += (double)a[i] * (double)b[i];
  double total;
  if (grid_sum_last(s, partials, ticket, sh, &total)) *out = total;
}

// Start of PCG/CG: state from |r0|^2 (scal[0]) and (r0, Pr0) (scal[1]).
__global__ void k_init_state(IterState *st, const double *scal, double *hist, int mode) {
  const double rr0 = scal[0];
  st->rr = rr0;
  st->it = 0;
  st->nhist = 0;
  st->done = 0;
  if (mode == 0) {
    if (st->hist_cap > 0) hist[0] = sqrt(rr0);
    st->nhist = 1;
  }
  if (mode == 2 ? !(rr0 > 0.0) : rr0 < 1.0e-30) {  // the refinement has no absolute floor
    st->done = 3;
    return;
  }
  if (!isfinite(rr0)) {
    st->done = 4;
    return;
  }
  st->inv_rr0 = 1.0 / rr0;
  st->rPr = mode != 1 ? scal[1] : rr0;
  if (st->max_iter == 0) {  // no iteration: Solve_PCG still appends the final |r|
    if (mode == 0) {
      if (st->nhist < st->hist_cap) hist[st->nhist] = sqrt(rr0);
      st->nhist++;
    }
    st->done = 2;
  }
}

template <typename T>
__global__ void k_scale_convert(size_t n, const double *__restrict__ in, double s, T *__restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (T)(in[i] * s);
}

template <typename T>
__global__ void k_accumulate(size_t n, double *__restrict__ x, double s, const T *__restrict__ d) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    x[i] += s * (double)d[i];
}

// ---------------------------------------------------------------------------
// Workspace shared by the solvers (grown on demand).
struct Workspace {
  DevBuf<IterState> st;
  DevBuf<double> partials, scal, hist;
  DevBuf<unsigned> tickets;
  DevBuf<unsigned> bar;  // grid_barrier words of the cooperative solver kernels
  DevBuf<double> v64[6];
  DevBuf<float> v32[6];
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};
static Workspace g_ws;

static unsigned reduce_blocks() { return (unsigned)ctx().num_sms * 4; }

static int ws_prepare(size_t n, unsigned hist_cap, bool need32) {
  DFM2G_TRY(g_ws.st.ensure(1));
  DFM2G_TRY(g_ws.partials.ensure((size_t)ctx().num_sms * 64));
  DFM2G_TRY(g_ws.scal.ensure(8));
  DFM2G_TRY(g_ws.tickets.ensure(4));
  DFM2G_TRY(g_ws.bar.ensure(2));
  DFM2G_CUDA(cudaMemsetAsync(g_ws.bar.p, 0, 2 * sizeof(unsigned), stream()));
  DFM2G_TRY(g_ws.hist.ensure(hist_cap + 4));
  for (auto &b : g_ws.v64) DFM2G_TRY(b.ensure(n + 1));
  if (need32)
    for (auto &b : g_ws.v32) DFM2G_TRY(b.ensure(n + 1));
  if (!g_ws.ev0) {
    DFM2G_CUDA(cudaEventCreate(&g_ws.ev0));
    DFM2G_CUDA(cudaEventCreate(&g_ws.ev1));
  }
  return DFM2G_OK;
}

static int dot_dev(size_t n, const void *a, const void *b, int prec, double *out_dev) {
  DFM2G_CUDA(cudaMemsetAsync(g_ws.tickets.p, 0, sizeof(unsigned), stream()));
  note_launches(1);
  if (prec == DFM2G_F64)
    k_dot<double><<<reduce_blocks(), kThreads, 0, stream()>>>(n, (const double *)a, (const double *)b,
                                                             g_ws.partials.p, g_ws.tickets.p, out_dev);
  else
    k_dot<float><<<reduce_blocks(), kThreads, 0, stream()>>>(n, (const float *)a, (const float *)b, g_ws.partials.p,
                                                            g_ws.tickets.p, out_dev);
  DFM2G_LAUNCH_CHECK();
  return DFM2G_OK;
}

static int dot_host(size_t n, const void *a, const void *b, int prec, double *out) {
  DFM2G_TRY(dot_dev(n, a, b, prec, g_ws.scal.p + 7));
  DFM2G_CUDA(cudaMemcpyAsync(out, g_ws.scal.p + 7, sizeof(double), cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  return DFM2G_OK;
}

// Cooperative launch of `kernel` with the given arguments (each must have the
// kernel parameter's exact type).
template <typename... A>
static int coop_launch(void (*kernel)(A...), unsigned grid, unsigned threads, size_t smem, A... args) {
  void *argv[] = {(void *)&args...};
  DFM2G_CUDA(cudaLaunchCooperativeKernel((void *)kernel, dim3(grid), dim3(threads), argv, smem, stream()));
  return DFM2G_OK;
}

// Lets a TMA-staged kernel use TileCfgC's shared memory (once per device).
template <typename K>
static int allow_tma_smem(K kernel, size_t smem, int &attr_device) {
  if (attr_device != ctx().device) {
    DFM2G_CUDA(cudaFuncSetAttribute((const void *)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_device = ctx().device;
  }
  return DFM2G_OK;
}

#ifndef DFM2G_DOT_CTAS_PER_SM
#define DFM2G_DOT_CTAS_PER_SM 4u  // CTAs per SM of k_dot_pupdate
#endif
// CTAs of k_dot_pupdate<T>: DFM2G_DOT_CTAS_PER_SM per SM, or as many as are resident at once.
template <typename T>
static int dot_pupdate_blocks(unsigned *grid) {
  static int per_sm_dev = -1, per_sm = 0;
  if (per_sm_dev != ctx().device) {
    DFM2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dot_pupdate<T>, kThreads, 0));
    per_sm_dev = ctx().device;
  }
  if (per_sm <= 0) return fail(DFM2G_ERR_CUDA, "k_dot_pupdate cannot be resident");
  *grid = std::min<unsigned>(DFM2G_DOT_CTAS_PER_SM * (unsigned)ctx().num_sms, (unsigned)per_sm * (unsigned)ctx().num_sms);
  return DFM2G_OK;
}

// Core preconditioned CG on device vectors of type T.
//  r: rhs in, final residual out; x: solution out (starts at 0);
//  w0..w3: scratch vectors (Pr/Ap share w0 as in the reference, p = w1,
//  sweep intermediate = w2).
// Reliable-update refinement (mode 2, T = float): `r` holds (float)b and `x`
// the FP32 correction on entry; x64 accumulates the solution in FP64 and the
// true residual b - K x64 is recomputed in FP64 whenever the FP32 residual has
// dropped by `delta` since the last refresh (the Krylov state p is kept).
struct Refine {
  double *x64 = nullptr;
  const double *b64 = nullptr;
  double delta = 0, bnorm = 0;
};

template <typename T>
static int pcg_core(dfm2g_bsr_s *m, dfm2g_ilu_s *p, T *r, T *x, T *w0, T *w1, T *w2, double tol,
                    unsigned max_iter, unsigned hist_cap, int mode, IterState *h_state,
                    const Refine &rf = Refine()) {
  const int prec = sizeof(T) == 8 ? DFM2G_F64 : DFM2G_F32;
  const unsigned nblk = m->nblk;
  const size_t n = (size_t)nblk * m->ndim;
  const T *vcrs = sizeof(T) == 8 ? (const T *)m->vcrs.p : (const T *)m->vcrs32.p;
  const T *vdia = sizeof(T) == 8 ? (const T *)m->vdia.p : (const T *)m->vdia32.p;
  if (mode == 2 && sizeof(T) != 4) return fail(DFM2G_ERR_ARG, "reliable-update PCG runs in FP32");
  IterState init{};
  init.tol = tol;
  init.max_iter = max_iter;
  init.hist_cap = hist_cap;
  init.mode = mode;
  init.bnorm = rf.bnorm;
  init.delta = rf.delta;
  init.rmax = rf.bnorm;
  init.rtrue = rf.bnorm;
  init.ratio = 1.0;
  init.scale = (mode == 2 && rf.bnorm > 0) ? 1.0 / rf.bnorm : 1.0;
  init.scale_next = init.scale;
  IterState *st = g_ws.st.p;
  DFM2G_CUDA(cudaMemcpyAsync(st, &init, sizeof(init), cudaMemcpyHostToDevice, stream()));
  DFM2G_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * n, stream()));
  DFM2G_TRY(dot_dev(n, r, r, prec, g_ws.scal.p + 0));
  T *Pr = w0, *pv = w1, *mid = w2;
  if (mode != 1) {
    // Pr = M^-1 r ; p = Pr ; rPr = (r, Pr)
    DFM2G_TRY(ilu_sweep(p, prec, true, r, mid));
    DFM2G_TRY(ilu_sweep(p, prec, false, mid, Pr));
    DFM2G_CUDA(cudaMemcpyAsync(pv, Pr, sizeof(T) * n, cudaMemcpyDeviceToDevice, stream()));
    DFM2G_TRY(dot_dev(n, r, Pr, prec, g_ws.scal.p + 1));
  } else {
    DFM2G_CUDA(cudaMemcpyAsync(pv, r, sizeof(T) * n, cudaMemcpyDeviceToDevice, stream()));
  }
  k_init_state<<<1, 1, 0, stream()>>>(st, g_ws.scal.p, g_ws.hist.p, mode);
  note_launches(1);
  DFM2G_LAUNCH_CHECK();
  const unsigned spmv_blocks = blocks_for((size_t)nblk * 32, kThreads, (unsigned)ctx().num_sms * 8);
  const unsigned vec_blocks = reduce_blocks();
  const int chunk = 16;
  // 3x3 patterns with SpMV tiles: two cooperative launches besides the SpMV
  // and the sweeps per iteration (k_spmv_update_tma_c, k_dot_pupdate) and the
  // refresh (k_refresh_tma) only does work when one is due; otherwise five
  // (k_spmv_pAp*, k_update, k_flush_x + k_true_residual*, k_dot_beta, k_p_update).
  const bool fused = m->ndim == 3 && m->tiles_ok;
  using CT = TileCfgC<T>;
  using C64 = TileCfgC<double>;
  const unsigned nt_T = sizeof(T) == 8 ? m->ntiles64 : m->ntiles32;
  const unsigned *tiles_T = sizeof(T) == 8 ? m->tiles64.p : m->tiles32.p;
  unsigned dp_grid = 0;
  if (fused) {
    static int attr_a = -1, attr_r = -1;
    DFM2G_TRY(allow_tma_smem(k_spmv_update_tma_c<T>, CT::kSmem, attr_a));
    DFM2G_TRY(allow_tma_smem(k_refresh_tma, C64::kSmem, attr_r));
    DFM2G_TRY(dot_pupdate_blocks<T>(&dp_grid));
  }
  for (;;) {
    for (int k = 0; k < chunk; ++k) {
      T *Ap = Pr;
      // the sweeps' outputs get their pending marker in the update (Ap is Pr: read first, element by element)
      const bool fill = mode != 1 && p->sweep_mode != DFM2G_SWEEP_LEVELS;
      T *fa = fill ? mid : nullptr, *fb = fill ? Pr : nullptr;
      if (fused) {
        ProfScope ps(DFM2G_PROF_SPMV, 1);
        DFM2G_TRY(coop_launch(k_spmv_update_tma_c<T>, std::min(nt_T, (unsigned)ctx().num_sms), CT::kThreads,
                              CT::kSmem, st, tiles_T, nt_T, (const unsigned *)m->row_start.p,
                              (const unsigned *)m->col.p, vcrs, vdia, (const T *)pv, Ap, r, x, n, g_ws.partials.p,
                              g_ws.hist.p, fa, fb, g_ws.bar.p, m->err.p, kWaitTimeoutNs));
      } else {
        {
          ProfScope ps(DFM2G_PROF_SPMV, 1);
          DFM2G_TRY(launch_spmv_pAp<T>(m, st, vcrs, vdia, pv, Ap, g_ws.partials.p, spmv_blocks));
        }
        {
          ProfScope ps(DFM2G_PROF_UPDATE, 1);
          k_update<T><<<vec_blocks, kThreads, 0, stream()>>>(st, n, r, x, pv, Ap, g_ws.partials.p, g_ws.hist.p, fa,
                                                             fb);
        }
      }
      if constexpr (sizeof(T) == 4) {
        if (mode == 2 && fused) {
          ProfScope ps(DFM2G_PROF_OUTER, 1);
          DFM2G_TRY(coop_launch(k_refresh_tma, std::min(m->ntiles64, (unsigned)ctx().num_sms), C64::kThreads,
                                C64::kSmem, st, (const unsigned *)m->tiles64.p, m->ntiles64,
                                (const unsigned *)m->row_start.p, (const unsigned *)m->col.p,
                                (const double *)m->vcrs.p, (const double *)m->vdia.p, rf.x64, (float *)x, rf.b64,
                                (float *)r, n, g_ws.partials.p, g_ws.bar.p, m->err.p, kWaitTimeoutNs));
        } else if (mode == 2) {
          ProfScope ps(DFM2G_PROF_OUTER, 2);
          k_flush_x<<<vec_blocks, kThreads, 0, stream()>>>(st, n, rf.x64, (float *)x);
          if (m->ndim == 3)
            k_true_residual<3><<<spmv_blocks, kThreads, 0, stream()>>>(st, nblk, m->row_start.p, m->col.p,
                                                                       m->vcrs.p, m->vdia.p, rf.x64, rf.b64,
                                                                       (float *)r, g_ws.partials.p);
          else if (m->ndim == 2)
            k_true_residual<2><<<spmv_blocks, kThreads, 0, stream()>>>(st, nblk, m->row_start.p, m->col.p,
                                                                       m->vcrs.p, m->vdia.p, rf.x64, rf.b64,
                                                                       (float *)r, g_ws.partials.p);
          else
            k_true_residual<1><<<spmv_blocks, kThreads, 0, stream()>>>(st, nblk, m->row_start.p, m->col.p,
                                                                       m->vcrs.p, m->vdia.p, rf.x64, rf.b64,
                                                                       (float *)r, g_ws.partials.p);
        }
      }
      if (mode != 1) {
        {
          ProfScope ps(DFM2G_PROF_FWD, 0);
          DFM2G_TRY(ilu_sweep_guarded(p, prec, true, r, mid, &st->done));
        }
        {
          ProfScope ps(DFM2G_PROF_BWD, 0);
          DFM2G_TRY(ilu_sweep_guarded(p, prec, false, mid, Pr, &st->done));
        }
        if (fused) {
          ProfScope ps(DFM2G_PROF_DOT, 1);
          DFM2G_TRY(coop_launch(k_dot_pupdate<T>, dp_grid, (unsigned)kThreads, (size_t)0, st, n, (const T *)r,
                                (const T *)Pr, pv, g_ws.partials.p, g_ws.bar.p, m->err.p, kWaitTimeoutNs));
        } else {
          {
            ProfScope ps(DFM2G_PROF_DOT, 1);
            k_dot_beta<T><<<vec_blocks, kThreads, 0, stream()>>>(st, n, r, Pr, g_ws.partials.p);
          }
          {
            ProfScope ps(DFM2G_PROF_PUPDATE, 1);
            k_p_update<T><<<vec_blocks, kThreads, 0, stream()>>>(st, n, pv, Pr);
          }
        }
      } else {
        ProfScope ps(DFM2G_PROF_PUPDATE, 1);
        k_p_update<T><<<vec_blocks, kThreads, 0, stream()>>>(st, n, pv, r);
      }
    }
    DFM2G_LAUNCH_CHECK();
    DFM2G_CUDA(cudaMemcpyAsync(h_state, st, sizeof(IterState), cudaMemcpyDeviceToHost, stream()));
    DFM2G_CUDA(cudaStreamSynchronize(stream()));
    if (h_state->done) break;
  }
  if (p) {
    int e = 0;
    DFM2G_CUDA(cudaMemcpyAsync(&e, p->err.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
    DFM2G_CUDA(cudaStreamSynchronize(stream()));
    if (e) {
      DFM2G_CUDA(cudaMemsetAsync(p->err.p, 0, sizeof(int), stream()));
      return fail(DFM2G_ERR_WAIT_TIMEOUT, "PCG: a triangular-sweep wait timed out");
    }
  }
  return bsr_check_err(m);
}

static int check_pair(dfm2g_bsr m, dfm2g_ilu p) {
  if (!m || !m->has_pattern) return fail(DFM2G_ERR_STATE, "matrix has no pattern");
  if (p && (!p->has_factor || p->nblk != m->nblk))
    return fail(DFM2G_ERR_STATE, "preconditioner not decomposed for this matrix");
  if (p && p->ndim != m->ndim)
    return fail(DFM2G_ERR_ARG, "preconditioner blocks are %ux%u, the matrix's %ux%u", p->ndim, p->ndim, m->ndim,
                m->ndim);
  return DFM2G_OK;
}

static int true_residual(dfm2g_bsr_s *m, const double *b, const double *x, double *res, double *rel) {
  const size_t n = (size_t)m->nblk * m->ndim;
  DFM2G_CUDA(cudaMemcpyAsync(res, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
  DFM2G_TRY(bsr_spmv(m, DFM2G_F64, res, -1.0, x, 1.0));
  double rr = 0, bb = 0;
  DFM2G_TRY(dot_host(n, res, res, DFM2G_F64, &rr));
  DFM2G_TRY(dot_host(n, b, b, DFM2G_F64, &bb));
  *rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
  return DFM2G_OK;
}

// An empty system (no block rows): nothing to queue on the device. The
// history is [|r0|] = [0] (the |r0|^2 < 1e-30 early return of Solve_PCG).
static int empty_solve(double *hist, unsigned hist_cap, unsigned *n_hist, dfm2g_solve_stats *stats) {
  if (hist && hist_cap) hist[0] = 0.0;
  if (n_hist) *n_hist = 1;
  if (stats) *stats = dfm2g_solve_stats{0u, 0u, 0.0, 0.0};
  return DFM2G_OK;
}

}  // namespace dfm2g

using namespace dfm2g;

extern "C" {

int dfm2g_solve_pcg(dfm2g_bsr m, dfm2g_ilu p, double *r, double *x, double tol, unsigned max_iter, double *hist,
                    unsigned hist_cap, unsigned *n_hist, int mem, dfm2g_solve_stats *stats) try {
  DFM2G_TRY(check_pair(m, p));
  if (!p) return fail(DFM2G_ERR_ARG, "solve_pcg: null preconditioner");
  if (!r || !x) return fail(DFM2G_ERR_ARG, "solve_pcg: null vector");
  const size_t n = (size_t)m->nblk * m->ndim;
  if (n == 0) return empty_solve(hist, hist_cap, n_hist, stats);
  DFM2G_TRY(ws_prepare(n, max_iter + 2, false));
  VecArg<double> ar, ax;
  DFM2G_TRY(ar.in(r, n, mem, true));
  DFM2G_TRY(ax.in(x, n, mem, false));
  if (stats) DFM2G_CUDA(cudaMemcpyAsync(g_ws.v64[4].p, ar.dev(), sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
  DFM2G_CUDA(cudaEventRecord(g_ws.ev0, stream()));
  IterState hs{};
  DFM2G_TRY(pcg_core<double>(m, p, ar.dev(), ax.dev(), g_ws.v64[0].p, g_ws.v64[1].p, g_ws.v64[2].p, tol, max_iter,
                             max_iter + 2, 0, &hs));
  DFM2G_CUDA(cudaEventRecord(g_ws.ev1, stream()));
  DFM2G_TRY(ar.copy_back());
  DFM2G_TRY(ax.copy_back());
  if (hist && hist_cap) {
    const unsigned k = std::min(hist_cap, hs.nhist);
    DFM2G_CUDA(cudaMemcpyAsync(hist, g_ws.hist.p, sizeof(double) * k, cudaMemcpyDeviceToHost, stream()));
    DFM2G_CUDA(cudaStreamSynchronize(stream()));
  }
  if (n_hist) *n_hist = hs.nhist;
  if (stats) {
    DFM2G_CUDA(cudaEventSynchronize(g_ws.ev1));
    float ms = 0.f;
    DFM2G_CUDA(cudaEventElapsedTime(&ms, g_ws.ev0, g_ws.ev1));
    stats->ms = ms;
    stats->iterations = hs.it;
    stats->outer = 1;
    DFM2G_TRY(true_residual(m, g_ws.v64[4].p, ax.dev(), g_ws.v64[5].p, &stats->rel_residual));
  }
  if (hs.done == 4) return fail(DFM2G_ERR_NONFINITE, "solve_pcg: non-finite residual");
  if (hs.done == 2) return fail(DFM2G_ERR_NOT_CONVERGED, "solve_pcg: %u iterations without reaching tol", max_iter);
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_solve_cg(dfm2g_bsr m, double *r, double *x, double tol, unsigned max_iter, double *hist, unsigned hist_cap,
                   unsigned *n_hist, int mem, dfm2g_solve_stats *stats) try {
  DFM2G_TRY(check_pair(m, nullptr));
  if (!r || !x) return fail(DFM2G_ERR_ARG, "solve_cg: null vector");
  const size_t n = (size_t)m->nblk * m->ndim;
  if (n == 0) {  // Solve_CG's history has no initial entry: empty for |r0|^2 < 1e-30
    if (n_hist) *n_hist = 0;
    if (stats) *stats = dfm2g_solve_stats{0u, 0u, 0.0, 0.0};
    return DFM2G_OK;
  }
  DFM2G_TRY(ws_prepare(n, max_iter + 2, false));
  VecArg<double> ar, ax;
  DFM2G_TRY(ar.in(r, n, mem, true));
  DFM2G_TRY(ax.in(x, n, mem, false));
  if (stats) DFM2G_CUDA(cudaMemcpyAsync(g_ws.v64[4].p, ar.dev(), sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
  DFM2G_CUDA(cudaEventRecord(g_ws.ev0, stream()));
  IterState hs{};
  DFM2G_TRY(pcg_core<double>(m, nullptr, ar.dev(), ax.dev(), g_ws.v64[0].p, g_ws.v64[1].p, g_ws.v64[2].p, tol,
                             max_iter, max_iter + 2, 1, &hs));
  DFM2G_CUDA(cudaEventRecord(g_ws.ev1, stream()));
  DFM2G_TRY(ar.copy_back());
  DFM2G_TRY(ax.copy_back());
  if (hist && hist_cap) {
    const unsigned k = std::min(hist_cap, hs.nhist);
    DFM2G_CUDA(cudaMemcpyAsync(hist, g_ws.hist.p, sizeof(double) * k, cudaMemcpyDeviceToHost, stream()));
    DFM2G_CUDA(cudaStreamSynchronize(stream()));
  }
  if (n_hist) *n_hist = hs.nhist;
  if (stats) {
    DFM2G_CUDA(cudaEventSynchronize(g_ws.ev1));
    float ms = 0.f;
    DFM2G_CUDA(cudaEventElapsedTime(&ms, g_ws.ev0, g_ws.ev1));
    stats->ms = ms;
    stats->iterations = hs.it;
    stats->outer = 1;
    DFM2G_TRY(true_residual(m, g_ws.v64[4].p, ax.dev(), g_ws.v64[5].p, &stats->rel_residual));
  }
  if (hs.done == 4) return fail(DFM2G_ERR_NONFINITE, "solve_cg: non-finite residual");
  if (hs.done == 2) return fail(DFM2G_ERR_NOT_CONVERGED, "solve_cg: %u iterations without reaching tol", max_iter);
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_solve_pcg_mixed_reliable(dfm2g_bsr m, dfm2g_ilu p, const double *b, double *x, double tol, double delta,
                                   unsigned max_iter, int mem, dfm2g_solve_stats *stats) try {
  DFM2G_TRY(check_pair(m, p));
  if (!p) return fail(DFM2G_ERR_ARG, "solve_pcg_mixed_reliable: null preconditioner");
  if (!b || !x) return fail(DFM2G_ERR_ARG, "solve_pcg_mixed_reliable: null vector");
  if (!(delta > 0 && delta < 1)) return fail(DFM2G_ERR_ARG, "delta must be in (0,1)");
  const size_t n = (size_t)m->nblk * m->ndim;
  if (n == 0) return empty_solve(nullptr, 0, nullptr, stats);
  DFM2G_TRY(ws_prepare(n, max_iter + 4, true));
  DFM2G_TRY(bsr_ensure_f32(m));
  DFM2G_TRY(ilu_ensure_f32(p));
  VecArg<double> ab, ax;
  DFM2G_TRY(ab.in(b, n, mem, true));
  DFM2G_TRY(ax.in(x, n, mem, false));
  float *r32 = g_ws.v32[3].p, *x32 = g_ws.v32[4].p;
  DFM2G_CUDA(cudaEventRecord(g_ws.ev0, stream()));
  DFM2G_CUDA(cudaMemsetAsync(ax.dev(), 0, sizeof(double) * n, stream()));
  double bb = 0;
  DFM2G_TRY(dot_host(n, ab.dev(), ab.dev(), DFM2G_F64, &bb));
  const double bnorm = std::sqrt(bb);
  IterState hs{};
  if (bnorm > 0) {
    {
      ProfScope ps(DFM2G_PROF_OUTER, 1);
      k_scale_convert<float><<<reduce_blocks(), kThreads, 0, stream()>>>(n, ab.dev(), 1.0 / bnorm, r32);
    }
    DFM2G_LAUNCH_CHECK();
    Refine rf;
    rf.x64 = ax.dev();
    rf.b64 = ab.dev();
    rf.delta = delta;
    rf.bnorm = bnorm;
    DFM2G_TRY(pcg_core<float>(m, p, r32, x32, g_ws.v32[0].p, g_ws.v32[1].p, g_ws.v32[2].p, tol, max_iter,
                              max_iter + 4, 2, &hs, rf));
  }
  DFM2G_CUDA(cudaEventRecord(g_ws.ev1, stream()));
  DFM2G_TRY(ax.copy_back());
  if (stats) {
    DFM2G_CUDA(cudaEventSynchronize(g_ws.ev1));
    float ms = 0.f;
    DFM2G_CUDA(cudaEventElapsedTime(&ms, g_ws.ev0, g_ws.ev1));
    stats->ms = ms;
    stats->iterations = hs.it;
    stats->outer = hs.n_updates;
    stats->rel_residual = bnorm > 0 ? hs.rtrue / bnorm : 0.0;
  }
  if (hs.done == 4) return fail(DFM2G_ERR_NONFINITE, "solve_pcg_mixed_reliable: non-finite residual");
  if (hs.done == 2)
    return fail(DFM2G_ERR_NOT_CONVERGED, "solve_pcg_mixed_reliable: stopped at relative residual %.3e",
                hs.rtrue / bnorm);
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_solve_pcg_mixed(dfm2g_bsr m, dfm2g_ilu p, const double *b, double *x, double tol, double inner_tol,
                          unsigned max_iter, unsigned max_outer, int mem, dfm2g_solve_stats *stats) try {
  DFM2G_TRY(check_pair(m, p));
  if (!p) return fail(DFM2G_ERR_ARG, "solve_pcg_mixed: null preconditioner");
  if (!b || !x) return fail(DFM2G_ERR_ARG, "solve_pcg_mixed: null vector");
  if (!(inner_tol > 0 && inner_tol < 1)) return fail(DFM2G_ERR_ARG, "inner_tol must be in (0,1)");
  const size_t n = (size_t)m->nblk * m->ndim;
  if (n == 0) return empty_solve(nullptr, 0, nullptr, stats);
  DFM2G_TRY(ws_prepare(n, 4, true));
  DFM2G_TRY(bsr_ensure_f32(m));
  DFM2G_TRY(ilu_ensure_f32(p));
  VecArg<double> ab, ax;
  DFM2G_TRY(ab.in(b, n, mem, true));
  DFM2G_TRY(ax.in(x, n, mem, false));
  double *r64 = g_ws.v64[3].p;
  float *r32 = g_ws.v32[3].p, *d32 = g_ws.v32[4].p;
  DFM2G_CUDA(cudaEventRecord(g_ws.ev0, stream()));
  DFM2G_CUDA(cudaMemsetAsync(ax.dev(), 0, sizeof(double) * n, stream()));
  DFM2G_CUDA(cudaMemcpyAsync(r64, ab.dev(), sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
  double bb = 0;
  DFM2G_TRY(dot_host(n, ab.dev(), ab.dev(), DFM2G_F64, &bb));
  const double bnorm = std::sqrt(bb);
  unsigned total_it = 0, outer = 0;
  double rel = bnorm > 0 ? 1.0 : 0.0;
  int status = DFM2G_OK;
  const unsigned vb = reduce_blocks();
  while (bnorm > 0) {
    double rr = 0;
    DFM2G_TRY(dot_host(n, r64, r64, DFM2G_F64, &rr));
    rel = std::sqrt(rr) / bnorm;
    if (!std::isfinite(rel)) {
      status = fail(DFM2G_ERR_NONFINITE, "solve_pcg_mixed: non-finite residual");
      break;
    }
    if (rel < tol) break;
    if (outer >= max_outer || total_it >= max_iter) {
      status = fail(DFM2G_ERR_NOT_CONVERGED, "solve_pcg_mixed: stopped at relative residual %.3e", rel);
      break;
    }
    const double s = std::sqrt(rr);
    {
      ProfScope ps(DFM2G_PROF_OUTER, 1);
      k_scale_convert<float><<<vb, kThreads, 0, stream()>>>(n, r64, 1.0 / s, r32);
    }
    DFM2G_LAUNCH_CHECK();
    IterState hs{};
    DFM2G_TRY(pcg_core<float>(m, p, r32, d32, g_ws.v32[0].p, g_ws.v32[1].p, g_ws.v32[2].p, inner_tol,
                              max_iter - total_it, 4, 0, &hs));
    total_it += hs.it;
    if (hs.done == 4) {
      status = fail(DFM2G_ERR_NONFINITE, "solve_pcg_mixed: non-finite inner residual");
      break;
    }
    {
      ProfScope ps(DFM2G_PROF_OUTER, 1);
      k_accumulate<float><<<vb, kThreads, 0, stream()>>>(n, ax.dev(), s, d32);
      DFM2G_CUDA(cudaMemcpyAsync(r64, ab.dev(), sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
      DFM2G_TRY(bsr_spmv(m, DFM2G_F64, r64, -1.0, ax.dev(), 1.0));
    }
    ++outer;
  }
  DFM2G_CUDA(cudaEventRecord(g_ws.ev1, stream()));
  DFM2G_TRY(ax.copy_back());
  if (stats) {
    DFM2G_CUDA(cudaEventSynchronize(g_ws.ev1));
    float ms = 0.f;
    DFM2G_CUDA(cudaEventElapsedTime(&ms, g_ws.ev0, g_ws.ev1));
    stats->ms = ms;
    stats->iterations = total_it;
    stats->outer = outer;
    stats->rel_residual = rel;
  }
  return status;
} catch (...) {
  return host_failure();
}

}  // extern "C"

// ---- device vectors of the compatibility path (view_vectorx.h:61-109) ----------------
namespace dfm2g {
namespace {
__global__ void k_vec_axpy(size_t n, double *__restrict__ y, double a, const double *__restrict__ x) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
__global__ void k_vec_scale_add(size_t n, double *__restrict__ y, double b, const double *__restrict__ x) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = b * y[i] + x[i];
}
int vec_ws() {
  DFM2G_TRY(ensure_context());
  DFM2G_TRY(g_ws.partials.ensure((size_t)ctx().num_sms * 64));
  DFM2G_TRY(g_ws.scal.ensure(8));
  DFM2G_TRY(g_ws.tickets.ensure(4));
  return DFM2G_OK;
}
}  // namespace
}  // namespace dfm2g

extern "C" {

int dfm2g_dev_alloc(void **p, size_t bytes) try {
  if (!p) return fail(DFM2G_ERR_ARG, "dev_alloc: null out");
  DFM2G_TRY(ensure_context());
  *p = nullptr;
  if (bytes == 0) return DFM2G_OK;
  note_alloc();
  DFM2G_CUDA(cudaMalloc(p, bytes));
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_dev_free(void *p) try {
  if (p) {
    cudaStreamSynchronize(stream());
    DFM2G_CUDA(cudaFree(p));
  }
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_dev_copy(void *dst, const void *src, size_t bytes, int kind) try {
  if ((!dst || !src) && bytes) return fail(DFM2G_ERR_ARG, "dev_copy: null pointer");
  DFM2G_TRY(ensure_context());
  cudaMemcpyKind k;
  switch (kind) {
    case DFM2G_COPY_H2D: k = cudaMemcpyHostToDevice; break;
    case DFM2G_COPY_D2H: k = cudaMemcpyDeviceToHost; break;
    case DFM2G_COPY_D2D: k = cudaMemcpyDeviceToDevice; break;
    default: return fail(DFM2G_ERR_ARG, "dev_copy: unknown kind %d", kind);
  }
  if (bytes) DFM2G_CUDA(cudaMemcpyAsync(dst, src, bytes, k, stream()));
  if (kind != DFM2G_COPY_D2D) DFM2G_CUDA(cudaStreamSynchronize(stream()));
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_vec_dot(const double *x, const double *y, size_t n, double *out, int mem) try {
  if (!x || !y || !out) return fail(DFM2G_ERR_ARG, "vec_dot: null argument");
  DFM2G_TRY(vec_ws());
  VecArg<double> ax, ay;
  DFM2G_TRY(ax.in(x, n, mem, true));
  DFM2G_TRY(ay.in(y, n, mem, true));
  return dot_host(n, ax.dev(), ay.dev(), DFM2G_F64, out);
} catch (...) {
  return host_failure();
}

int dfm2g_vec_axpy(double *y, double alpha, const double *x, size_t n, int mem) try {
  if (!x || !y) return fail(DFM2G_ERR_ARG, "vec_axpy: null argument");
  DFM2G_TRY(ensure_context());
  VecArg<double> ax, ay;
  DFM2G_TRY(ax.in(x, n, mem, true));
  DFM2G_TRY(ay.in(y, n, mem, true));
  if (n) k_vec_axpy<<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(n, ay.dev(), alpha, ax.dev());
  note_launches(1);
  DFM2G_LAUNCH_CHECK();
  return ay.copy_back();
} catch (...) {
  return host_failure();
}

int dfm2g_vec_scale_add(double *y, double beta, const double *x, size_t n, int mem) try {
  if (!x || !y) return fail(DFM2G_ERR_ARG, "vec_scale_add: null argument");
  DFM2G_TRY(ensure_context());
  VecArg<double> ax, ay;
  DFM2G_TRY(ax.in(x, n, mem, true));
  DFM2G_TRY(ay.in(y, n, mem, true));
  if (n) k_vec_scale_add<<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(n, ay.dev(), beta, ax.dev());
  note_launches(1);
  DFM2G_LAUNCH_CHECK();
  return ay.copy_back();
} catch (...) {
  return host_failure();
}

int dfm2g_vec_set_zero(double *x, size_t n, int mem) try {
  if (!x) return fail(DFM2G_ERR_ARG, "vec_set_zero: null argument");
  if (mem == DFM2G_MEM_HOST) {
    std::memset(x, 0, sizeof(double) * n);
    return DFM2G_OK;
  }
  if (mem != DFM2G_MEM_DEVICE) return fail(DFM2G_ERR_ARG, "mem flag must be 0 (host) or 1 (device)");
  DFM2G_TRY(ensure_context());
  if (n) DFM2G_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, stream()));
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

}  // extern "C"

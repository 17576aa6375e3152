// Solve_PBiCGStab (include/delfem2/vecxitrsol.h:350-437) on the device, FP64,
// with the ILU preconditioner of ilu.cu and the SpMV of bsr.cu.
//
// x = 0; |r0|^2 < 1e-60 returns [|r0|]; r0* = r, p = r; for iitr = 1 ..
// max_niter-1: Mp = M^-1 p, alpha = (r, r0*)/(A Mp, r0*), s = r - alpha A Mp,
// Ms = M^-1 s, omega = (s, A Ms)/(A Ms, A Ms), x += alpha Mp, x += omega Ms,
// r = s - omega A Ms, history += |r|/|r0| (stop below tol),
// beta = (r, r0*) alpha / ((r, r0*)_old omega), p = beta p + r - beta omega A Mp.
// The scalars live on the device: each pair of dot products is one
// deterministic grid reduction whose last block applies the step's scalar
// update. The host reads the state once per iteration.
#include <cmath>

#include "common.cuh"

namespace dfm2g {

namespace {

struct BiState {
  double inv0, r_r2, alpha, omega, beta, tol;
  unsigned it, max_iter, nhist, hist_cap;
  int done;  // 0 running, 1 converged, 2 exhausted, 3 |r0|^2 < 1e-60, 4 non-finite
  unsigned ticket;
};

constexpr int kBiThreads = 256;
enum { kOpInit = 0, kOpRR2 = 1, kOpAlpha = 2, kOpOmega = 3, kOpConvBeta = 4 };

template <int OP>
__global__ void __launch_bounds__(kBiThreads) k_bi_dots(size_t n, const double *__restrict__ a1,
                                                        const double *__restrict__ b1, const double *__restrict__ a2,
                                                        const double *__restrict__ b2, double *partials, BiState *st,
                                                        double *hist) {
  __shared__ double sh[32];
  __shared__ bool last;
  double s1 = 0.0, s2 = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    s1 += a1[i] * b1[i];
    if (a2) s2 += a2[i] * b2[i];
  }
  s1 = block_sum(s1, sh);
  s2 = block_sum(s2, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = s1;
    partials[2 * blockIdx.x + 1] = s2;
    __threadfence();
    last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double t1 = 0.0, t2 = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    t1 += ld_relaxed(partials + 2 * b);
    t2 += ld_relaxed(partials + 2 * b + 1);
  }
  t1 = block_sum(t1, sh);
  t2 = block_sum(t2, sh);
  if (threadIdx.x != 0) return;
  st->ticket = 0;
  if (OP == kOpInit) {
    if (t1 < 1.0e-60) {
      if (st->hist_cap) hist[0] = sqrt(t1);
      st->nhist = 1;
      st->done = 3;
    } else {
      st->inv0 = 1.0 / t1;
    }
  } else if (OP == kOpRR2) {
    st->r_r2 = t1;
  } else if (OP == kOpAlpha) {
    st->alpha = st->r_r2 / t1;
  } else if (OP == kOpOmega) {
    st->omega = t2 / t1;  // t1 = (A Ms, A Ms), t2 = (s, A Ms)
  } else {                // t1 = (r, r), t2 = (r, r0*)
    const double ratio = sqrt(t1 * st->inv0);
    if (st->nhist < st->hist_cap) hist[st->nhist] = ratio;
    st->nhist++;
    st->it++;
    if (!isfinite(ratio))
      st->done = 4;
    else if (ratio < st->tol)
      st->done = 1;
    else if (st->it + 1 >= st->max_iter)
      st->done = 2;
    st->beta = t2 * st->alpha / (st->r_r2 * st->omega);
  }
}

// s = r - alpha A Mp
__global__ void k_bi_s(size_t n, const BiState *st, const double *__restrict__ r, const double *__restrict__ AMp,
                       double *__restrict__ s) {
  const double a = st->alpha;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s[i] = r[i] - a * AMp[i];
}

// x += alpha Mp; x += omega Ms; r = s - omega A Ms (the reference's order)
__global__ void k_bi_xr(size_t n, const BiState *st, double *__restrict__ x, double *__restrict__ r,
                        const double *__restrict__ Mp, const double *__restrict__ Ms, const double *__restrict__ s,
                        const double *__restrict__ AMs) {
  const double a = st->alpha, w = st->omega;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double xi = x[i];
    xi += a * Mp[i];
    xi += w * Ms[i];
    x[i] = xi;
    r[i] = s[i] + (-w) * AMs[i];
  }
}

// p = beta p + r - beta omega A Mp
__global__ void k_bi_p(size_t n, const BiState *st, double *__restrict__ p, const double *__restrict__ r,
                       const double *__restrict__ AMp) {
  if (st->done) return;
  const double b = st->beta, bw = -st->beta * st->omega;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = (b * p[i] + r[i]) + bw * AMp[i];
}

struct BiWorkspace {
  DevBuf<BiState> st;
  DevBuf<double> partials, hist, v[9];  // r0*, p, s, Mp, AMp, Ms, AMs, sweep scratch, b copy
};
BiWorkspace g_bi;

}  // namespace

}  // namespace dfm2g

using namespace dfm2g;

extern "C" {

int dfm2g_solve_pbicgstab(dfm2g_bsr m, dfm2g_ilu p, double *r, double *x, double tol, unsigned max_iter,
                          double *hist, unsigned hist_cap, unsigned *n_hist, int mem, dfm2g_solve_stats *stats) try {
  if (!m || !m->has_pattern) return fail(DFM2G_ERR_STATE, "solve_pbicgstab: matrix has no pattern");
  if (!p || !p->has_factor || p->nblk != m->nblk)
    return fail(DFM2G_ERR_STATE, "solve_pbicgstab: preconditioner not decomposed for this matrix");
  if (p->ndim != m->ndim) return fail(DFM2G_ERR_ARG, "solve_pbicgstab: preconditioner and matrix block sizes differ");
  if (!r || !x) return fail(DFM2G_ERR_ARG, "solve_pbicgstab: null vector");
  DFM2G_TRY(ensure_context());
  const size_t n = (size_t)m->nblk * m->ndim;
  if (n == 0) {  // an empty system: history [|r0|] = [0], as the |r0|^2 < 1e-60 early return
    if (hist && hist_cap) hist[0] = 0.0;
    if (n_hist) *n_hist = 1;
    if (stats) *stats = dfm2g_solve_stats{0u, 0u, 0.0, 0.0};
    return DFM2G_OK;
  }
  auto &W = g_bi;
  const unsigned grid = (unsigned)ctx().num_sms * 4;
  DFM2G_TRY(W.st.ensure(1));
  DFM2G_TRY(W.partials.ensure(2 * (size_t)grid));
  DFM2G_TRY(W.hist.ensure((size_t)max_iter + 4));
  for (auto &b : W.v) DFM2G_TRY(b.ensure(n + 1));
  double *r0 = W.v[0].p, *pv = W.v[1].p, *s = W.v[2].p, *Mp = W.v[3].p, *AMp = W.v[4].p, *Ms = W.v[5].p,
         *AMs = W.v[6].p, *tmp = W.v[7].p, *b0 = W.v[8].p;
  VecArg<double> ar, ax;
  DFM2G_TRY(ar.in(r, n, mem, true));
  DFM2G_TRY(ax.in(x, n, mem, false));
  double *rd = ar.dev(), *xd = ax.dev();
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (stats) {
    DFM2G_CUDA(cudaEventCreate(&e0));
    DFM2G_CUDA(cudaEventCreate(&e1));
    DFM2G_CUDA(cudaMemcpyAsync(b0, rd, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
    DFM2G_CUDA(cudaEventRecord(e0, stream()));
  }
  BiState init{};
  init.tol = tol;
  init.max_iter = max_iter;
  init.hist_cap = hist_cap;
  DFM2G_CUDA(cudaMemcpyAsync(W.st.p, &init, sizeof(init), cudaMemcpyHostToDevice, stream()));
  DFM2G_CUDA(cudaMemsetAsync(xd, 0, sizeof(double) * n, stream()));
  // A Mp and A Ms come from MatVec with beta = 0, which keeps a NaN already in
  // y (the reference's semantics): start them at zero, as its std::vectors do
  DFM2G_CUDA(cudaMemsetAsync(AMp, 0, sizeof(double) * n, stream()));
  DFM2G_CUDA(cudaMemsetAsync(AMs, 0, sizeof(double) * n, stream()));
  const unsigned vb = blocks_for(n, kBiThreads, grid);
  k_bi_dots<kOpInit><<<grid, kBiThreads, 0, stream()>>>(n, rd, rd, nullptr, nullptr, W.partials.p, W.st.p, W.hist.p);
  note_launches(1);
  DFM2G_LAUNCH_CHECK();
  BiState h{};
  DFM2G_CUDA(cudaMemcpyAsync(&h, W.st.p, sizeof(h), cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  if (!h.done && max_iter <= 1) h.done = 2;  // no iteration fits below max_niter
  if (!h.done) {
    DFM2G_CUDA(cudaMemcpyAsync(r0, rd, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
    DFM2G_CUDA(cudaMemcpyAsync(pv, rd, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
  }
  while (!h.done) {
    DFM2G_TRY(ilu_sweep(p, DFM2G_F64, true, pv, tmp));
    DFM2G_TRY(ilu_sweep(p, DFM2G_F64, false, tmp, Mp));
    k_bi_dots<kOpRR2><<<grid, kBiThreads, 0, stream()>>>(n, rd, r0, nullptr, nullptr, W.partials.p, W.st.p,
                                                          W.hist.p);
    DFM2G_TRY(bsr_spmv(m, DFM2G_F64, AMp, 1.0, Mp, 0.0));
    k_bi_dots<kOpAlpha><<<grid, kBiThreads, 0, stream()>>>(n, AMp, r0, nullptr, nullptr, W.partials.p, W.st.p,
                                                            W.hist.p);
    k_bi_s<<<vb, kBiThreads, 0, stream()>>>(n, W.st.p, rd, AMp, s);
    DFM2G_TRY(ilu_sweep(p, DFM2G_F64, true, s, tmp));
    DFM2G_TRY(ilu_sweep(p, DFM2G_F64, false, tmp, Ms));
    DFM2G_TRY(bsr_spmv(m, DFM2G_F64, AMs, 1.0, Ms, 0.0));
    k_bi_dots<kOpOmega><<<grid, kBiThreads, 0, stream()>>>(n, AMs, AMs, s, AMs, W.partials.p, W.st.p, W.hist.p);
    k_bi_xr<<<vb, kBiThreads, 0, stream()>>>(n, W.st.p, xd, rd, Mp, Ms, s, AMs);
    k_bi_dots<kOpConvBeta><<<grid, kBiThreads, 0, stream()>>>(n, rd, rd, rd, r0, W.partials.p, W.st.p, W.hist.p);
    k_bi_p<<<vb, kBiThreads, 0, stream()>>>(n, W.st.p, pv, rd, AMp);
    note_launches(8);
    DFM2G_LAUNCH_CHECK();
    DFM2G_CUDA(cudaMemcpyAsync(&h, W.st.p, sizeof(h), cudaMemcpyDeviceToHost, stream()));
    DFM2G_CUDA(cudaStreamSynchronize(stream()));
  }
  if (stats) DFM2G_CUDA(cudaEventRecord(e1, stream()));
  {  // a sweep wait that timed out, or an SpMV pipeline wait
    int e = 0;
    DFM2G_CUDA(cudaMemcpyAsync(&e, p->err.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
    DFM2G_CUDA(cudaStreamSynchronize(stream()));
    if (e) {
      DFM2G_CUDA(cudaMemsetAsync(p->err.p, 0, sizeof(int), stream()));
      return fail(DFM2G_ERR_WAIT_TIMEOUT, "solve_pbicgstab: a triangular-sweep wait timed out");
    }
    DFM2G_TRY(bsr_check_err(m));
  }
  if (hist && hist_cap) {
    const unsigned k = std::min(hist_cap, h.nhist);
    DFM2G_CUDA(cudaMemcpyAsync(hist, W.hist.p, sizeof(double) * k, cudaMemcpyDeviceToHost, stream()));
  }
  if (n_hist) *n_hist = h.nhist;
  if (stats) {
    DFM2G_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    DFM2G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    stats->ms = ms;
    stats->iterations = h.it;
    stats->outer = 1;
    // |b - A x| / |b| in FP64
    DFM2G_CUDA(cudaMemcpyAsync(tmp, b0, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream()));
    DFM2G_TRY(bsr_spmv(m, DFM2G_F64, tmp, -1.0, xd, 1.0));
    double rr = 0, bb = 0;
    DFM2G_TRY(dfm2g_vec_dot(tmp, tmp, n, &rr, DFM2G_MEM_DEVICE));
    DFM2G_TRY(dfm2g_vec_dot(b0, b0, n, &bb, DFM2G_MEM_DEVICE));
    stats->rel_residual = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  DFM2G_TRY(ar.copy_back());
  DFM2G_TRY(ax.copy_back());
  if (h.done == 4) return fail(DFM2G_ERR_NONFINITE, "solve_pbicgstab: non-finite residual");
  if (h.done == 2) return fail(DFM2G_ERR_NOT_CONVERGED, "solve_pbicgstab: %u iterations without reaching tol", h.it);
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

}  // extern "C"

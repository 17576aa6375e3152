// Row-range partitioned sync-free sweep (DFM2G_SWEEP_PARTS).
//
// The rows are split into P contiguous index ranges ("parts"), one per CTA of
// one co-resident (cooperative) grid. The forward sweep's dependencies point
// to lower row indices and the backward sweep's to higher ones, so part p only
// ever waits on itself and on parts before it (forward) or after it
// (backward). A CTA keeps the results of its own rows in shared memory
// (pending marker until written, like the global vector) and publishes every
// result to global memory too. A dependency inside the part is polled in
// shared memory (no L2 round trip); only cross-part dependencies are polled in
// global memory. Along any dependency path the number of global hand-offs is
// bounded by the number of part boundaries it crosses.
//
// Within a part, warp w takes positions w, w+NW, ... of the part's rows in the
// global (level, row) order. Every warp walks its positions in that order and
// all CTAs are resident, so the smallest unfinished position of the whole
// sweep can always proceed (its dependencies are all smaller): no deadlock.
// All waits are bounded (DFM2G_ERR_WAIT_TIMEOUT).
#include <algorithm>
#include <vector>

#include "rowkern.cuh"

namespace dfm2g {

namespace {

constexpr unsigned kPartThreads = 512;
constexpr size_t kPartSmemCap = 220 * 1024;  // per CTA, below the 227 KiB opt-in limit

template <typename T>
__device__ __forceinline__ T pending_value();
template <>
__device__ __forceinline__ float pending_value<float>() {
  return __uint_as_float(0xffffffffu);
}
template <>
__device__ __forceinline__ double pending_value<double>() {
  return __longlong_as_double(-1ll);
}

template <typename T>
__device__ __forceinline__ T ld_shared_poll(const T *p) {
  return *(const volatile T *)p;
}

// Sum of the lane's products; x_j comes from the part's shared copy when j is
// one of the part's rows (r0 <= j < r0 + len), else from global memory. All
// still-pending values are re-polled together each round.
template <typename T, unsigned R>
__device__ __forceinline__ T row_dot_wait_part(const RowFrag<T, R> &f, const RowLane &L, const T *x, const T *xs,
                                               unsigned r0, unsigned len, int *err,
                                               unsigned long long timeout_ns) {
  T xv[R];
  const T *px[R];
  bool loc[R];
#pragma unroll
  for (unsigned k = 0; k < R; ++k) {
    const unsigned j = f.j[k];
    loc[k] = (j - r0) < len;
    px[k] = loc[k] ? xs + (size_t)(j - r0) * 3 + L.c : x + (size_t)j * 3 + L.c;
    xv[k] = (L.active && 3u * k + L.g < f.nb) ? (loc[k] ? ld_shared_poll(px[k]) : ld_relaxed(px[k])) : T(0);
  }
  bool pending = false;
#pragma unroll
  for (unsigned k = 0; k < R; ++k) pending |= is_pending(xv[k]);
  if (pending) {
    const unsigned long long t0 = globaltimer_ns();
    unsigned spins = 0;
    for (;;) {
#pragma unroll
      for (unsigned k = 0; k < R; ++k)
        if (is_pending(xv[k])) xv[k] = loc[k] ? ld_shared_poll(px[k]) : ld_relaxed(px[k]);
      pending = false;
#pragma unroll
      for (unsigned k = 0; k < R; ++k) pending |= is_pending(xv[k]);
      if (!pending) break;
      if ((++spins & 15u) == 0 && (ld_relaxed(err) != 0 || globaltimer_ns() - t0 > timeout_ns)) {
        atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
#pragma unroll
        for (unsigned k = 0; k < R; ++k)
          if (is_pending(xv[k])) xv[k] = T(0);
        break;
      }
    }
  }
  T acc = T(0);
#pragma unroll
  for (unsigned k = 0; k < R; ++k) acc += f.v[k] * xv[k];
  return acc;
}

template <typename T>
__device__ __forceinline__ T wait_part_value(const T *p, bool local, int *err, unsigned long long timeout_ns) {
  T v = local ? ld_shared_poll(p) : ld_relaxed(p);
  if (!is_pending(v)) return v;
  const unsigned long long t0 = globaltimer_ns();
  unsigned spins = 0;
  while (is_pending(v = (local ? ld_shared_poll(p) : ld_relaxed(p)))) {
    if ((++spins & 15u) == 0 && (ld_relaxed(err) != 0 || globaltimer_ns() - t0 > timeout_ns)) {
      atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
      return T(0);
    }
  }
  return v;
}

template <typename T>
struct PartRow {
  static constexpr unsigned kRounds = 4;
  RowFrag<T, kRounds> f;
  unsigned i, s0, s1;
  T in[3];
  T d[3];
};

template <typename T, bool FWD>
__device__ __forceinline__ void part_load(PartRow<T> &R, const RowLane &L, unsigned lane, uint4 m,
                                          const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                          const T *__restrict__ vdia, const T *in) {
  R.i = m.x;
  R.s0 = m.y;
  R.s1 = m.z;
  row_load(R.f, L, m.y, m.z, col, vcrs, ~0u, (const T *)nullptr);
  if (lane < 3) {
#pragma unroll
    for (int k = 0; k < 3; ++k) R.in[k] = in[(size_t)m.x * 3 + k];
    if (FWD) {
#pragma unroll
      for (int k = 0; k < 3; ++k) R.d[k] = vdia[(size_t)m.x * 9 + lane * 3 + k];
    }
  }
}

template <typename T, bool FWD>
__device__ __forceinline__ void part_finish(const PartRow<T> &R, const RowLane &L, unsigned lane,
                                            const unsigned *__restrict__ col, const T *__restrict__ vcrs, T *out,
                                            T *xs, unsigned r0, unsigned len, int *err,
                                            unsigned long long timeout_ns) {
  T acc = T(0);
  if (R.f.nb <= 3 * PartRow<T>::kRounds) {
    acc = row_dot_wait_part(R.f, L, out, xs, r0, len, err, timeout_ns);
  } else if (L.active) {
    for (unsigned t = R.s0 + L.g; t < R.s1; t += 3u) {
      const unsigned j = col[t];
      const bool local = (j - r0) < len;
      const T *p = local ? xs + (size_t)(j - r0) * 3 + L.c : out + (size_t)j * 3 + L.c;
      acc += vcrs[(size_t)t * 9 + L.e] * wait_part_value(p, local, err, timeout_ns);
    }
  }
  T s[3];
  row_reduce(acc, s);
  if (lane < 3) {
    const T t0 = R.in[0] - s[0], t1 = R.in[1] - s[1], t2 = R.in[2] - s[2];
    T z;
    if (FWD)
      z = R.d[0] * t0 + R.d[1] * t1 + R.d[2] * t2;
    else
      z = lane == 0 ? t0 : (lane == 1 ? t1 : t2);
    *(volatile T *)(xs + (size_t)(R.i - r0) * 3 + lane) = z;
    st_relaxed(out + (size_t)R.i * 3 + lane, z);
  }
}

template <typename T, bool FWD>
__global__ void __launch_bounds__(kPartThreads) k_sweep_parts(const uint4 *__restrict__ meta,
                                                              const unsigned *__restrict__ pstart,
                                                              unsigned rows_per_part, unsigned nblk,
                                                              const unsigned *__restrict__ col,
                                                              const T *__restrict__ vcrs, const T *__restrict__ vdia,
                                                              const T *in, T *out, int *err,
                                                              unsigned long long timeout_ns, const int *skip) {
  extern __shared__ __align__(16) unsigned char part_smem[];
  T *xs = reinterpret_cast<T *>(part_smem);
  if (skip && *skip) return;
  const unsigned p = blockIdx.x;
  const unsigned r0 = p * rows_per_part;
  const unsigned len = r0 < nblk ? min(rows_per_part, nblk - r0) : 0u;
  for (unsigned k = threadIdx.x; k < len * 3u; k += blockDim.x) xs[k] = pending_value<T>();
  __syncthreads();
  constexpr unsigned NW = kPartThreads / 32u;
  const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  const unsigned qend = pstart[p + 1];
  unsigned q = pstart[p] + w;
  if (q >= qend) return;
  const RowLane L(lane);
  PartRow<T> cur, nxt;
  part_load<T, FWD>(cur, L, lane, meta[q], col, vcrs, vdia, in);
  uint4 m1 = (q + NW < qend) ? meta[q + NW] : make_uint4(0u, 0u, 0u, 0u);
  for (;;) {
    const unsigned q1 = q + NW;
    if (q1 < qend) part_load<T, FWD>(nxt, L, lane, m1, col, vcrs, vdia, in);
    const unsigned q2 = q1 + NW;
    const uint4 m2 = (q2 < qend) ? meta[q2] : make_uint4(0u, 0u, 0u, 0u);
    part_finish<T, FWD>(cur, L, lane, col, vcrs, out, xs, r0, len, err, timeout_ns);
    if (q1 >= qend) break;
    q = q1;
    cur = nxt;
    m1 = m2;
  }
}

// Opts the kernel in to the full cap (patterns of any size share the kernel)
// and reports how many CTAs with `smem` bytes fit on one SM.
template <typename T, bool FWD>
int part_kernel_setup(size_t smem, int *blocks_per_sm) {
  auto kernel = k_sweep_parts<T, FWD>;
  DFM2G_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPartSmemCap));
  DFM2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel, kPartThreads, smem));
  return DFM2G_OK;
}

__global__ void k_part_meta(unsigned n, const unsigned *__restrict__ order, const unsigned *__restrict__ row_start,
                            const unsigned *__restrict__ dia_ind, int backward, uint4 *__restrict__ meta) {
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const unsigned i = order[q];
    const unsigned s0 = backward ? dia_ind[i] : row_start[i];
    const unsigned s1 = backward ? row_start[i + 1] : dia_ind[i];
    meta[q] = make_uint4(i, s0, s1, 0u);
  }
}

// Per part, its rows in the level order of the sweep (a stable partition of
// the global order by part), as position metadata, and the part offsets.
int build_direction(dfm2g_ilu_s *p, bool backward, unsigned nparts, unsigned rpp, PartSched &ps) {
  const unsigned n = p->nblk;
  std::vector<unsigned> order(n), out(n), start(nparts + 1, 0);
  DFM2G_CUDA(cudaMemcpyAsync(order.data(), backward ? p->order_b.p : p->order_f.p, sizeof(unsigned) * n,
                             cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  for (unsigned q = 0; q < n; ++q) start[order[q] / rpp + 1]++;
  for (unsigned k = 0; k < nparts; ++k) start[k + 1] += start[k];
  std::vector<unsigned> cur(start.begin(), start.end() - 1);
  for (unsigned q = 0; q < n; ++q) out[cur[order[q] / rpp]++] = order[q];
  DevBuf<unsigned> d_order;
  DFM2G_TRY(d_order.resize(n));
  DFM2G_TRY(ps.meta.resize((size_t)n + 1));
  DFM2G_TRY(ps.pstart.resize(nparts + 1));
  DFM2G_CUDA(cudaMemcpyAsync(d_order.p, out.data(), sizeof(unsigned) * n, cudaMemcpyHostToDevice, stream()));
  DFM2G_CUDA(cudaMemcpyAsync(ps.pstart.p, start.data(), sizeof(unsigned) * (nparts + 1), cudaMemcpyHostToDevice,
                             stream()));
  k_part_meta<<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(n, d_order.p, p->row_start.p,
                                                                           p->dia_ind.p, backward ? 1 : 0, ps.meta.p);
  DFM2G_LAUNCH_CHECK();
  DFM2G_CUDA(cudaStreamSynchronize(stream()));  // d_order is freed on return
  return DFM2G_OK;
}

}  // namespace

// Partition: one part per SM (rows_per_part = ceil(n / SMs)), usable when a
// part's FP64 results fit in shared memory and every part's CTA is resident.
int part_schedules_build(dfm2g_ilu_s *p) {
  p->parts_ok = false;
  const unsigned n = p->nblk;
  const unsigned nsm = (unsigned)ctx().num_sms;
  if (n == 0) return DFM2G_OK;
  const unsigned rpp = (n + nsm - 1) / nsm;
  const unsigned nparts = (n + rpp - 1) / rpp;
  const size_t smem64 = (size_t)rpp * 3 * sizeof(double), smem32 = (size_t)rpp * 3 * sizeof(float);
  if (smem64 > kPartSmemCap) return DFM2G_OK;
  int b64f = 0, b64b = 0, b32f = 0, b32b = 0;
  DFM2G_TRY((part_kernel_setup<double, true>(smem64, &b64f)));
  DFM2G_TRY((part_kernel_setup<double, false>(smem64, &b64b)));
  DFM2G_TRY((part_kernel_setup<float, true>(smem32, &b32f)));
  DFM2G_TRY((part_kernel_setup<float, false>(smem32, &b32b)));
  const int resident = (int)nsm * std::min(std::min(b64f, b64b), std::min(b32f, b32b));
  if (resident < (int)nparts) return DFM2G_OK;
  DFM2G_TRY(build_direction(p, false, nparts, rpp, p->parts_f));
  DFM2G_TRY(build_direction(p, true, nparts, rpp, p->parts_b));
  p->parts_rpp = rpp;
  p->parts_n = nparts;
  p->parts_ok = true;
  return DFM2G_OK;
}

template <typename T>
int part_sweep(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia, const int *skip,
               unsigned long long timeout) {
  const PartSched &ps = forward ? p->parts_f : p->parts_b;
  const size_t smem = (size_t)p->parts_rpp * 3 * sizeof(T);
  void *kernel = forward ? (void *)k_sweep_parts<T, true> : (void *)k_sweep_parts<T, false>;
  unsigned rpp = p->parts_rpp, n = p->nblk;
  int *err = p->err.p;
  const uint4 *meta = ps.meta.p;
  const unsigned *pstart = ps.pstart.p;
  void *args[] = {(void *)&meta, (void *)&pstart, (void *)&rpp,  (void *)&n,   (void *)&p->col.p, (void *)&vcrs,
                  (void *)&vdia, (void *)&in,     (void *)&out,  (void *)&err, (void *)&timeout,  (void *)&skip};
  DFM2G_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(p->parts_n), dim3(kPartThreads), args, smem, stream()));
  note_launches(1);
  return DFM2G_OK;
}

template int part_sweep<float>(dfm2g_ilu_s *, bool, const float *, float *, const float *, const float *,
                               const int *, unsigned long long);
template int part_sweep<double>(dfm2g_ilu_s *, bool, const double *, double *, const double *, const double *,
                                const int *, unsigned long long);

}  // namespace dfm2g

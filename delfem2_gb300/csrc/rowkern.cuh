// Warp-per-block-row building blocks shared by the SpMV, the residual and the
// triangular sweeps.
//
// Lane layout: lanes 0..26 form three groups of nine; group g = lane/9 takes
// block 3k+g of the row in round k, and lane e = lane%9 inside the group always
// takes entry (r, c) = (e/3, e%3) of that 3x3 block. So each lane accumulates
// into ONE row component with one FMA per matrix entry, and the row's three
// sums need only 7 shuffles (sum over c, then over the three groups, then a
// broadcast). A row's blocks are [s0, s1) of the block arrays, optionally
// followed by one extra block (the diagonal, at `extra_row`).
//
// R rounds (3R blocks) of a row are held in registers; longer rows take the
// *_long paths, which read everything inline.
#pragma once

#include "common.cuh"

namespace dfm2g {

// Pause between polls of a value another warp has not written yet (limits the
// L2 request traffic of thousands of waiting warps). 0 = spin.
#ifndef DFM2G_POLL_BACKOFF_NS
#define DFM2G_POLL_BACKOFF_NS 0
#endif
constexpr unsigned kPollBackoffNs = DFM2G_POLL_BACKOFF_NS;

template <typename T, unsigned R>
struct RowFrag {
  T v[R];
  unsigned j[R];  // block column of each round's block (for the lane's c)
  unsigned nb;    // blocks in this row (including the extra block)
};

struct RowLane {
  unsigned g, e, r, c;
  bool active;
  __device__ __forceinline__ RowLane(unsigned lane) {
    g = lane / 9u;
    e = lane - g * 9u;
    r = e / 3u;
    c = e - r * 3u;
    active = lane < 27u;
  }
};

// Issue the loads of a row's values and block columns (no use of them yet).
// `extra_row` != ~0u appends the block (extra_row, extra_row) read from `vextra`.
template <typename T, unsigned R>
__device__ __forceinline__ void row_load(RowFrag<T, R> &f, const RowLane &L, unsigned s0, unsigned s1,
                                         const unsigned *__restrict__ col, const T *__restrict__ vals,
                                         unsigned extra_row, const T *__restrict__ vextra) {
  const unsigned noff = s1 - s0;
  f.nb = noff + (extra_row != ~0u ? 1u : 0u);
#pragma unroll
  for (unsigned k = 0; k < R; ++k) {
    const unsigned t = 3u * k + L.g;
    f.v[k] = T(0);
    f.j[k] = 0u;
    if (L.active && t < f.nb) {
      if (t < noff) {
        f.j[k] = col[s0 + t];
        f.v[k] = vals[(size_t)(s0 + t) * 9 + L.e];
      } else {
        f.j[k] = extra_row;
        f.v[k] = vextra[(size_t)extra_row * 9 + L.e];
      }
    }
  }
}

// Sum of the lane's products over a fragment. x is read with plain loads.
template <typename T, unsigned R>
__device__ __forceinline__ T row_dot(const RowFrag<T, R> &f, const RowLane &L, const T *__restrict__ x) {
  T xv[R];
#pragma unroll
  for (unsigned k = 0; k < R; ++k) xv[k] = (L.active && 3u * k + L.g < f.nb) ? x[(size_t)f.j[k] * 3 + L.c] : T(0);
  T acc = T(0);
#pragma unroll
  for (unsigned k = 0; k < R; ++k) acc += f.v[k] * xv[k];
  return acc;
}

// Same, for rows longer than the register path (any length), loads inline.
template <typename T>
__device__ __forceinline__ T row_dot_long(const RowLane &L, unsigned s0, unsigned s1,
                                          const unsigned *__restrict__ col, const T *__restrict__ vals,
                                          unsigned extra_row, const T *__restrict__ vextra,
                                          const T *__restrict__ x) {
  const unsigned noff = s1 - s0, nb = noff + (extra_row != ~0u ? 1u : 0u);
  T acc = T(0);
  for (unsigned t = L.g; t < nb; t += 3u) {
    if (!L.active) break;
    unsigned j;
    T v;
    if (t < noff) {
      j = col[s0 + t];
      v = vals[(size_t)(s0 + t) * 9 + L.e];
    } else {
      j = extra_row;
      v = vextra[(size_t)extra_row * 9 + L.e];
    }
    acc += v * x[(size_t)j * 3 + L.c];
  }
  return acc;
}

// Row sums from the per-lane partials: returns them in s[0..2] on every lane.
template <typename T>
__device__ __forceinline__ void row_reduce(T acc, T s[3]) {
  acc += __shfl_down_sync(0xffffffffu, acc, 1) + __shfl_down_sync(0xffffffffu, acc, 2);
  acc += __shfl_down_sync(0xffffffffu, acc, 9) + __shfl_down_sync(0xffffffffu, acc, 18);
  s[0] = __shfl_sync(0xffffffffu, acc, 0);
  s[1] = __shfl_sync(0xffffffffu, acc, 3);
  s[2] = __shfl_sync(0xffffffffu, acc, 6);
}

template <typename T>
__device__ __forceinline__ T pick3(const T s[3], unsigned i) {
  return i == 0 ? s[0] : (i == 1 ? s[1] : s[2]);
}

// Walk this warp's block rows (w, w+W, ...) of K (off-diagonal blocks then
// the diagonal) computing s = (K x)_row, and hand each row to epi(row, s).
// Software-pipelined: the next row's block columns and values are requested
// before the current row's x entries are gathered, and the row offsets two
// rows ahead before that.
template <typename T, typename Epi>
__device__ __forceinline__ void spmv_rows(unsigned nblk, const unsigned *__restrict__ row_start,
                                          const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                          const T *__restrict__ vdia, const T *__restrict__ x, Epi &&epi) {
  constexpr unsigned R = 6;  // 17 off-diagonal blocks + the diagonal in registers
  const RowLane L(threadIdx.x & 31);
  const unsigned nwarp = (gridDim.x * blockDim.x) >> 5;
  unsigned row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (row >= nblk) return;
  unsigned a0 = row_start[row], a1 = row_start[row + 1];
  RowFrag<T, R> f;
  row_load(f, L, a0, a1, col, vcrs, row, vdia);
  unsigned nrow = row + nwarp;
  unsigned b0 = 0, b1 = 0;
  if (nrow < nblk) {
    b0 = row_start[nrow];
    b1 = row_start[nrow + 1];
  }
  for (;;) {
    RowFrag<T, R> fn;
    if (nrow < nblk) row_load(fn, L, b0, b1, col, vcrs, nrow, vdia);
    const unsigned nn = nrow + nwarp;
    unsigned c0 = 0, c1 = 0;
    if (nn < nblk) {
      c0 = row_start[nn];
      c1 = row_start[nn + 1];
    }
    const T acc = (f.nb <= 3 * R) ? row_dot(f, L, x) : row_dot_long(L, a0, a1, col, vcrs, row, vdia, x);
    T s[3];
    row_reduce(acc, s);
    epi(row, s);
    if (nrow >= nblk) break;
    row = nrow;
    nrow = nn;
    f = fn;
    a0 = b0;
    a1 = b1;
    b0 = c0;
    b1 = c1;
  }
}

// Bounded wait until *p is no longer the pending marker; returns the value.
// On timeout (or when another warp already reported one) records the error
// and returns 0.
template <typename T>
__device__ __forceinline__ T wait_value(const T *p, int *err, unsigned long long timeout_ns) {
  T v = ld_relaxed(p);
  if (!is_pending(v)) return v;
  const unsigned long long t0 = globaltimer_ns();
  unsigned spins = 0;
  while (is_pending(v = ld_relaxed(p))) {
    if ((++spins & 15u) == 0 && (ld_relaxed(err) != 0 || globaltimer_ns() - t0 > timeout_ns)) {
      atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
      return T(0);
    }
  }
  return v;
}

// Sum of the lane's products where x values are produced concurrently by other
// warps. Every poll round re-reads ALL of the lane's still-pending values at
// once, so a lane waits one round trip per poll, not one per dependency.
template <typename T, unsigned R>
__device__ __forceinline__ T row_dot_wait(const RowFrag<T, R> &f, const RowLane &L, const T *x, int *err,
                                          unsigned long long timeout_ns) {
  T xv[R];
  const T *px[R];
#pragma unroll
  for (unsigned k = 0; k < R; ++k) {
    px[k] = x + (size_t)f.j[k] * 3 + L.c;
    xv[k] = (L.active && 3u * k + L.g < f.nb) ? ld_relaxed(px[k]) : T(0);
  }
  bool pending = false;
#pragma unroll
  for (unsigned k = 0; k < R; ++k) pending |= is_pending(xv[k]);
  if (pending) {
    const unsigned long long t0 = globaltimer_ns();
    unsigned spins = 0;
    for (;;) {
      if (kPollBackoffNs) __nanosleep(kPollBackoffNs);
#pragma unroll
      for (unsigned k = 0; k < R; ++k)
        if (is_pending(xv[k])) xv[k] = ld_relaxed(px[k]);
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
__device__ __forceinline__ T row_dot_wait_long(const RowLane &L, unsigned s0, unsigned s1,
                                               const unsigned *__restrict__ col, const T *__restrict__ vals,
                                               const T *x, int *err, unsigned long long timeout_ns) {
  T acc = T(0);
  for (unsigned t = s0 + L.g; t < s1; t += 3u) {
    if (!L.active) break;
    const unsigned j = col[t];
    acc += vals[(size_t)t * 9 + L.e] * wait_value(x + (size_t)j * 3 + L.c, err, timeout_ns);
  }
  return acc;
}

}  // namespace dfm2g

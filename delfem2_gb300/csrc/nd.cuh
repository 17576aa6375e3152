// Row primitives for 1x1 and 2x2 blocks (CMatrixSparse with ndim 1 or 2; the
// 3x3 path has its own lane layout in rowkern.cuh).
//
// The lanes given a block row stride over its off-diagonal blocks; each lane
// keeps B partial sums (one per row of the block), and shuffles add them, so
// every lane ends with the row's B sums. The sweeps give a row a warp (one
// pass covers a triangle of up to 32 blocks); the products give a row eight
// lanes (scalar rows of a tet mesh hold about 14 blocks, 2-D triangle rows
// about 6).
#pragma once

#include "common.cuh"
#include "rowkern.cuh"

namespace dfm2g {

// This lane's share of acc[r] += sum over blocks s in [s0, s1) of
// sum_c A_s[r][c] x[col[s]][c] (blocks s0 + lane, s0 + lane + 32, ...; no
// reduction). With WAIT, each x entry is read with a bounded wait on the
// pending marker (the sync-free sweeps); a timeout records
// DFM2G_ERR_WAIT_TIMEOUT in *err and reads 0.
template <typename T, int B, bool WAIT>
__device__ __forceinline__ void nd_row_partial(unsigned lane, unsigned s0, unsigned s1,
                                               const unsigned *__restrict__ col, const T *__restrict__ vals,
                                               const T *x, T acc[B], int *err, unsigned long long timeout_ns) {
  for (unsigned s = s0 + lane; s < s1; s += 32) {
    const unsigned j = col[s];
    T xj[B];
#pragma unroll
    for (int c = 0; c < B; ++c) {
      if constexpr (WAIT)
        xj[c] = wait_value(x + (size_t)j * B + c, err, timeout_ns);
      else
        xj[c] = x[(size_t)j * B + c];
    }
    const T *a = vals + (size_t)s * (B * B);
#pragma unroll
    for (int r = 0; r < B; ++r) {
      T t = a[r * B] * xj[0];
#pragma unroll
      for (int c = 1; c < B; ++c) t += a[r * B + c] * xj[c];
      acc[r] += t;
    }
  }
}

// acc[r] = the whole warp's sum of nd_row_partial, in every lane.
template <typename T, int B, bool WAIT>
__device__ __forceinline__ void nd_row_sum(unsigned lane, unsigned s0, unsigned s1,
                                           const unsigned *__restrict__ col, const T *__restrict__ vals,
                                           const T *x, T acc[B], int *err, unsigned long long timeout_ns) {
#pragma unroll
  for (int r = 0; r < B; ++r) acc[r] = T(0);
  nd_row_partial<T, B, WAIT>(lane, s0, s1, col, vals, x, acc, err, timeout_ns);
#pragma unroll
  for (int r = 0; r < B; ++r) acc[r] = warp_sum(acc[r]);
}

// v[lane] for lane < B without indexing a register array by a lane number.
template <typename T, int B>
__device__ __forceinline__ T nd_pick(const T v[B], unsigned lane) {
  T out = v[0];
#pragma unroll
  for (int r = 1; r < B; ++r)
    if ((unsigned)r == lane) out = v[r];
  return out;
}

// Calls f(row, s, sub) for every block row, s = (row of A) x, in every lane
// of the row's group: kNdGroup consecutive lanes per row (4 rows per warp), so
// a warp has four rows' dependent loads in flight instead of one; sub is the
// lane's index in its group. The loop is uniform across the warp (rows past
// the end are skipped inside), so the group shuffles run with every lane.
constexpr unsigned kNdGroup = 8;

template <typename T, int B, typename F>
__device__ __forceinline__ void nd_spmv_rows(unsigned nblk, const unsigned *__restrict__ row_start,
                                             const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                             const T *__restrict__ vdia, const T *__restrict__ x, F &&f) {
  constexpr unsigned G = kNdGroup, GPW = 32 / G;
  const unsigned lane = threadIdx.x & 31, sub = lane % G, grp = lane / G;
  const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned nwarp = (gridDim.x * blockDim.x) >> 5;
  for (size_t base = (size_t)warp * GPW; base < nblk; base += (size_t)nwarp * GPW) {
    const size_t row = base + grp;
    T acc[B];
#pragma unroll
    for (int r = 0; r < B; ++r) acc[r] = T(0);
    if (row < nblk) {
      const unsigned s0 = row_start[row], s1 = row_start[row + 1];
      for (unsigned s = s0 + sub; s < s1; s += G) {
        const unsigned j = col[s];
        const T *a = vcrs + (size_t)s * (B * B);
#pragma unroll
        for (int r = 0; r < B; ++r) {
          T t = a[r * B] * x[(size_t)j * B];
#pragma unroll
          for (int c = 1; c < B; ++c) t += a[r * B + c] * x[(size_t)j * B + c];
          acc[r] += t;
        }
      }
      if (sub == G - 1) {  // the diagonal block
        const T *d = vdia + row * (B * B);
#pragma unroll
        for (int r = 0; r < B; ++r)
#pragma unroll
          for (int c = 0; c < B; ++c) acc[r] += d[r * B + c] * x[row * B + c];
      }
    }
#pragma unroll
    for (int r = 0; r < B; ++r)
#pragma unroll
      for (unsigned o = G / 2; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
    if (row < nblk) f((unsigned)row, acc, sub);
  }
}

}  // namespace dfm2g

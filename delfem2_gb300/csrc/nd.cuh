// Warp-per-block-row primitives for 1x1 and 2x2 blocks (CMatrixSparse with
// ndim 1 or 2; the 3x3 path has its own lane layout in rowkern.cuh).
//
// A warp owns one block row. Its lanes stride over the row's off-diagonal
// blocks; each lane keeps B partial sums (one per row of the block), and the
// warp adds them with shuffles, so every lane ends with the row's B sums.
// Scalar rows of a tet mesh hold about 14 blocks and 2-D triangle rows about
// 6, so one pass of the lanes covers a row.
#pragma once

#include "common.cuh"
#include "rowkern.cuh"

namespace dfm2g {

// acc[r] = sum over blocks s in [s0, s1) of sum_c A_s[r][c] x[col[s]][c]. With
// WAIT, each x entry is read with a bounded wait on the pending marker (the
// sync-free sweeps); a timeout records DFM2G_ERR_WAIT_TIMEOUT in *err and
// reads 0.
template <typename T, int B, bool WAIT>
__device__ __forceinline__ void nd_row_sum(unsigned lane, unsigned s0, unsigned s1,
                                           const unsigned *__restrict__ col, const T *__restrict__ vals,
                                           const T *x, T acc[B], int *err, unsigned long long timeout_ns) {
#pragma unroll
  for (int r = 0; r < B; ++r) acc[r] = T(0);
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
#pragma unroll
  for (int r = 0; r < B; ++r) acc[r] = warp_sum(acc[r]);
}

// s = (row i of A) x: the off-diagonal blocks, then the diagonal block.
template <typename T, int B>
__device__ __forceinline__ void nd_row_product(unsigned lane, unsigned i, const unsigned *__restrict__ row_start,
                                               const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                               const T *__restrict__ vdia, const T *__restrict__ x, T s[B]) {
  nd_row_sum<T, B, false>(lane, row_start[i], row_start[i + 1], col, vcrs, x, s, nullptr, 0);
  const T *d = vdia + (size_t)i * (B * B);
  const T *xi = x + (size_t)i * B;
#pragma unroll
  for (int r = 0; r < B; ++r)
#pragma unroll
    for (int c = 0; c < B; ++c) s[r] += d[r * B + c] * xi[c];
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

// Calls f(row, s) for every block row of the grid's warps, s = (row of A) x.
template <typename T, int B, typename F>
__device__ __forceinline__ void nd_spmv_rows(unsigned nblk, const unsigned *__restrict__ row_start,
                                             const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                             const T *__restrict__ vdia, const T *__restrict__ x, F &&f) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned nwarp = (gridDim.x * blockDim.x) >> 5;
  for (unsigned row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nblk; row += nwarp) {
    T s[B];
    nd_row_product<T, B>(lane, row, row_start, col, vcrs, vdia, x, s);
    f(row, s);
  }
}

}  // namespace dfm2g

// TMA-staged 3x3 block SpMV: warp-specialised, persistent.
//
// The block rows are cut into tiles of consecutive rows (at most kBlocks
// off-diagonal blocks and kRows rows each; tile table built on the host from
// the pattern). A persistent grid (one CTA per SM) takes tiles round-robin. In
// each CTA one producer warp streams a tile's off-diagonal values, block
// columns, diagonal blocks and row offsets - four contiguous byte ranges,
// rounded out to 16 bytes - into a double-buffered shared-memory ring with
// cp.async.bulk, completing on a "full" mbarrier per stage; the consumer warps
// compute the tile's rows from shared memory (x gathered from global memory,
// read-only) and release the stage on an "empty" mbarrier. Every wait is
// bounded; on a timeout the kernel records DFM2G_ERR_WAIT_TIMEOUT and the
// producer still waits (bounded) for its copies in flight before exiting.
#pragma once

#include "rowkern.cuh"
#include "tma.cuh"

namespace dfm2g {

// Byte range [off, end) rounded out to 16 bytes: (aligned start, length).
__device__ __forceinline__ void round16(size_t off, size_t end, size_t &a, unsigned &len) {
  a = off & ~size_t(15);
  len = (unsigned)(((end + 15) & ~size_t(15)) - a);
}

// ---------------------------------------------------------------------------
// Component layout: lane 3q + a of a consumer warp computes component a of
// row q of the warp's ten rows, summing K_b[a][0..2] x_b over the row's
// blocks with no cross-lane reduction. A warp instruction then serves ten rows
// (the lane layout above: one row per 27 lanes plus a 7-shuffle reduction), so
// the kernel issues a fraction of the instructions per row (and, in FP64, of
// the FP64 instructions). Tiles hold ten rows per consumer warp and are
// double-buffered; the tile's row offsets are staged with its values, block
// columns and diagonal blocks. FP32: 15 consumer warps (150-row tiles), FP64:
// 7 (70-row tiles), one CTA per SM.
#ifndef DFM2G_SPMV_F32_CONSUMERS
#define DFM2G_SPMV_F32_CONSUMERS 15u  // FP32 tile: consumer warps (ten rows each)
#endif
#ifndef DFM2G_SPMV_F32_BLOCKS
#define DFM2G_SPMV_F32_BLOCKS 2304u  // FP32 tile: blocks at most
#endif
#ifndef DFM2G_SPMV_F32_STAGES
#define DFM2G_SPMV_F32_STAGES 2u  // FP32 ring stages
#endif
template <typename T>
struct TileCfgC {
  static constexpr unsigned kConsumers = sizeof(T) == 8 ? 7u : DFM2G_SPMV_F32_CONSUMERS;
  static constexpr unsigned kThreads = 32u * (kConsumers + 1u);
  static constexpr unsigned kRows = kConsumers * 10u;
  static constexpr unsigned kBlocks = sizeof(T) == 8 ? 1152u : DFM2G_SPMV_F32_BLOCKS;
  static constexpr unsigned kStages = sizeof(T) == 8 ? 2u : DFM2G_SPMV_F32_STAGES;
  static constexpr unsigned kValBytes = kBlocks * 9 * sizeof(T) + 32;
  static constexpr unsigned kColBytes = kBlocks * 4 + 32;
  static constexpr unsigned kDiaBytes = (kRows * 9 * sizeof(T) + 32 + 15) / 16 * 16;
  static constexpr unsigned kRsBytes = ((kRows + 1) * 4 + 32 + 15) / 16 * 16;
  static constexpr unsigned kStageBytes = kValBytes + kColBytes + kDiaBytes + kRsBytes;
  static constexpr unsigned kBarBytes = 128;
  static constexpr size_t kSmem = kBarBytes + (size_t)kStages * kStageBytes;
  static_assert(kValBytes % 16 == 0 && kColBytes % 16 == 0 && kDiaBytes % 16 == 0 && kRsBytes % 16 == 0,
                "16-byte stage layout");
  static_assert(kSmem <= 227u * 1024u, "fits one CTA's shared memory");
};

// Runs the pipeline over all tiles; epi(row, a, v) is called by the lane that
// computed component a of `row` (v = (K x)_{3 row + a}). Must be called by all
// TileCfgC<T>::kThreads threads of the CTA; `smem` holds TileCfgC<T>::kSmem bytes.
template <typename T, typename Epi>
__device__ __forceinline__ void spmv_tma_rows_c(const unsigned *__restrict__ tiles, unsigned ntiles,
                                                const unsigned *__restrict__ row_start,
                                                const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                                const T *__restrict__ vdia, const T *__restrict__ x, int *err,
                                                unsigned long long timeout_ns, unsigned char *smem, Epi &&epi) {
  using C = TileCfgC<T>;
  constexpr size_t B9 = 9 * sizeof(T);  // bytes of one 3x3 block
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  uint64_t *empty = full + C::kStages;
  unsigned char *ring = smem + C::kBarBytes;
  const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  if (threadIdx.x == 0) {
    for (unsigned s = 0; s < C::kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], C::kConsumers);
    }
    mbar_fence_init();
  }
  __syncthreads();
  const unsigned G = gridDim.x;
  if (warp == C::kConsumers) {
    // producer: values, block columns, diagonal blocks and row offsets of a tile
    if (lane != 0) return;
    unsigned k = 0;
    for (unsigned t = blockIdx.x; t < ntiles; t += G, ++k) {
      const unsigned s = k % C::kStages;
      if (k >= C::kStages && !mbar_wait_bounded(&empty[s], ((k / C::kStages) - 1) & 1u, timeout_ns)) {
        atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
        break;
      }
      const unsigned r0 = tiles[t], r1 = tiles[t + 1];
      const unsigned b0 = row_start[r0], b1 = row_start[r1];
      unsigned char *st = ring + (size_t)s * C::kStageBytes;
      size_t av, ac, ad, ar;
      unsigned lv, lc, ld, lr;
      round16((size_t)b0 * B9, (size_t)b1 * B9, av, lv);
      round16((size_t)b0 * 4, (size_t)b1 * 4, ac, lc);
      round16((size_t)r0 * B9, (size_t)r1 * B9, ad, ld);
      round16((size_t)r0 * 4, (size_t)(r1 + 1) * 4, ar, lr);
      mbar_arrive_expect_tx(&full[s], lv + lc + ld + lr);
      if (lv) tma_load_1d(st, reinterpret_cast<const unsigned char *>(vcrs) + av, lv, &full[s]);
      if (lc) tma_load_1d(st + C::kValBytes, reinterpret_cast<const unsigned char *>(col) + ac, lc, &full[s]);
      tma_load_1d(st + C::kValBytes + C::kColBytes, reinterpret_cast<const unsigned char *>(vdia) + ad, ld,
                  &full[s]);
      tma_load_1d(st + C::kValBytes + C::kColBytes + C::kDiaBytes,
                  reinterpret_cast<const unsigned char *>(row_start) + ar, lr, &full[s]);
    }
    const unsigned first = k > C::kStages ? k - C::kStages : 0u;
    for (unsigned j = first; j < k; ++j) mbar_wait_bounded(&full[j % C::kStages], (j / C::kStages) & 1u, timeout_ns);
    return;
  }
  const unsigned q = lane / 3u, a = lane - 3u * q;
  unsigned k = 0;
  for (unsigned t = blockIdx.x; t < ntiles; t += G, ++k) {
    const unsigned s = k % C::kStages;
    if (!mbar_wait_bounded(&full[s], (k / C::kStages) & 1u, timeout_ns)) {
      atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
      break;
    }
    const unsigned r0 = tiles[t], r1 = tiles[t + 1];
    const unsigned char *st = ring + (size_t)s * C::kStageBytes;
    const unsigned *rsv = reinterpret_cast<const unsigned *>(st + C::kValBytes + C::kColBytes + C::kDiaBytes +
                                                             (((size_t)r0 * 4) & 15));
    const unsigned b0 = rsv[0];
    const T *vv = reinterpret_cast<const T *>(st + (((size_t)b0 * B9) & 15));
    const unsigned *cv = reinterpret_cast<const unsigned *>(st + C::kValBytes + (((size_t)b0 * 4) & 15));
    const T *dv = reinterpret_cast<const T *>(st + C::kValBytes + C::kColBytes + (((size_t)r0 * B9) & 15));
    const unsigned i = r0 + warp * 10u + q;
    if (lane < 30 && i < r1) {
      const unsigned s0 = rsv[i - r0] - b0, s1 = rsv[i - r0 + 1] - b0;
      T acc0 = T(0), acc1 = T(0);
      unsigned u = s0;
      for (; u + 1 < s1; u += 2) {  // two blocks per step: both x gathers in flight
        const unsigned j0 = cv[u], j1 = cv[u + 1];
        const T *v0 = vv + (size_t)u * 9 + a * 3, *v1 = v0 + 9;
        const T *x0 = x + (size_t)j0 * 3, *x1 = x + (size_t)j1 * 3;
        acc0 += v0[0] * __ldg(x0) + v0[1] * __ldg(x0 + 1) + v0[2] * __ldg(x0 + 2);
        acc1 += v1[0] * __ldg(x1) + v1[1] * __ldg(x1 + 1) + v1[2] * __ldg(x1 + 2);
      }
      if (u < s1) {
        const T *v0 = vv + (size_t)u * 9 + a * 3, *x0 = x + (size_t)cv[u] * 3;
        acc0 += v0[0] * __ldg(x0) + v0[1] * __ldg(x0 + 1) + v0[2] * __ldg(x0 + 2);
      }
      const T *d = dv + (size_t)(i - r0) * 9 + a * 3, *xi = x + (size_t)i * 3;
      acc1 += d[0] * __ldg(xi) + d[1] * __ldg(xi + 1) + d[2] * __ldg(xi + 2);
      epi(i, a, acc0 + acc1);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

}  // namespace dfm2g

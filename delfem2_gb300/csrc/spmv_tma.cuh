// TMA-staged 3x3 block SpMV: warp-specialised, persistent.
//
// The block rows are cut into tiles of consecutive rows (at most kBlocks
// off-diagonal blocks and kRows rows each; tile table built on the host from
// the pattern). A persistent grid takes tiles round-robin. In each CTA one
// producer warp streams a tile's off-diagonal values, block columns and
// diagonal blocks - three contiguous byte ranges, rounded out to 16 bytes - into
// a kStages-deep shared-memory ring with cp.async.bulk, completing on a "full"
// mbarrier per stage; the consumer warps compute the tile's rows from shared
// memory in the lane layout of rowkern.cuh (x gathered from global memory,
// read-only) and release the stage on an "empty" mbarrier. Every wait is
// bounded; on a timeout the kernel records DFM2G_ERR_WAIT_TIMEOUT and the
// producer still waits (bounded) for its copies in flight before exiting.
#pragma once

#include "rowkern.cuh"
#include "tma.cuh"

namespace dfm2g {

template <typename T>
struct TileCfg {
  static constexpr unsigned kBlocks = sizeof(T) == 8 ? 384u : 768u;  // ~27 KiB of values per tile
  static constexpr unsigned kRows = 64;
  static constexpr unsigned kStages = 3;
  static constexpr unsigned kValBytes = kBlocks * 9 * sizeof(T) + 32;
  static constexpr unsigned kColBytes = kBlocks * 4 + 32;
  static constexpr unsigned kDiaBytes = kRows * 9 * sizeof(T) + 32;
  static constexpr unsigned kStageBytes = kValBytes + kColBytes + kDiaBytes;
  static constexpr unsigned kBarBytes = 128;
  static constexpr size_t kSmem = kBarBytes + (size_t)kStages * kStageBytes;
  static_assert(kValBytes % 16 == 0 && kColBytes % 16 == 0 && kDiaBytes % 16 == 0, "16-byte stage layout");
};

constexpr unsigned kTmaThreads = 512;                  // 15 consumer warps + 1 producer warp
constexpr unsigned kTmaConsumers = kTmaThreads / 32 - 1;

// Byte range [off, end) rounded out to 16 bytes: (aligned start, length).
__device__ __forceinline__ void round16(size_t off, size_t end, size_t &a, unsigned &len) {
  a = off & ~size_t(15);
  len = (unsigned)(((end + 15) & ~size_t(15)) - a);
}

template <typename T>
struct TileView {
  const T *v;         // v[(s - b0) * 9 + e]: off-diagonal block s of the tile
  const unsigned *c;  // c[s - b0]: its block column
  const T *d;         // d[(i - r0) * 9 + e]: diagonal block of row i
  unsigned r0, r1, b0;
};

template <typename T>
__device__ __forceinline__ TileView<T> tile_view(const unsigned char *stage, unsigned r0, unsigned r1, unsigned b0) {
  using C = TileCfg<T>;
  TileView<T> t;
  t.r0 = r0;
  t.r1 = r1;
  t.b0 = b0;
  const size_t ov = (size_t)b0 * 9 * sizeof(T), oc = (size_t)b0 * 4, od = (size_t)r0 * 9 * sizeof(T);
  t.v = reinterpret_cast<const T *>(stage + (ov & 15));
  t.c = reinterpret_cast<const unsigned *>(stage + C::kValBytes + (oc & 15));
  t.d = reinterpret_cast<const T *>(stage + C::kValBytes + C::kColBytes + (od & 15));
  return t;
}

// Row sums (K x)_i of one row from a staged tile: R rounds of 3 blocks in
// registers (off-diagonal blocks, then the diagonal); longer rows loop.
template <typename T, unsigned R>
struct TileRow {
  T v[R];
  unsigned j[R];
  unsigned nb, s0, s1;
};

template <typename T, unsigned R>
__device__ __forceinline__ void tile_row_load(TileRow<T, R> &f, const TileView<T> &tv, const RowLane &L, unsigned i,
                                              const unsigned *__restrict__ row_start) {
  f.s0 = row_start[i] - tv.b0;
  f.s1 = row_start[i + 1] - tv.b0;
  const unsigned noff = f.s1 - f.s0;
  f.nb = noff + 1;
#pragma unroll
  for (unsigned k = 0; k < R; ++k) {
    const unsigned t = 3u * k + L.g;
    f.v[k] = T(0);
    f.j[k] = 0u;
    if (L.active && t < f.nb) {
      if (t < noff) {
        f.j[k] = tv.c[f.s0 + t];
        f.v[k] = tv.v[(size_t)(f.s0 + t) * 9 + L.e];
      } else {
        f.j[k] = i;
        f.v[k] = tv.d[(size_t)(i - tv.r0) * 9 + L.e];
      }
    }
  }
}

template <typename T, unsigned R>
__device__ __forceinline__ T tile_row_dot(const TileRow<T, R> &f, const TileView<T> &tv, const RowLane &L,
                                          unsigned i, const T *__restrict__ x) {
  T acc = T(0);
  if (f.nb <= 3 * R) {
    T xv[R];
#pragma unroll
    for (unsigned k = 0; k < R; ++k)
      xv[k] = (L.active && 3u * k + L.g < f.nb) ? __ldg(x + (size_t)f.j[k] * 3 + L.c) : T(0);
#pragma unroll
    for (unsigned k = 0; k < R; ++k) acc += f.v[k] * xv[k];
  } else if (L.active) {
    const unsigned noff = f.s1 - f.s0;
    for (unsigned t = L.g; t < f.nb; t += 3u) {
      unsigned j;
      T v;
      if (t < noff) {
        j = tv.c[f.s0 + t];
        v = tv.v[(size_t)(f.s0 + t) * 9 + L.e];
      } else {
        j = i;
        v = tv.d[(size_t)(i - tv.r0) * 9 + L.e];
      }
      acc += v * __ldg(x + (size_t)j * 3 + L.c);
    }
  }
  return acc;
}

// Runs the pipeline over all tiles; epi(row, s[3]) is called by every lane of
// the consumer warp that owns the row (s on every lane). Must be called by all
// kTmaThreads threads of the CTA; `smem` is the dynamic shared memory
// (TileCfg<T>::kSmem bytes, 128-byte aligned).
template <typename T, typename Epi>
__device__ __forceinline__ void spmv_tma_rows(const unsigned *__restrict__ tiles, unsigned ntiles,
                                              const unsigned *__restrict__ row_start,
                                              const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                              const T *__restrict__ vdia, const T *__restrict__ x, int *err,
                                              unsigned long long timeout_ns, unsigned char *smem, Epi &&epi) {
  using C = TileCfg<T>;
  constexpr unsigned R = 5;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  uint64_t *empty = full + C::kStages;
  unsigned char *ring = smem + C::kBarBytes;
  const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  if (threadIdx.x == 0) {
    for (unsigned s = 0; s < C::kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kTmaConsumers);
    }
    mbar_fence_init();
  }
  __syncthreads();
  const unsigned G = gridDim.x;
  if (warp == kTmaConsumers) {
    // producer
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
      size_t av, ac, ad;
      unsigned lv, lc, ld;
      round16((size_t)b0 * 9 * sizeof(T), (size_t)b1 * 9 * sizeof(T), av, lv);
      round16((size_t)b0 * 4, (size_t)b1 * 4, ac, lc);
      round16((size_t)r0 * 9 * sizeof(T), (size_t)r1 * 9 * sizeof(T), ad, ld);
      mbar_arrive_expect_tx(&full[s], lv + lc + ld);
      if (lv) tma_load_1d(st, reinterpret_cast<const unsigned char *>(vcrs) + av, lv, &full[s]);
      if (lc) tma_load_1d(st + C::kValBytes, reinterpret_cast<const unsigned char *>(col) + ac, lc, &full[s]);
      tma_load_1d(st + C::kValBytes + C::kColBytes, reinterpret_cast<const unsigned char *>(vdia) + ad, ld,
                  &full[s]);
    }
    // let the copies in flight land before the CTA exits (bounded)
    const unsigned first = k > C::kStages ? k - C::kStages : 0u;
    for (unsigned j = first; j < k; ++j) mbar_wait_bounded(&full[j % C::kStages], (j / C::kStages) & 1u, timeout_ns);
    return;
  }
  const RowLane L(lane);
  unsigned k = 0;
  for (unsigned t = blockIdx.x; t < ntiles; t += G, ++k) {
    const unsigned s = k % C::kStages;
    if (!mbar_wait_bounded(&full[s], (k / C::kStages) & 1u, timeout_ns)) {
      atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
      break;
    }
    const unsigned r0 = tiles[t], r1 = tiles[t + 1];
    const TileView<T> tv = tile_view<T>(ring + (size_t)s * C::kStageBytes, r0, r1, row_start[r0]);
    // two rows per pass: both rows' x gathers are in flight together
    for (unsigned i = r0 + warp; i < r1; i += 2 * kTmaConsumers) {
      const unsigned i2 = i + kTmaConsumers;
      TileRow<T, R> fa, fb;
      tile_row_load(fa, tv, L, i, row_start);
      if (i2 < r1) tile_row_load(fb, tv, L, i2, row_start);
      const T acc_a = tile_row_dot(fa, tv, L, i, x);
      const T acc_b = i2 < r1 ? tile_row_dot(fb, tv, L, i2, x) : T(0);
      T sa[3], sb[3];
      row_reduce(acc_a, sa);
      row_reduce(acc_b, sb);
      epi(i, sa);
      if (i2 < r1) epi(i2, sb);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

// ---------------------------------------------------------------------------
// Component layout (FP32): lane 3q + a of a consumer warp computes component a
// of row q of the warp's ten rows, summing K_b[a][0..2] x_b over the row's
// blocks with no cross-lane reduction. A warp instruction then serves ten rows
// (the lane layout above: one row per 27 lanes plus a 7-shuffle reduction), so
// the kernel issues a fraction of the instructions per row. Tiles hold up to
// 150 rows (15 consumer warps x 10 rows) and are double-buffered; the tile's
// row offsets are staged with its values, block columns and diagonal blocks.
struct TileCfgC {
  static constexpr unsigned kRows = 150;  // kTmaConsumers x 10
  static constexpr unsigned kBlocks = 2304;
  static constexpr unsigned kStages = 2;
  static constexpr unsigned kValBytes = kBlocks * 9 * 4 + 32;
  static constexpr unsigned kColBytes = kBlocks * 4 + 32;
  static constexpr unsigned kDiaBytes = (kRows * 9 * 4 + 32 + 15) / 16 * 16;
  static constexpr unsigned kRsBytes = ((kRows + 1) * 4 + 32 + 15) / 16 * 16;
  static constexpr unsigned kStageBytes = kValBytes + kColBytes + kDiaBytes + kRsBytes;
  static constexpr unsigned kBarBytes = 128;
  static constexpr size_t kSmem = kBarBytes + (size_t)kStages * kStageBytes;
  static_assert(kRows == kTmaConsumers * 10, "ten rows per consumer warp");
  static_assert(kValBytes % 16 == 0 && kColBytes % 16 == 0 && kDiaBytes % 16 == 0 && kRsBytes % 16 == 0,
                "16-byte stage layout");
  static_assert(kSmem <= 227u * 1024u, "fits one CTA's shared memory");
};

// Runs the pipeline over all tiles; epi(row, a, v) is called by the lane that
// computed component a of `row` (v = (K x)_{3 row + a}). Must be called by all
// kTmaThreads threads of the CTA; `smem` holds TileCfgC::kSmem bytes.
template <typename Epi>
__device__ __forceinline__ void spmv_tma_rows_c(const unsigned *__restrict__ tiles, unsigned ntiles,
                                                const unsigned *__restrict__ row_start,
                                                const unsigned *__restrict__ col, const float *__restrict__ vcrs,
                                                const float *__restrict__ vdia, const float *__restrict__ x,
                                                int *err, unsigned long long timeout_ns, unsigned char *smem,
                                                Epi &&epi) {
  using C = TileCfgC;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  uint64_t *empty = full + C::kStages;
  unsigned char *ring = smem + C::kBarBytes;
  const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  if (threadIdx.x == 0) {
    for (unsigned s = 0; s < C::kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kTmaConsumers);
    }
    mbar_fence_init();
  }
  __syncthreads();
  const unsigned G = gridDim.x;
  if (warp == kTmaConsumers) {
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
      round16((size_t)b0 * 36, (size_t)b1 * 36, av, lv);
      round16((size_t)b0 * 4, (size_t)b1 * 4, ac, lc);
      round16((size_t)r0 * 36, (size_t)r1 * 36, ad, ld);
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
    const float *vv = reinterpret_cast<const float *>(st + (((size_t)b0 * 36) & 15));
    const unsigned *cv = reinterpret_cast<const unsigned *>(st + C::kValBytes + (((size_t)b0 * 4) & 15));
    const float *dv = reinterpret_cast<const float *>(st + C::kValBytes + C::kColBytes + (((size_t)r0 * 36) & 15));
    const unsigned i = r0 + warp * 10u + q;
    if (lane < 30 && i < r1) {
      const unsigned s0 = rsv[i - r0] - b0, s1 = rsv[i - r0 + 1] - b0;
      float acc0 = 0.f, acc1 = 0.f;
      unsigned u = s0;
      for (; u + 1 < s1; u += 2) {  // two blocks per step: both x gathers in flight
        const unsigned j0 = cv[u], j1 = cv[u + 1];
        const float *v0 = vv + (size_t)u * 9 + a * 3, *v1 = v0 + 9;
        const float *x0 = x + (size_t)j0 * 3, *x1 = x + (size_t)j1 * 3;
        acc0 += v0[0] * __ldg(x0) + v0[1] * __ldg(x0 + 1) + v0[2] * __ldg(x0 + 2);
        acc1 += v1[0] * __ldg(x1) + v1[1] * __ldg(x1 + 1) + v1[2] * __ldg(x1 + 2);
      }
      if (u < s1) {
        const float *v0 = vv + (size_t)u * 9 + a * 3, *x0 = x + (size_t)cv[u] * 3;
        acc0 += v0[0] * __ldg(x0) + v0[1] * __ldg(x0 + 1) + v0[2] * __ldg(x0 + 2);
      }
      const float *d = dv + (size_t)(i - r0) * 9 + a * 3, *xi = x + (size_t)i * 3;
      acc1 += d[0] * __ldg(xi) + d[1] * __ldg(xi + 1) + d[2] * __ldg(xi + 2);
      epi(i, a, acc0 + acc1);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

}  // namespace dfm2g

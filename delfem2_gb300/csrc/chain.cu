// Chain-scheduled sync-free triangular sweep (DFM2G_SWEEP_CHAINS), 1x1, 2x2 and 3x3 blocks.
//
// A chain is a run of consecutive rows i, i+1, ..., i+k (descending in the
// backward sweep) in which every row depends on the one before it: the last
// block of row i+1's lower triangle sits in column i (backward: the first
// block of row i-1's upper triangle in column i). One warp sweeps a whole
// chain, so that dependency is handed over in registers; only the other
// ("cross") dependencies are polled in global memory, as in the sync-free
// schedule. On a structured mesh in its natural ordering the chains are the
// grid lines along the fastest index: 65-row pencils along z on a
// 128x128x64 voxel mesh (nodes numbered z fastest), where a dependency path
// then changes warp on 256 of its 320 steps instead of all of them.
//
// Chains are numbered in the (level, row) order of their first rows. A row
// joins its predecessor's chain only if each of its cross dependencies lies in
// a chain numbered no higher than that chain, so every dependency of a chain's
// row lies in a lower-numbered chain or earlier in the same chain. Warps take
// chains in increasing number (their first one by warp index, later ones from
// an atomic counter, each taken shortly before the warp's current chain ends
// so that chains go to warps in the order the warps become free) and walk
// each chain in order; all CTAs are co-resident (cooperative launch). So the
// lowest-numbered unfinished chain has a warp, and the dependencies of its
// next row are all finished: the sweep cannot deadlock. Every wait is bounded
// (DFM2G_ERR_WAIT_TIMEOUT).
//
// Each direction and value type is stored once as fixed-size row records in
// chain order, rewritten from the factors after each decomposition:
//   [16 B: number of cross blocks nc, 0, 0, 0][m u32 cross columns, to 16 B]
//   [m x B*B cross values][B*B: block on the chain predecessor, zero on a
//   chain's first row][B*B: D^-1, forward only], padded to 16 B,
// m being the longest cross list of the pattern (FP64 3x3 records keep the
// predecessor's block right after the nc cross blocks instead). Lane 0 of
// each warp streams its chains' records into a ring of kChSlots shared-memory
// slots with cp.async.bulk, kChGroup rows per copy and mbarrier, up to
// kChSlots rows ahead of the row being finished; the polls of a row's cross
// values and the loads of its right-hand side are issued kChLook rows ahead.
// The step from one row of a chain to the next is then the row's reduction
// and the chain step in registers.
//
// Measured on GB300 (128x128x64 voxels x 6 tets, 1,081,665 block rows, 321
// levels per direction), forward / backward ms: FP32 0.58 / 0.56 and FP64
// 1.23 / 1.04, against 0.91 / 0.90 and 2.19 / 1.76 for the sync-free
// schedule. One chain alone (a block-tridiagonal matrix, one warp) advances
// 0.61 us per row in FP32 and 0.93 us in FP64; the sync-free schedule takes
// 1.21 / 2.93 us per row there (one row per level).
#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "rowkern.cuh"
#include "tma.cuh"  // smem_u32, mbarrier helpers

namespace dfm2g {

namespace {

constexpr unsigned kChThreads = 128;
constexpr unsigned kChWarps = kChThreads / 32;
constexpr unsigned kChLook = 3;       // rows whose polls are issued ahead
constexpr unsigned kChBarBytes = 64;  // per-warp copy-group barriers (up to 8)
constexpr unsigned kChGrabLead = 8;   // rows before a chain's end at which the next chain is taken
constexpr size_t kChSmemCap = 227u * 1024u;  // shared memory one CTA may opt in to

// Record ring of one warp: 16 slots in copy groups of 4 rows, or, for the
// kernels of long records (3x3 rows with more than 9 cross blocks), 12 slots
// in groups of 2 so that those still fit two CTAs per SM and keep at least
// 7 rows of records ahead. Per-warp header: the copy-group barriers, then one
// {row, chain start} per slot, 128-byte aligned; then the slots.
template <int B, unsigned R>
struct ChainRing {
  static constexpr bool kLong = B == 3 && R >= 4;
  static constexpr unsigned kSlots = kLong ? 12u : 16u;
  static constexpr unsigned kGroup = kLong ? 2u : 4u;
  static constexpr unsigned kGroups = kSlots / kGroup;
  static constexpr unsigned kHead = (kChBarBytes + 8 * kSlots + 127) / 128 * 128;
  static_assert(kSlots % kGroup == 0, "whole copy groups");
  static_assert(kGroups * 8 <= kChBarBytes, "copy-group barriers fit their header part");
};

inline unsigned pad16u(unsigned x) { return (x + 15u) & ~15u; }

struct ChainGeom {
  unsigned m, vo, rec;  // cross blocks per record, offset of the values, record bytes
};

inline ChainGeom chain_geom(unsigned m, unsigned vs, bool fwd, unsigned B) {
  ChainGeom g;
  g.m = m;
  g.vo = 16u + pad16u(4u * m);
  g.rec = pad16u(g.vo + (m + (fwd ? 2u : 1u)) * B * B * vs);
  return g;
}

inline size_t chain_smem(unsigned rec, unsigned slots, unsigned head) {
  return (size_t)kChWarps * (head + (size_t)slots * rec);
}

template <typename T, unsigned NV>
struct ChainStage {
  T xv[NV];  // the lane's cross values: 3x3, one per round (lane layout of
             // rowkern.cuh); 1x1 and 2x2, the components of the lane's block
  T in[3];   // the row's right-hand side (B values), on every lane
};

// Records of the rows: header, cross columns and values (rec_of[i] = record
// index of row i, linked[i] = 1 when row i continues its predecessor's chain).
template <typename T, bool FWD, int B>
__global__ void k_chain_fill(unsigned n, const unsigned *__restrict__ rs, const unsigned *__restrict__ col,
                             const unsigned *__restrict__ dia, const T *__restrict__ vcrs,
                             const T *__restrict__ vdia, const unsigned *__restrict__ rec_of,
                             const unsigned char *__restrict__ linked, unsigned char *__restrict__ bytes,
                             unsigned rec, unsigned m, unsigned vo) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned nw = (gridDim.x * blockDim.x) >> 5;
  for (unsigned i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nw) {
    const unsigned s0 = FWD ? rs[i] : dia[i], s1 = FWD ? dia[i] : rs[i + 1];
    const unsigned lk = linked[i];
    const unsigned nc = (s1 - s0) - lk;
    const unsigned c0 = FWD ? s0 : s0 + lk;  // first cross block
    unsigned char *rp = bytes + (size_t)rec_of[i] * rec;
    if (lane < 4) reinterpret_cast<unsigned *>(rp)[lane] = lane == 0 ? nc : 0u;
    unsigned *cols = reinterpret_cast<unsigned *>(rp + 16);
    for (unsigned t = lane; t < nc; t += 32) cols[t] = col[c0 + t];
    T *vals = reinterpret_cast<T *>(rp + vo);
    constexpr unsigned BB = B * B;
    for (unsigned e = lane; e < nc * BB; e += 32) vals[e] = vcrs[(size_t)c0 * BB + e];
    const unsigned lb = FWD ? s1 - 1u : s0;  // the block on the chain predecessor
    // FP64 3x3 records keep it right after the cross blocks (the sweep sums it
    // with them); the others in slot m
    const unsigned lslot = (sizeof(T) == 8 && B == 3) ? nc : m;
    if (lane < BB) {
      vals[(size_t)lslot * BB + lane] = lk ? vcrs[(size_t)lb * BB + lane] : T(0);
      if (FWD) vals[(size_t)(m + 1) * BB + lane] = vdia[(size_t)i * BB + lane];
    }
  }
}

// chains[c] = {first row, rows, record index of the first row, 0};
// ctr[0] hands out chain numbers beyond the grid's warps, ctr[1] counts the
// warps that are done (the last one resets both for the next launch).
// B = 3 uses the lane layout of rowkern.cuh (R rounds of three blocks);
// B = 1, 2 give each lane one cross block (32 per pass; R unused).
template <typename T, bool FWD, int B, unsigned R>
__global__ void __launch_bounds__(kChThreads) k_sweep_chain(unsigned nchain, const uint4 *__restrict__ chains,
                                                            const unsigned char *__restrict__ bytes, unsigned rec,
                                                            unsigned m, unsigned vo, const T *in, T *out,
                                                            unsigned *ctr, int *err, unsigned long long timeout_ns,
                                                            const int *skip) {
  extern __shared__ __align__(128) unsigned char ch_smem[];
  if (skip && *skip) return;
  const unsigned lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  const unsigned nwarp = gridDim.x * kChWarps;
  const unsigned w = blockIdx.x * kChWarps + wib;
  using Ring = ChainRing<B, R>;
  constexpr unsigned kChSlots = Ring::kSlots, kChGroup = Ring::kGroup, kChGroups = Ring::kGroups,
                     kChHead = Ring::kHead;
  unsigned char *wb = ch_smem + (size_t)wib * (kChHead + (size_t)kChSlots * rec);
  uint64_t *bar = reinterpret_cast<uint64_t *>(wb);
  uint2 *smeta = reinterpret_cast<uint2 *>(wb + kChBarBytes);  // {row, 1 if first row of its chain}
  unsigned char *slots = wb + kChHead;
  if (w < nchain) {
    if (lane == 0) {
      for (unsigned g = 0; g < kChGroups; ++g) mbar_init(&bar[g], 1);
      mbar_fence_init();
    }
    __syncwarp();
    const RowLane L(lane);
    bool abort = false;

    // ---- producer: lane 0 copies the records of this warp's rows, in order,
    // into the slot ring (cp.async.bulk), kChGroup slots per copy group and
    // mbarrier (a group's rows from one chain are one contiguous copy)
    // The next chain is taken from the counter only kChGrabLead rows before
    // the producer reaches the end of the current one (its number is read
    // kChGrabLead / 2 rows later), so chains go to warps in the order the
    // warps become free: a chain taken early could wait behind a long one.
    unsigned pc = w, pt = 0, issued = 0, grabbed = 0, nc = nchain, next_state = 0;  // 0 none, 1 taken, 2 read
    uint4 pd = chains[pc], nd = make_uint4(0u, 0u, 0u, 0u);
    // advances the cursor by one row (taking the next chain when it ends)
    auto advance = [&]() {
      ++issued;
      ++pt;
      if (next_state == 0 && pt + kChGrabLead >= pd.y) {
        if (lane == 0) grabbed = atomicAdd(ctr, 1u);
        next_state = 1;
      }
      if (next_state == 1 && pt + kChGrabLead / 2 >= pd.y) {
        nc = nwarp + __shfl_sync(0xffffffffu, grabbed, 0);
        nd = nc < nchain ? chains[nc] : make_uint4(0u, 0u, 0u, 0u);
        next_state = 2;
      }
      if (pt == pd.y) {
        pc = nc;
        pd = nd;
        pt = 0;
        next_state = 0;
      }
    };
    // fills the next copy group with up to kChGroup rows
    auto produce = [&]() {
      if (pc >= nchain) return;
      const unsigned s0 = issued % kChSlots, g = s0 / kChGroup;
      unsigned ri[kChGroup];  // record index of each row of the group (~0u: none)
      unsigned total = 0;
#pragma unroll
      for (unsigned q = 0; q < kChGroup; ++q) {
        ri[q] = ~0u;
        if (pc < nchain) {
          ri[q] = pd.z + pt;
          if (lane == 0) smeta[s0 + q] = make_uint2(FWD ? pd.x + pt : pd.x - pt, pt == 0 ? 1u : 0u);
          ++total;
          advance();
        }
      }
      if (lane == 0) {
        // relaxed: a release here would wait for this warp's polls in flight
        mbar_arrive_expect_tx_relaxed(&bar[g], total * rec);
        // one copy per run of consecutive records (rows of one chain)
#pragma unroll
        for (unsigned q = 0; q < kChGroup; ++q) {
          if (ri[q] != ~0u && (q == 0 || ri[q] != ri[q - 1] + 1)) {
            unsigned len = 1;
            bool run = true;
#pragma unroll
            for (unsigned q2 = q + 1; q2 < kChGroup; ++q2) {
              run = run && ri[q2] != ~0u && ri[q2] == ri[q2 - 1] + 1;
              if (run) ++len;
            }
            tma_load_1d(slots + (size_t)(s0 + q) * rec, bytes + (size_t)ri[q] * rec, len * rec, &bar[g]);
          }
        }
      }
    };

    // ---- issue the loads of row u (its record must have landed)
    constexpr unsigned NV = B == 3 ? R : (unsigned)B;
    auto poll = [&](unsigned u, ChainStage<T, NV> &S) {
      const unsigned s = u % kChSlots;
      if (!mbar_wait_bounded(&bar[s / kChGroup], (u / kChSlots) & 1u, timeout_ns)) {
        atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
        abort = true;
      }
      const unsigned char *rp = slots + (size_t)s * rec;
      const unsigned ncr = *reinterpret_cast<const unsigned *>(rp);
      const unsigned *cols = reinterpret_cast<const unsigned *>(rp + 16);
      const unsigned row = smeta[s].x;
      if constexpr (B == 3) {
#pragma unroll
        for (unsigned k = 0; k < R; ++k) {
          const unsigned blk = 3u * k + L.g;
          S.xv[k] = T(0);
          if (L.active && blk < ncr) S.xv[k] = ld_relaxed(out + (size_t)cols[blk] * 3 + L.c);
        }
      } else {
#pragma unroll
        for (int c = 0; c < B; ++c) {
          S.xv[c] = T(0);
          if (lane < ncr) S.xv[c] = ld_relaxed(out + (size_t)cols[lane] * B + c);
        }
      }
#pragma unroll
      for (int c = 0; c < B; ++c) S.in[c] = in[(size_t)row * B + c];
    };

    // ---- finish row t: wait for its cross values, reduce, chain step, store
    T zp0 = T(0), zp1 = T(0), zp2 = T(0);
    // 1x1 and 2x2 blocks: each lane's block row sums, the warp sum, then the
    // chain step on every lane (zp0, zp1 hold the predecessor's values)
    auto finish_nd = [&](unsigned ncr, const unsigned *cols, const T *vals, uint2 sm, ChainStage<T, NV> &S) {
      constexpr unsigned BB = (unsigned)(B * B);
      T acc[2] = {T(0), T(0)};
      if (lane < ncr) {
        const T *a = vals + (size_t)lane * BB;
#pragma unroll
        for (int r = 0; r < B; ++r)
#pragma unroll
          for (int c = 0; c < B; ++c) acc[r] += a[r * B + c] * S.xv[c];
      }
      for (unsigned blk = 32u + lane; blk < ncr; blk += 32u) {  // more than 32 cross blocks: read inline
        const T *a = vals + (size_t)blk * BB;
#pragma unroll
        for (int c = 0; c < B; ++c) {
          const T x = abort ? T(0) : wait_value(out + (size_t)cols[blk] * B + c, err, timeout_ns);
#pragma unroll
          for (int r = 0; r < B; ++r) acc[r] += a[r * B + c] * x;
        }
      }
#pragma unroll
      for (int r = 0; r < B; ++r) acc[r] = warp_sum(acc[r]);
      if (sm.y) zp0 = zp1 = T(0);
      const T *lc = vals + (size_t)m * BB;
      T u[2];
      if constexpr (B == 1) {
        u[0] = S.in[0] - acc[0] - lc[0] * zp0;
        zp0 = FWD ? vals[(size_t)(m + 1)] * u[0] : u[0];
      } else {
        u[0] = S.in[0] - acc[0] - (lc[0] * zp0 + lc[1] * zp1);
        u[1] = S.in[1] - acc[1] - (lc[2] * zp0 + lc[3] * zp1);
        if (FWD) {
          const T *d = vals + (size_t)(m + 1) * BB;
          zp0 = d[0] * u[0] + d[1] * u[1];
          zp1 = d[2] * u[0] + d[3] * u[1];
        } else {
          zp0 = u[0];
          zp1 = u[1];
        }
      }
      if (lane < (unsigned)B) st_relaxed(out + (size_t)sm.x * B + lane, lane == 0 ? zp0 : zp1);
    };
    auto finish = [&](unsigned t, ChainStage<T, NV> &S) {
      const unsigned s = t % kChSlots;
      const unsigned char *rp = slots + (size_t)s * rec;
      const unsigned ncr = *reinterpret_cast<const unsigned *>(rp);
      const unsigned *cols = reinterpret_cast<const unsigned *>(rp + 16);
      const T *vals = reinterpret_cast<const T *>(rp + vo);
      const uint2 sm = smeta[s];
      // address of the lane's cross value k (pending ones are re-read)
      auto xaddr = [&](unsigned k) -> const T * {
        if constexpr (B == 3)
          return out + (size_t)cols[3u * k + L.g] * 3 + L.c;
        else
          return out + (size_t)cols[lane] * B + k;
      };
      bool pend = false;
#pragma unroll
      for (unsigned k = 0; k < NV; ++k) pend |= is_pending(S.xv[k]);
      if (pend && !abort) {
        const unsigned long long t0 = globaltimer_ns();
        unsigned spins = 0;
        for (;;) {
#pragma unroll
          for (unsigned k = 0; k < NV; ++k)
            if (is_pending(S.xv[k])) S.xv[k] = ld_relaxed(xaddr(k));
          pend = false;
#pragma unroll
          for (unsigned k = 0; k < NV; ++k) pend |= is_pending(S.xv[k]);
          if (!pend) break;
          if ((++spins & 15u) == 0 && (ld_relaxed(err) != 0 || globaltimer_ns() - t0 > timeout_ns)) {
            atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
            abort = true;
            break;
          }
        }
      }
      if (abort) {
#pragma unroll
        for (unsigned k = 0; k < NV; ++k)
          if (is_pending(S.xv[k])) S.xv[k] = T(0);
      }
      if constexpr (B < 3) {
        finish_nd(ncr, cols, vals, sm, S);
        return;
      }
      if constexpr (sizeof(T) == 8) {
        // FP64: the block on the chain predecessor (record slot ncr, x = zp)
        // and -in join the row's reduction, and D^-1 is applied to the
        // reduced sums on lanes 0..2: s = L x + Lc zp - in, z = -D^-1 s
        // (forward) or -s (backward). Fewer FP64 instructions per row than
        // a separate chain step (GB300's FP64 pipe is narrow).
        if (sm.y) zp0 = zp1 = zp2 = T(0);
        const T zpa[3] = {zp0, zp1, zp2};
        T acc = (L.g == 0 && L.c == 0) ? -pick3(S.in, L.r) : T(0);
#pragma unroll
        for (unsigned k = 0; k < R; ++k) {
          const unsigned blk = 3u * k + L.g;
          if (L.active && blk <= ncr)
            acc += vals[(size_t)blk * 9 + L.e] * (blk < ncr ? S.xv[k] : pick3(zpa, L.c));
        }
        if (ncr + 1u > 3u * R && L.active) {  // longer than the registers: read inline
          for (unsigned blk = 3u * R + L.g; blk <= ncr; blk += 3u) {
            const T x = blk == ncr ? pick3(zpa, L.c)
                                   : (abort ? T(0) : wait_value(out + (size_t)cols[blk] * 3 + L.c, err, timeout_ns));
            acc += vals[(size_t)blk * 9 + L.e] * x;
          }
        }
        T s3[3];
        row_reduce(acc, s3);
        const unsigned a = lane < 3 ? lane : 2u;
        T za;
        if (FWD) {
          const T *d = vals + (size_t)(m + 1) * 9 + a * 3;
          za = -(d[0] * s3[0] + d[1] * s3[1] + d[2] * s3[2]);
        } else {
          za = -pick3(s3, a);
        }
        if (lane < 3) st_relaxed(out + (size_t)sm.x * 3 + lane, za);
        zp0 = __shfl_sync(0xffffffffu, za, 0);
        zp1 = __shfl_sync(0xffffffffu, za, 1);
        zp2 = __shfl_sync(0xffffffffu, za, 2);
        return;
      }
      T acc = T(0);
#pragma unroll
      for (unsigned k = 0; k < R; ++k) {
        const unsigned blk = 3u * k + L.g;
        if (L.active && blk < ncr) acc += vals[(size_t)blk * 9 + L.e] * S.xv[k];
      }
      if (ncr > 3u * R && L.active) {  // cross lists longer than the registers: read inline
        for (unsigned blk = 3u * R + L.g; blk < ncr; blk += 3u) {
          const T x = abort ? T(0) : wait_value(out + (size_t)cols[blk] * 3 + L.c, err, timeout_ns);
          acc += vals[(size_t)blk * 9 + L.e] * x;
        }
      }
      T s3[3];
      row_reduce(acc, s3);
      if (sm.y) zp0 = zp1 = zp2 = T(0);
      const T *lc = vals + (size_t)m * 9;
      {
        // FP32: every lane computes all three components (no shuffle on the
        // row-to-row path)
        const T u0 = S.in[0] - s3[0] - (lc[0] * zp0 + lc[1] * zp1 + lc[2] * zp2);
        const T u1 = S.in[1] - s3[1] - (lc[3] * zp0 + lc[4] * zp1 + lc[5] * zp2);
        const T u2 = S.in[2] - s3[2] - (lc[6] * zp0 + lc[7] * zp1 + lc[8] * zp2);
        if (FWD) {
          const T *d = vals + (size_t)(m + 1) * 9;
          zp0 = d[0] * u0 + d[1] * u1 + d[2] * u2;
          zp1 = d[3] * u0 + d[4] * u1 + d[5] * u2;
          zp2 = d[6] * u0 + d[7] * u1 + d[8] * u2;
        } else {
          zp0 = u0;
          zp1 = u1;
          zp2 = u2;
        }
        if (lane < 3) st_relaxed(out + (size_t)sm.x * 3 + lane, lane == 0 ? zp0 : (lane == 1 ? zp1 : zp2));
      }
    };

    for (unsigned j = 0; j < kChGroups; ++j) produce();
    // kChLook + 1 stages used in rotation: the loop is unrolled by that count
    // so every stage is a fixed set of registers. (Copying a register whose
    // load is still in flight waits for the load, which would put a round
    // trip to L2 back on every row.)
    constexpr unsigned NST = kChLook + 1;
    ChainStage<T, NV> st[NST];
#pragma unroll
    for (unsigned k = 0; k < NST; ++k) {
#pragma unroll
      for (unsigned q = 0; q < NV; ++q) st[k].xv[q] = T(0);
      st[k].in[0] = st[k].in[1] = st[k].in[2] = T(0);
      if (k < kChLook && k < issued) poll(k, st[k]);
    }
    for (unsigned t0 = 0; t0 < issued; t0 += NST) {
#pragma unroll
      for (unsigned u = 0; u < NST; ++u) {
        const unsigned t = t0 + u;
        if (t < issued) {
          if (t + kChLook < issued) poll(t + kChLook, st[(u + kChLook) % NST]);
          finish(t, st[u]);
          if ((t + 1) % kChGroup == 0) {  // its copy group is consumed
            __syncwarp();                  // every lane is done with the group before the next copy overwrites it
            produce();
          }
        }
      }
    }
  }
  if (lane == 0) {
    __threadfence();
    const unsigned done = atomicAdd(ctr + 1, 1u);
    if (done == nwarp - 1) {
      atomicExch(ctr, 0u);
      atomicExch(ctr + 1, 0u);
    }
  }
}

template <typename V>
int chain_to_host(std::vector<V> &h, const V *d, size_t n) {
  h.resize(n);
  if (n) DFM2G_CUDA(cudaMemcpy(h.data(), d, n * sizeof(V), cudaMemcpyDeviceToHost));
  return DFM2G_OK;
}

// Chains of one direction (host, from the sorted pattern and the level order).
// The chain partition of one direction (host only). Rows are visited in the
// sweep's (level, row) order; a row joins its predecessor's chain when its
// triangle's block nearest the diagonal is on that predecessor and every other
// block's row lies in a chain numbered no higher. m = the longest cross list.
void chain_partition(unsigned n, const unsigned *rs, const unsigned *col, const unsigned *dia,
                     const unsigned *order, bool fwd, std::vector<unsigned> &chain_of, std::vector<unsigned> &first,
                     std::vector<unsigned> &len, std::vector<unsigned char> &linked, unsigned &m) {
  chain_of.assign(n, 0u);
  linked.assign(n, 0);
  first.clear();
  len.clear();
  m = 0;
  for (unsigned q = 0; q < n; ++q) {
    const unsigned i = order[q];
    const unsigned s0 = fwd ? rs[i] : dia[i], s1 = fwd ? dia[i] : rs[i + 1];
    bool link = false;
    unsigned c = 0;
    if (s1 > s0) {
      const unsigned lb = fwd ? s1 - 1 : s0;
      const bool has_prev = fwd ? i > 0 : i + 1 < n;
      if (has_prev && col[lb] == (fwd ? i - 1 : i + 1)) {
        c = chain_of[col[lb]];
        link = true;
        for (unsigned s = s0; s < s1 && link; ++s)
          if (s != lb && chain_of[col[s]] > c) link = false;
      }
    }
    if (link) {
      chain_of[i] = c;
      ++len[c];
      linked[i] = 1;
    } else {
      chain_of[i] = (unsigned)first.size();
      first.push_back(i);
      len.push_back(1);
    }
    m = std::max(m, (s1 - s0) - (link ? 1u : 0u));
  }
}

int chain_build(dfm2g_ilu_s *p, bool fwd, ChainSched &cs) {
  cs.ok = false;
  const unsigned n = p->nblk;
  std::vector<unsigned> rs, col, dia, order;
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  DFM2G_TRY(chain_to_host(rs, p->row_start.p, (size_t)n + 1));
  DFM2G_TRY(chain_to_host(col, p->col.p, p->nnz));
  DFM2G_TRY(chain_to_host(dia, p->dia_ind.p, n));
  DFM2G_TRY(chain_to_host(order, fwd ? p->order_f.p : p->order_b.p, n));
  std::vector<unsigned> chain_of, first, len;
  std::vector<unsigned char> linked;
  unsigned m = 0;
  chain_partition(n, rs.data(), col.data(), dia.data(), order.data(), fwd, chain_of, first, len, linked, m);
  const unsigned nchain = (unsigned)first.size();
  std::vector<uint4> chains(nchain);
  std::vector<unsigned> rec_of(n);
  unsigned base = 0;
  for (unsigned c = 0; c < nchain; ++c) {
    chains[c] = make_uint4(first[c], len[c], base, 0u);
    base += len[c];
  }
  for (unsigned i = 0; i < n; ++i) {
    const unsigned c = chain_of[i];
    rec_of[i] = chains[c].z + (fwd ? i - first[c] : first[c] - i);
  }
  cs.nchain = nchain;
  cs.m = m;
  DFM2G_TRY(cs.chains.resize((size_t)nchain + 1));
  DFM2G_TRY(cs.rec_of.resize((size_t)n + 1));
  DFM2G_TRY(cs.linked.resize((size_t)n + 1));
  DFM2G_TRY(cs.ctr.resize(2));
  DFM2G_CUDA(cudaMemcpy(cs.chains.p, chains.data(), sizeof(uint4) * nchain, cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(cs.rec_of.p, rec_of.data(), sizeof(unsigned) * n, cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(cs.linked.p, linked.data(), n, cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemset(cs.ctr.p, 0, 2 * sizeof(unsigned)));
  cs.ok = true;
  return DFM2G_OK;
}

// Register rounds of the 3x3 kernel for cross lists of up to m blocks (FP64
// also sums the chain predecessor's block with them); 1 for 1x1 and 2x2.
inline unsigned chain_rounds(unsigned m, unsigned B, bool f64) {
  if (B != 3) return 1;
  const unsigned need = f64 ? m + 1 : m;
  if (need <= 6) return 2;
  if (need <= 9 && f64) return 3;
  if (need <= 12) return 4;
  return 8;
}

// Ring slots and per-warp header bytes of the kernel for (B, R).
inline void chain_ring(unsigned B, unsigned R, unsigned &slots, unsigned &head) {
  if (B == 3 && R >= 4) {
    slots = ChainRing<3, 4>::kSlots;
    head = ChainRing<3, 4>::kHead;
  } else {
    slots = ChainRing<3, 2>::kSlots;
    head = ChainRing<3, 2>::kHead;
  }
}

template <typename T, bool FWD>
void *chain_kernel(unsigned R, unsigned B) {
  if (B == 1) return (void *)k_sweep_chain<T, FWD, 1, 1>;
  if (B == 2) return (void *)k_sweep_chain<T, FWD, 2, 1>;
  if (R == 2) return (void *)k_sweep_chain<T, FWD, 3, 2>;
  if (R == 3) return (void *)k_sweep_chain<T, FWD, 3, 3>;
  if (R == 4) return (void *)k_sweep_chain<T, FWD, 3, 4>;
  return (void *)k_sweep_chain<T, FWD, 3, 8>;
}

template <typename T, bool FWD>
void chain_fill_launch(unsigned B, unsigned blocks, dfm2g_ilu_s *p, const T *vcrs, const T *vdia,
                       const ChainSched &cs, unsigned char *bytes, const ChainGeom &g) {
  const unsigned n = p->nblk;
  if (B == 1)
    k_chain_fill<T, FWD, 1><<<blocks, 256, 0, stream()>>>(n, p->row_start.p, p->col.p, p->dia_ind.p, vcrs, vdia,
                                                          cs.rec_of.p, cs.linked.p, bytes, g.rec, g.m, g.vo);
  else if (B == 2)
    k_chain_fill<T, FWD, 2><<<blocks, 256, 0, stream()>>>(n, p->row_start.p, p->col.p, p->dia_ind.p, vcrs, vdia,
                                                          cs.rec_of.p, cs.linked.p, bytes, g.rec, g.m, g.vo);
  else
    k_chain_fill<T, FWD, 3><<<blocks, 256, 0, stream()>>>(n, p->row_start.p, p->col.p, p->dia_ind.p, vcrs, vdia,
                                                          cs.rec_of.p, cs.linked.p, bytes, g.rec, g.m, g.vo);
}

// Lets `kernel` launch with `smem` bytes of dynamic shared memory. The
// attribute belongs to the kernel, not to a pattern, so it only ever grows
// (per kernel and device): a handle with shorter records must not lower the
// limit another handle's launches rely on.
int chain_allow_smem(void *kernel, size_t smem) {
  struct Entry {
    void *kernel;
    int device;
    size_t smem;
  };
  static std::mutex mu;
  static std::vector<Entry> done;
  std::lock_guard<std::mutex> lock(mu);
  const int dev = ctx().device;
  for (auto &d : done) {
    if (d.kernel != kernel || d.device != dev) continue;
    if (d.smem >= smem) return DFM2G_OK;
    DFM2G_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    d.smem = smem;
    return DFM2G_OK;
  }
  DFM2G_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  done.push_back(Entry{kernel, dev, smem});
  return DFM2G_OK;
}

DevBuf<unsigned char> &chain_bytes(ChainSched &cs, double) { return cs.bytes64; }
DevBuf<unsigned char> &chain_bytes(ChainSched &cs, float) { return cs.bytes32; }

}  // namespace

// Builds the chains of one direction (first use), rewrites the records of the
// value type after each decomposition, and launches the sweep; false in
// *usable when the pattern's records do not fit the shared-memory ring, or
// when !may_alloc and the chains or records do not exist yet.
template <typename T>
int chain_sweep(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia, const int *skip,
                unsigned long long timeout, bool may_alloc, bool *usable) {
  ChainSched &cs = forward ? p->cs_f : p->cs_b;
  *usable = false;
  if (!may_alloc && (!cs.built || !cs.ok || !chain_bytes(cs, T(0)).p)) return DFM2G_OK;
  if (!cs.built) {
    cs.built = true;
    DFM2G_TRY(chain_build(p, forward, cs));
  }
  if (!cs.ok) return DFM2G_OK;
  const bool f64 = sizeof(T) == 8;
  const unsigned B = p->ndim;
  const ChainGeom g = chain_geom(cs.m, (unsigned)sizeof(T), forward, B);
  const unsigned R = chain_rounds(cs.m, B, f64);
  unsigned slots = 0, head = 0;
  chain_ring(B, R, slots, head);
  const size_t smem = chain_smem(g.rec, slots, head);
  if (smem > kChSmemCap) return DFM2G_OK;  // records too long for the rings
  const unsigned n = p->nblk;
  DevBuf<unsigned char> &bytes = chain_bytes(cs, T(0));
  unsigned &ver = f64 ? cs.ver64 : cs.ver32;
  if (!bytes.p) {
    DFM2G_TRY(bytes.resize((size_t)n * g.rec + 16));
    ver = ~0u;
  }
  if (ver != p->factor_version) {
    const unsigned blocks = blocks_for((size_t)n * 32, 256, ctx().num_sms * 16);
    if (forward)
      chain_fill_launch<T, true>(B, blocks, p, vcrs, vdia, cs, bytes.p, g);
    else
      chain_fill_launch<T, false>(B, blocks, p, vcrs, vdia, cs, bytes.p, g);
    DFM2G_LAUNCH_CHECK();
    note_launches(1);
    ver = p->factor_version;
  }
  void *kernel = forward ? chain_kernel<T, true>(R, B) : chain_kernel<T, false>(R, B);
  DFM2G_TRY(chain_allow_smem(kernel, smem));
  int &cap = cs.coop[f64 ? 1 : 0];
  if (cap <= 0) {
    int per_sm = 0;
    DFM2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kChThreads, smem));
    if (per_sm <= 0) return DFM2G_OK;
    cap = per_sm * ctx().num_sms;
  }
  const unsigned blocks = std::min<unsigned>((unsigned)cap, (cs.nchain + kChWarps - 1) / kChWarps);
  unsigned nchain = cs.nchain, rec = g.rec, m = g.m, vo = g.vo;
  const uint4 *chains = cs.chains.p;
  const unsigned char *bp = bytes.p;
  unsigned *ctr = cs.ctr.p;
  int *err = p->err.p;
  void *args[] = {(void *)&nchain, (void *)&chains, (void *)&bp, (void *)&rec, (void *)&m, (void *)&vo,
                  (void *)&in, (void *)&out, (void *)&ctr, (void *)&err, (void *)&timeout, (void *)&skip};
  DFM2G_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(blocks), dim3(kChThreads), args, smem, stream()));
  note_launches(1);
  *usable = true;
  return DFM2G_OK;
}

template int chain_sweep<float>(dfm2g_ilu_s *, bool, const float *, float *, const float *, const float *,
                                const int *, unsigned long long, bool, bool *);
template int chain_sweep<double>(dfm2g_ilu_s *, bool, const double *, double *, const double *, const double *,
                                 const int *, unsigned long long, bool, bool *);

// Drops the chains and records (a new pattern); rebuilt on first use.
void chain_schedules_reset(dfm2g_ilu_s *p) {
  for (ChainSched *cs : {&p->cs_f, &p->cs_b}) {
    cs->built = cs->ok = false;
    cs->nchain = cs->m = 0;
    cs->ver32 = cs->ver64 = ~0u;
    cs->coop[0] = cs->coop[1] = 0;
    cs->chains.release();
    cs->rec_of.release();
    cs->linked.release();
    cs->bytes32.release();
    cs->bytes64.release();
    cs->ctr.release();
  }
}

}  // namespace dfm2g

using namespace dfm2g;

extern "C" {

// Host-only: the chain partition the chain schedule uses, from a sorted ILU
// pattern (row offsets, columns, diagonal positions) and the sweep's level
// order. No device work.
int dfm2g_chain_partition(unsigned n, const unsigned *row_start, const unsigned *col, const unsigned *dia_ind,
                          const unsigned *order, int backward, unsigned *chain_of, unsigned *nchain,
                          unsigned *max_cross) try {
  if (n && (!row_start || !col || !dia_ind || !order || !chain_of))
    return fail(DFM2G_ERR_ARG, "chain_partition: null array");
  std::vector<unsigned> co, first, len;
  std::vector<unsigned char> linked;
  unsigned m = 0;
  chain_partition(n, row_start, col, dia_ind, order, backward == 0, co, first, len, linked, m);
  if (n) std::copy(co.begin(), co.end(), chain_of);
  if (nchain) *nchain = (unsigned)first.size();
  if (max_cross) *max_cross = m;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

}  // extern "C"

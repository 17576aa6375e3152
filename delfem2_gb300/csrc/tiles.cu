// Tile-scheduled triangular sweep (DFM2G_SWEEP_TILES), 3x3 blocks, FP32 and FP64.
//
// The rows of one sweep direction are partitioned into tiles: bundles of up
// to 49 segments of dependency chains (strands), grown from a seed row, a row
// joining the tile only once every row it depends on is in an earlier tile or
// already in this one. Seeds are taken in the sweep's (level, row) order, so
// the tiles are numbered in a dependency order that follows the wavefront.
// Inside a tile the rows are grouped by their local level (1 + the highest
// local level of the rows of the same tile they depend on): the tile's steps,
// at most one row per segment each. On a structured mesh in its natural order
// the tiles are columns of the grid (7 x 7 z lines on the voxel meshes, whose
// dependencies all point to lower neighbours: whole lines of up to 65 rows for
// FP32 sweeps, 33-row segments for FP64, whose tiles hold at most 1,617 rows):
// steps of up to 49 rows, and a dependency path crosses a tile boundary once
// per tile instead of once per row or pencil of rows.
//
// One CTA sweeps one tile at a time, step by step: ten rows per consumer
// warp and step, three lanes per row (lane 3q + c of row q): lane c reads
// component c of each dependency's x and sums column c of the blocks into the
// three row components, the three lanes' sums are exchanged by shuffles, and
// lane c keeps row component c. Nothing on a step's path reads global memory:
//  - values of rows of the same tile come from a shared-memory copy of the
//    tile's results (visible after the consumers' barrier of the step that
//    wrote them);
//  - values of rows of other tiles (the step's halo, listed per step) are
//    copied from global memory into the step's slot ahead of the step
//    (cp.async through L2, completing on the slot's halo mbarrier); a copy
//    still holding the pending marker (the sync-free schedules' NaN) is read
//    again in global memory a step ahead, and polled there when the step runs;
//  - the right-hand side is copied into the step's slot with the halo values
//    (4- or 8-byte cp.async per row component, in the records' row order:
//    group-major, 32 values per group of ten rows).
// A producer warp streams each step's records and halo list into a ring of
// shared-memory slots (cp.async.bulk, one mbarrier per slot), issues each
// step's halo and right-hand-side copies `lead` steps before the consumers
// reach it (late enough that the halo values are usually written), takes the
// CTA's next tile from a counter a few steps before the current one ends (so
// tiles go to CTAs in the order CTAs become free) and then prefetches that
// tile's records into L2.
//
// Progress: tiles are handed out in increasing number (the first by CTA
// index, later ones from the counter), every CTA is resident (cooperative
// launch), and every dependency of a tile's row lies in a lower-numbered tile
// or in an earlier step of the same tile. The lowest-numbered unfinished tile
// is the current tile of some CTA (a CTA's next tile is numbered above its
// current one), and all its outside dependencies are finished, so the sweep
// cannot deadlock. Every wait is bounded (DFM2G_ERR_WAIT_TIMEOUT); a CTA that
// stops early first waits (bounded) for the copies it issued.
//
// Record layout of one group of ten rows (G = 10 rows, M = dependency slots
// of the pattern, Mc = M rounded up to 4, S = value bytes, NV = 3M (+3 for
// D^-1 in the forward sweep) values per lane):
//   [0, 48)   u32 row id of each of the ten rows (~0u: none), padding
//   [48, ..)  u32 code[G][Mc]: 0x80000000 | local index (a row of the same
//             tile, or tile_rows for an unused slot); 0x40000000 | row (a row
//             of another tile read in global memory: beyond the step's first
//             kTiHalo, or so close to the end of the vector that its 32-byte
//             copy would pass it); else a halo entry: bits 0-7 its index in
//             the step's halo list, bits 8-9 / bit 10 the offset (in 4 / 8
//             bytes) of the row's FP32 / FP64 values inside their copy
//   [vo, ..)  the lanes' values in 16-byte chunks, chunk k of lane l at
//             vo + (30 k + l) 16: lane 3q + c holds (forward) row c of D^-1,
//             then column c of each block, L_b[0..2][c] for b < M
// A step's groups are consecutive in the stream, so one copy moves a step.
#include <algorithm>
#include <atomic>
#include <functional>
#include <mutex>
#include <queue>
#include <thread>
#include <vector>

#include "common.cuh"
#include "tma.cuh"

namespace dfm2g {

namespace {

// rows per tile at most: FP32 49 segments of 65 rows (7 x 7 whole z lines on
// the voxel grids up to 64 cells high), FP64 49 of 33 (its shared-memory copy
// of the tile's results is twice as wide and would leave too few ring slots)
#ifndef DFM2G_TILE_ROWS_F32
#define DFM2G_TILE_ROWS_F32 3185
#endif
#ifndef DFM2G_TILE_ROWS_F64
#define DFM2G_TILE_ROWS_F64 1617
#endif
#ifndef DFM2G_TILE_WARPS
#define DFM2G_TILE_WARPS 5  // consumer warps per CTA (ten rows each per step)
#endif
constexpr unsigned kTiWarps = DFM2G_TILE_WARPS;
constexpr unsigned kTiG = 10;                   // rows per group (30 lanes)
constexpr unsigned kTiWidth = kTiG * kTiWarps;  // rows per step at most
// segments per tile (so rows per step) the partition takes: 49 = 7 x 7 z lines,
// a full square of them on the voxel grids, where a 50th would stick out
#ifndef DFM2G_TILE_SEGS
#define DFM2G_TILE_SEGS (kTiWidth - 1)
#endif
constexpr unsigned kTiSegs = DFM2G_TILE_SEGS;
static_assert(kTiSegs >= 1 && kTiSegs <= kTiWidth, "segments per tile");
constexpr unsigned kTiThreads = 32 * (kTiWarps + 1);
constexpr unsigned kTiCons = 32 * kTiWarps;     // consumer threads
constexpr unsigned kTiHead = 48;
constexpr unsigned kTiLocal = 0x80000000u;
constexpr unsigned kTiGlobal = 0x40000000u;     // code: a row read in global memory (low 30 bits)
constexpr unsigned kTiEnd = 0xFFFFFFFFu;
constexpr unsigned kTiMaxSlots = 12;
constexpr unsigned kTiHalo = 128;               // halo rows copied per step (32 B each; index in 8 bits)
#ifndef DFM2G_TILE_HALO_LEAD
#define DFM2G_TILE_HALO_LEAD 4  // steps between a step's halo copies and its use, where the ring allows
#endif
constexpr unsigned kTiHaloLead = DFM2G_TILE_HALO_LEAD;
constexpr unsigned kTiMinLead = 2;  // consumers wait for step s + 1's halo before step s's barrier
constexpr double kTiAutoRows = 20.0;            // DFM2G_SWEEP_AUTO: least rows per step for tiles
constexpr unsigned kTiAutoDeps = 8;             // DFM2G_SWEEP_AUTO: most dependency blocks per row for tiles
constexpr unsigned kTiGrabLead = 4;             // steps before a tile's end at which the next tile is taken
constexpr size_t kTiSmemCap = 227u * 1024u;
static_assert(kTiWarps >= 1 && kTiWarps <= 15, "named barrier of the consumer warps");
static_assert(kTiHalo <= 256, "halo index in 8 bits");
static_assert(kTiHaloLead >= kTiMinLead, "halo lead");

__host__ __device__ inline unsigned pad16u(unsigned x) { return (x + 15u) & ~15u; }
// rows per tile at most for values of S bytes; also the local index of the
// all-zero row that unused dependency slots point to
__host__ __device__ constexpr unsigned tile_rows(unsigned S) {
  return S == 8u ? DFM2G_TILE_ROWS_F64 : DFM2G_TILE_ROWS_F32;
}
__host__ __device__ inline unsigned round4u(unsigned x) { return (x + 3u) & ~3u; }

struct TileGeom {
  unsigned M, Mc, nv, nch, vo, gbytes;
};

inline TileGeom tile_geom(unsigned M, unsigned S, bool fwd) {
  TileGeom g;
  g.M = M;
  g.Mc = round4u(M);
  g.nv = 3u * M + (fwd ? 3u : 0u);
  g.nch = (g.nv * S + 15u) / 16u;
  g.vo = kTiHead + 4u * kTiG * g.Mc;
  g.gbytes = g.vo + g.nch * 30u * 16u;
  return g;
}

}  // namespace

// Slot layout: records (max_groups groups), right-hand side (32 values per
// group), halo list (kTiHalo u32), halo values (kTiHalo x 32 bytes).
struct SlotGeom {
  unsigned in_off, hl_off, hd_off, bytes;
};

namespace {

inline SlotGeom slot_geom(unsigned max_groups, unsigned gbytes, unsigned S) {
  SlotGeom s;
  s.in_off = max_groups * gbytes;
  s.hl_off = s.in_off + max_groups * 32u * S;
  s.hd_off = s.hl_off + kTiHalo * 4u;
  s.bytes = s.hd_off + kTiHalo * 32u;
  return s;
}

// Shared memory of the sweep kernel: barriers [0, 288), slot descriptors
// [512, 896), stop flags [960, 968), the tile's results (tile_rows + 1 rows),
// the slot ring.
__host__ __device__ inline size_t tile_xs_off() { return 1024; }
__host__ __device__ inline size_t tile_ring_off(unsigned S) {
  return tile_xs_off() + pad16u((tile_rows(S) + 1u) * 3u * S);
}
inline size_t tile_smem(unsigned S, unsigned slots, unsigned slot_bytes) {
  return tile_ring_off(S) + (size_t)slots * slot_bytes;
}

// The records of one value type: group headers and codes from `gmeta`
// (10 + 10 Mc u32 per group), values from the factors.
template <typename T, bool FWD>
__global__ void k_tile_fill(unsigned n, size_t ngroups, const unsigned *__restrict__ rs,
                            const unsigned *__restrict__ dia, const T *__restrict__ vcrs,
                            const T *__restrict__ vdia, const unsigned *__restrict__ rec_of,
                            const unsigned *__restrict__ gmeta, unsigned M, unsigned Mc, unsigned vo,
                            unsigned gbytes, unsigned char *__restrict__ bytes) {
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nth = (size_t)gridDim.x * blockDim.x;
  const size_t words = (size_t)kTiG * (Mc + 1u);
  for (size_t e = tid; e < ngroups * words; e += nth) {
    const size_t g = e / words, k = e - g * words;
    unsigned *gp = reinterpret_cast<unsigned *>(bytes + g * gbytes);
    const unsigned w = gmeta[e];
    if (k < kTiG)
      gp[k] = w;
    else
      gp[kTiHead / 4 + (k - kTiG)] = w;
  }
  const unsigned nv = 3u * M + (FWD ? 3u : 0u);
  const size_t per_row = 3u * (size_t)nv;
  for (size_t e = tid; e < (size_t)n * per_row; e += nth) {
    const unsigned i = (unsigned)(e / per_row);
    const unsigned r = (unsigned)(e - (size_t)i * per_row);
    const unsigned a = r / nv, j = r - a * nv;
    const unsigned s0 = FWD ? rs[i] : dia[i], s1 = FWD ? dia[i] : rs[i + 1];
    T v;
    if (FWD && j < 3u) {
      v = vdia[(size_t)i * 9 + a * 3 + j];  // row a of D^-1
    } else {
      const unsigned jb = FWD ? j - 3u : j;
      const unsigned b = jb / 3u, r2 = jb - 3u * b;
      v = (s0 + b < s1) ? vcrs[(size_t)(s0 + b) * 9 + r2 * 3 + a] : T(0);  // column a of block b
    }
    const unsigned rec = rec_of[i];
    const size_t g = rec / kTiG;
    const unsigned q = rec - (unsigned)g * kTiG;
    const unsigned lane = 3u * q + a;
    const unsigned byte = j * (unsigned)sizeof(T);
    *reinterpret_cast<T *>(bytes + g * gbytes + vo + ((byte >> 4) * 30u + lane) * 16u + (byte & 15u)) = v;
  }
}

__device__ __forceinline__ void bar_consumers() {
  asm volatile("bar.sync 1, %0;" ::"r"(kTiCons) : "memory");
}

// tiles[2t] = {first step, steps, first group, groups}, tiles[2t+1] = {first
// halo word, halo words, 0, 0}; steps[2s] = {first group, rows, local index of
// the step's first row, groups}, steps[2s+1] = {first halo word, halo rows, 0,
// 0} (halo words of a step padded to four). ctr[0] hands out tiles beyond the
// grid, ctr[1] counts finished CTAs (the last one resets both).
template <typename T, bool FWD, unsigned MR>
__global__ void __launch_bounds__(kTiThreads, 1)
    k_sweep_tiles(unsigned ntiles, const uint4 *__restrict__ tiles, const uint4 *__restrict__ steps,
                  const unsigned char *__restrict__ bytes, const T *__restrict__ in,
                  const unsigned *__restrict__ halo, unsigned M, unsigned vo, unsigned gbytes, unsigned nslots,
                  unsigned lead, SlotGeom sg, T *out, unsigned *ctr, int *err, unsigned long long timeout_ns,
                  const int *skip) {
  extern __shared__ __align__(128) unsigned char ti_smem[];
  if (skip && *skip) return;
  constexpr unsigned kZero = tile_rows((unsigned)sizeof(T));  // local index of the all-zero row
  uint64_t *full = reinterpret_cast<uint64_t *>(ti_smem);
  uint64_t *empty = full + kTiMaxSlots;
  uint64_t *hbar = empty + kTiMaxSlots;
  uint4 *smeta = reinterpret_cast<uint4 *>(ti_smem + 512);  // 2 per slot
  volatile int *sflag = reinterpret_cast<volatile int *>(ti_smem + 960);  // [2]
  T *xs = reinterpret_cast<T *>(ti_smem + tile_xs_off());
  unsigned char *ring = ti_smem + tile_ring_off((unsigned)sizeof(T));
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;

  if (threadIdx.x == 0) {
    for (unsigned k = 0; k < nslots; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], 1);
      mbar_init(&hbar[k], 32);  // one cp.async arrival per producer lane
    }
    sflag[0] = sflag[1] = 0;
    mbar_fence_init();
  }
  if (threadIdx.x < 3) xs[(size_t)kZero * 3 + threadIdx.x] = T(0);
  __syncthreads();

  if (warp == kTiWarps) {
    // ---- producer warp: walks the CTA's tiles and copies their steps (lane
    // 0 issues the bulk copies), and each step's halo values `lead` steps
    // before the consumers reach it (all lanes). Step descriptors come in
    // batches of 32, one per lane.
    auto shfl4 = [&](const uint4 &v, unsigned src) {
      return make_uint4(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
                        __shfl_sync(0xffffffffu, v.z, src), __shfl_sync(0xffffffffu, v.w, src));
    };
    auto load_batch = [&](const uint4 &t0, unsigned base, uint4 &sa, uint4 &sb) {
      sa = sb = make_uint4(0u, 0u, 0u, 0u);
      if (base + lane < t0.y) {
        sa = steps[2 * (t0.x + base + lane)];
        sb = steps[2 * (t0.x + base + lane) + 1];
      }
    };
    // halo values and right-hand side of step u into its slot; every lane
    // arrives on the slot's halo barrier once its copies are complete
    auto halo_copy = [&](unsigned u) {
      const unsigned su = u % nslots;
      if (mbar_wait_bounded(&full[su], (u / nslots) & 1u, timeout_ns)) {
        const uint4 m0 = smeta[2 * su], m1 = smeta[2 * su + 1];
        if (m0.w != kTiEnd) {
          const unsigned hc = min(m1.y, kTiHalo);
          unsigned char *sp = ring + (size_t)su * sg.bytes;
          // right-hand side: component a of row q of group g to lane 3q + a of the group's 32 values
          for (unsigned k = lane; k < m0.z * 30u; k += 32u) {
            const unsigned g = k / 30u, l = k - 30u * g, q = l / 3u, a = l - 3u * q;
            const unsigned row = reinterpret_cast<const unsigned *>(sp + (size_t)g * gbytes)[q];
            if (row != ~0u)
              cpa_small<sizeof(T)>(sp + sg.in_off + (size_t)(g * 32u + l) * sizeof(T), in + (size_t)row * 3 + a);
          }
          const unsigned *hl = reinterpret_cast<const unsigned *>(sp + sg.hl_off);
          for (unsigned k = lane; k < 2u * hc; k += 32u) {
            const unsigned h = k >> 1, hr = hl[h];
            const size_t byte = ((size_t)hr * 3u * sizeof(T)) & ~(size_t)15;
            cpa16_l2(sp + sg.hd_off + h * 32u + (k & 1u) * 16u,
                     reinterpret_cast<const unsigned char *>(out) + byte + (k & 1u) * 16u);
          }
        }
      } else if (lane == 0) {
        atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
      }
      cpa_arrive_noinc(&hbar[su]);
    };
    unsigned cur = blockIdx.x, cs = 0, base = 0, issued = 0, halo_next = 0;
    const unsigned halo_lag = nslots - lead;
    uint4 td = tiles[2 * cur], sa, sb;
    load_batch(td, 0, sa, sb);
    unsigned tok = 0;
    int grab = 0;  // 0: next tile not taken, 1: taken, 2: its descriptors loaded
    unsigned next = kTiEnd;
    uint4 ntd = make_uint4(0u, 0u, 0u, 0u), nsa, nsb;
    auto take_next = [&]() {
      if (lane == 0) tok = atomicAdd(ctr, 1u);
      grab = 1;
    };
    auto load_next = [&]() {
      next = gridDim.x + __shfl_sync(0xffffffffu, tok, 0);
      if (next < ntiles) {
        ntd = tiles[2 * next];
        load_batch(ntd, 0, nsa, nsb);
        if (lane == 0) {
          // the next tile's records and halo lists into L2
          const uint4 n1 = tiles[2 * next + 1];
          bulk_prefetch_l2(bytes + (size_t)ntd.z * gbytes, ntd.w * gbytes);
          if (n1.y) bulk_prefetch_l2(halo + n1.x, n1.y * 4u);
        }
      }
      grab = 2;
    };
    for (;;) {
      if (cs == td.y) {  // the current tile is issued: switch to the next one
        if (grab == 0) take_next();
        if (grab == 1) load_next();
        cur = next;
        cs = base = 0;
        grab = 0;
        if (cur < ntiles) {
          td = ntd;
          sa = nsa;
          sb = nsb;
        }
      }
      const unsigned slot = issued % nslots;
      int ok = 1;
      if (lane == 0 && issued >= nslots &&
          !mbar_wait_bounded(&empty[slot], ((issued / nslots) - 1u) & 1u, timeout_ns)) {
        atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
        ok = 0;
      }
      if (!__shfl_sync(0xffffffffu, ok, 0)) break;  // the consumers stop on their own bounded waits
      if (cur >= ntiles) {
        if (lane == 0) {
          smeta[2 * slot] = make_uint4(0u, 0u, 0u, kTiEnd);
          mbar_arrive(&full[slot]);
        }
        ++issued;
        break;
      }
      if (cs - base == 32u) {
        base += 32u;
        load_batch(td, base, sa, sb);
      }
      if (grab == 0 && cs + kTiGrabLead >= td.y)
        take_next();
      else if (grab == 1 && cs + kTiGrabLead / 2 >= td.y)
        load_next();
      const uint4 st = shfl4(sa, cs - base), sh = shfl4(sb, cs - base);
      if (lane == 0) {
        smeta[2 * slot] = make_uint4(st.y, st.z, st.w, cur);
        smeta[2 * slot + 1] = sh;
        unsigned char *sp = ring + (size_t)slot * sg.bytes;
        const unsigned nrec = st.w * gbytes;
        const unsigned nhl = round4u(sh.y) * 4u;
        mbar_arrive_expect_tx(&full[slot], nrec + nhl);
        tma_load_1d(sp, bytes + (size_t)st.x * gbytes, nrec, &full[slot]);
        if (nhl) tma_load_1d(sp + sg.hl_off, halo + sh.x, nhl, &full[slot]);
      }
      ++cs;
      ++issued;
      // step u's halo is copied when the producer issues step u + nslots -
      // lead, i.e. once the consumers are `lead` steps before u
      while (halo_next + halo_lag < issued) halo_copy(halo_next++);
    }
    // the halo copies of the steps issued last (the END slot needs none)
    const unsigned last = issued > 0 ? issued - 1u : 0u;
    while (halo_next < last) halo_copy(halo_next++);
    cpa_wait<0>();
    if (lane == 0) {
      // wait (bounded) for the bulk copies of the last slots before leaving
      const unsigned lo = issued > nslots ? issued - nslots : 0u;
      for (unsigned i = lo; i < issued; ++i) mbar_wait_bounded(&full[i % nslots], (i / nslots) & 1u, timeout_ns);
      __threadfence();
      const unsigned done = atomicAdd(ctr + 1, 1u);
      if (done == gridDim.x - 1u) {
        atomicExch(ctr, 0u);
        atomicExch(ctr + 1, 0u);
      }
    }
    return;
  }

  // ---- consumers. Software-pipelined over the steps: everything a step
  // reads that does not depend on the step before it (its slot's barriers and
  // descriptor, the lane's row, codes, values and right-hand side, and the x
  // values of halo rows) is loaded before the previous step's barrier; after
  // it, only the x values of the tile's own rows, the products, the three-lane
  // exchange and the store remain on the path from one step to the next.
  const unsigned q = lane / 3u, a = lane - 3u * q;
  const bool lane_ok = lane < 30u;
  const unsigned Mc = round4u(M);
  constexpr unsigned NVR = 3u * MR + 3u;
  constexpr unsigned PER = 16u / sizeof(T);
  const unsigned nv = FWD ? 3u * M + 3u : 3u * M;
  // the next step's data, loaded ahead
  struct Pre {
    bool ok, end, work;
    unsigned slot, row, local;
    unsigned cd[MR];
    T v[NVR];
    T xh[MR];  // halo x values (component a); the tile's own rows are read later
    T in;
  };
  auto preload = [&](Pre &P, unsigned u) {
    P.slot = u % nslots;
    const unsigned par = (u / nslots) & 1u;
    P.ok = mbar_wait_bounded(&full[P.slot], par, timeout_ns);
    const uint4 meta = smeta[2 * P.slot];  // {rows, local base, groups, tile}
    P.end = P.ok && meta.w == kTiEnd;
    if (P.ok && !P.end) P.ok = mbar_wait_bounded(&hbar[P.slot], par, timeout_ns);
    if (!P.ok) {
      atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
      sflag[u & 1u] = 1;
    }
    P.work = P.ok && !P.end && warp < meta.z;
    P.row = ~0u;
    if (!P.work) return;
    unsigned char *sp = ring + (size_t)P.slot * sg.bytes;
    const unsigned char *gp = sp + (size_t)warp * gbytes;
    P.row = lane_ok ? reinterpret_cast<const unsigned *>(gp)[q] : ~0u;
    P.local = meta.y + warp * kTiG + q;
    const unsigned char *vp = gp + vo + (lane_ok ? lane : 0u) * 16u;
#pragma unroll
    for (unsigned k = 0; k < (NVR + PER - 1) / PER; ++k) {
      if (k * PER < nv) {
        if constexpr (sizeof(T) == 4) {
          const float4 c = *reinterpret_cast<const float4 *>(vp + k * 480u);
          if (k * 4 + 0 < NVR) P.v[k * 4 + 0] = c.x;
          if (k * 4 + 1 < NVR) P.v[k * 4 + 1] = c.y;
          if (k * 4 + 2 < NVR) P.v[k * 4 + 2] = c.z;
          if (k * 4 + 3 < NVR) P.v[k * 4 + 3] = c.w;
        } else {
          const double2 c = *reinterpret_cast<const double2 *>(vp + k * 480u);
          if (k * 2 + 0 < NVR) P.v[k * 2 + 0] = c.x;
          if (k * 2 + 1 < NVR) P.v[k * 2 + 1] = c.y;
        }
      } else {
#pragma unroll
        for (unsigned e = 0; e < PER; ++e)
          if (k * PER + e < NVR) P.v[k * PER + e] = T(0);
      }
    }
    const uint4 *cw = reinterpret_cast<const uint4 *>(gp + kTiHead + (lane_ok ? q : 0u) * Mc * 4u);
#pragma unroll
    for (unsigned k = 0; k < MR / 4; ++k) {
      const uint4 c = (4u * k < Mc) ? cw[k]
                                    : make_uint4(kTiLocal | kZero, kTiLocal | kZero, kTiLocal | kZero,
                                                 kTiLocal | kZero);
      P.cd[4 * k + 0] = c.x;
      P.cd[4 * k + 1] = c.y;
      P.cd[4 * k + 2] = c.z;
      P.cd[4 * k + 3] = c.w;
    }
    // halo copies of this step. A copy still holding the pending marker was
    // taken before its row was written (the tile runs close behind the one it
    // depends on): the row is read again in global memory now, a step before
    // its use, as are rows without a copy, so the read's round trip overlaps
    // this step's barrier instead of delaying the next step.
    const unsigned char *hd = sp + sg.hd_off;
    const unsigned *hl = reinterpret_cast<const unsigned *>(sp + sg.hl_off);
#pragma unroll
    for (unsigned b = 0; b < MR; ++b) {
      const unsigned c = P.cd[b];
      const bool loc = (c & kTiLocal) != 0u, glob = !loc && (c & kTiGlobal) != 0u;
      const unsigned off = sizeof(T) == 4 ? ((c >> 8) & 3u) * 4u : ((c >> 10) & 1u) * 8u;
      const T *xp = (loc || glob) ? xs + (size_t)kZero * 3 : reinterpret_cast<const T *>(hd + (c & 0xFFu) * 32u + off);
      T x = xp[a];
      if (!loc && (glob || is_pending(x))) {
        const unsigned r = glob ? (c & ~kTiGlobal) : hl[c & 0xFFu];
        x = ld_relaxed(out + (size_t)r * 3 + a);
      }
      P.xh[b] = x;
    }
    P.in = reinterpret_cast<const T *>(sp + sg.in_off)[warp * 32u + lane];
  };

  // The next step's loads follow this step's products (issued before them
  // they measured slower: the step's shared-memory reads queue behind them).
  Pre P, Q;
  preload(P, 0);
  for (unsigned s = 0;; ++s) {
    const bool end = P.end;
    const unsigned slot = P.slot;
    // not past the CTA's last step, where the producer stops
    const bool more = !end && sflag[s & 1u] == 0;
    if (P.work) {
      // the tile's own rows: written by earlier steps, visible after their barriers
      T xv[MR];
#pragma unroll
      for (unsigned b = 0; b < MR; ++b) {
        const unsigned c = P.cd[b];
        // codes of other tiles' rows are no index into xs: the zero row is read instead
        const unsigned li = (c & kTiLocal) ? (c & ~kTiLocal) : kZero;
        const T x = xs[(size_t)li * 3 + a];
        xv[b] = (c & kTiLocal) ? x : P.xh[b];
      }
      const unsigned row = P.row;
      if (row != ~0u) {
        // values still pending (a halo copy taken too early, or a row read in
        // global memory): polled in global memory
        bool pend = false;
#pragma unroll
        for (unsigned b = 0; b < MR; ++b) pend |= is_pending(xv[b]);
        if (pend) {
          const unsigned *hl = reinterpret_cast<const unsigned *>(ring + (size_t)slot * sg.bytes + sg.hl_off);
          const unsigned long long t0 = globaltimer_ns();
          unsigned spins = 0;
          for (;;) {
            pend = false;
#pragma unroll
            for (unsigned b = 0; b < MR; ++b) {
              const unsigned c = P.cd[b];
              if ((c & kTiLocal) || !is_pending(xv[b])) continue;
              const unsigned r = (c & kTiGlobal) ? (c & ~kTiGlobal) : hl[c & 0xFFu];
              xv[b] = ld_relaxed(out + (size_t)r * 3 + a);
              pend |= is_pending(xv[b]);
            }
            if (!pend) break;
            if ((++spins & 15u) == 0 && (ld_relaxed(err) != 0 || globaltimer_ns() - t0 > timeout_ns)) {
              atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
#pragma unroll
              for (unsigned b = 0; b < MR; ++b)
                if (is_pending(xv[b])) xv[b] = T(0);
              break;
            }
          }
        }
      }
      // column a of each block against x_b[a], into the three row sums
      constexpr unsigned off = FWD ? 3u : 0u;
      T p0 = T(0), p1 = T(0), p2 = T(0);
#pragma unroll
      for (unsigned b = 0; b < MR; ++b) {
        if (b < M) {
          p0 += P.v[off + 3 * b + 0] * xv[b];
          p1 += P.v[off + 3 * b + 1] * xv[b];
          p2 += P.v[off + 3 * b + 2] * xv[b];
        }
      }
      // row a's sum over the three lanes of the row: in round r each lane
      // sends its sum for row (a + r) % 3 and receives row a's from lane (a - r) % 3
      const unsigned base = 3u * q;
      const unsigned a1 = a == 2u ? 0u : a + 1u, a2 = a == 0u ? 2u : a - 1u;  // a + 1, a - 1 (mod 3)
      const T own = a == 0u ? p0 : (a == 1u ? p1 : p2);
      const T s1 = a1 == 0u ? p0 : (a1 == 1u ? p1 : p2);  // row a + 1, sent in round 1
      const T s2 = a2 == 0u ? p0 : (a2 == 1u ? p1 : p2);  // row a + 2 = a - 1, sent in round 2
      const T r1 = __shfl_sync(0xffffffffu, s1, base + a2);  // from lane a - 1: its row (a - 1) + 1 = a
      const T r2 = __shfl_sync(0xffffffffu, s2, base + a1);  // from lane a + 1: its row (a + 1) - 1 = a
      const T acc = P.in - ((own + r1) + r2);
      T z;
      if constexpr (FWD) {
        // z_a = sum_c Dinv[a][c] u_c, u_c on lane 3q + c (every lane takes part)
        const T u0 = __shfl_sync(0xffffffffu, acc, base);
        const T u1 = __shfl_sync(0xffffffffu, acc, base + 1u);
        const T u2 = __shfl_sync(0xffffffffu, acc, base + 2u);
        z = P.v[0] * u0 + P.v[1] * u1 + P.v[2] * u2;
      } else {
        z = acc;
      }
      if (row != ~0u) {
        xs[(size_t)P.local * 3 + a] = z;
        st_relaxed(out + (size_t)row * 3 + a, z);
      }
    }
    if (more) preload(Q, s + 1);
    bar_consumers();
    if (sflag[s & 1u] != 0 || end) break;
    if (threadIdx.x == 0) mbar_arrive(&empty[slot]);
    P = Q;
  }
}

// ---- host: the tile partition -----------------------------------------------

template <typename V>
int tile_to_host(std::vector<V> &h, const V *d, size_t n) {
  h.resize(n);
  if (n) DFM2G_CUDA(cudaMemcpy(h.data(), d, n * sizeof(V), cudaMemcpyDeviceToHost));
  return DFM2G_OK;
}

}  // namespace

// The tile partition of one direction (host only). `order` is the sweep's
// (level, row) order.
//
// Strands first: a row continues the strand of the dependency nearest to it
// in row number when it is also that row's successor nearest to it (on a grid
// numbered z fastest: its z neighbour, so the strands are the grid's z lines);
// any other row starts a strand. Each strand is cut into segments of nearly equal
// length, at most max_rows / max_width rows. The rows of a segment depend on
// one another in a chain, so a segment has at most one row on each local
// level of a tile.
//
// Then the tiles: each grows from the first unassigned row of the level order
// (its seed: every row it depends on has a lower level, so it is assigned) by
// offers (layer, rank in the level order), smallest first. A row's successors
// are offered at the row's layer when they are in its segment, one layer
// further when they are in another strand, and after every other offer within
// reach when they start the next segment of its strand, so a tile takes the
// seed's segment, then the segments next to it at the same depth, and so on:
// on the voxel grids, columns of 7 x 7 z-line segments. A row joins once every
// row it depends on is assigned (to an earlier
// tile or this one), as long as the tile has fewer than max_rows rows, its
// segment is in the tile or the tile has fewer than max_width segments, and
// its local level has fewer than max_width rows. The tiles are numbered along
// the wavefront. Outputs per row: its tile and local level; m = the most
// dependencies of a row.
constexpr unsigned kTiSegFar = 1u << 20;  // layer step to the next segment of the same strand

void tile_partition(unsigned n, const unsigned *rs, const unsigned *dia, const unsigned *col, const unsigned *order,
                    bool fwd, unsigned max_rows, unsigned max_width, std::vector<unsigned> &tile_of,
                    std::vector<unsigned> &lev, unsigned &ntiles, unsigned &m) {
  const unsigned none = ~0u;
  tile_of.assign(n, none);
  lev.assign(n, 0u);
  m = 0;
  auto dep_range = [&](unsigned i, unsigned &s0, unsigned &s1) {
    s0 = fwd ? rs[i] : dia[i];
    s1 = fwd ? dia[i] : rs[i + 1];
  };
  std::vector<unsigned> pos(n);  // rank in the level order
  for (unsigned k = 0; k < n; ++k) pos[order[k]] = k;
  // successors: rows that depend on each row
  std::vector<unsigned> sptr(n + 1, 0u), succ;
  for (unsigned i = 0; i < n; ++i) {
    unsigned s0, s1;
    dep_range(i, s0, s1);
    m = std::max(m, s1 - s0);
    for (unsigned s = s0; s < s1; ++s) sptr[col[s] + 1]++;
  }
  for (unsigned i = 0; i < n; ++i) sptr[i + 1] += sptr[i];
  succ.resize(sptr[n]);
  {
    std::vector<unsigned> fill(sptr.begin(), sptr.end() - 1);
    for (unsigned i = 0; i < n; ++i) {
      unsigned s0, s1;
      dep_range(i, s0, s1);
      for (unsigned s = s0; s < s1; ++s) succ[fill[col[s]]++] = i;
    }
  }
  // strands: r continues the strand of d when d is the dependency of r
  // nearest to it in row number and r the successor of d nearest to d (ties:
  // the earlier in the level order), so a row cannot take another's strand
  std::vector<unsigned> next(n, none), prev(n, none), near_succ(n, none);
  auto nearer = [&](unsigned r, unsigned cand, unsigned cur) {  // cand nearer to r than cur
    if (cur == none) return true;
    const unsigned dc = cand > r ? cand - r : r - cand, du = cur > r ? cur - r : r - cur;
    return dc < du || (dc == du && pos[cand] < pos[cur]);
  };
  for (unsigned d = 0; d < n; ++d)
    for (unsigned k = sptr[d]; k < sptr[d + 1]; ++k)
      if (nearer(d, succ[k], near_succ[d])) near_succ[d] = succ[k];
  for (unsigned r = 0; r < n; ++r) {
    unsigned s0, s1;
    dep_range(r, s0, s1);
    unsigned best = none;
    for (unsigned s = s0; s < s1; ++s)
      if (nearer(r, col[s], best)) best = col[s];
    if (best != none && near_succ[best] == r) {
      next[best] = r;
      prev[r] = best;
    }
  }
  // segments: strands cut into ceil(len / seg_max) pieces of nearly equal length
  const unsigned seg_max = std::max(1u, max_rows / std::max(1u, max_width));
  std::vector<unsigned> seg_of(n, none);
  unsigned nseg_total = 0;
  for (unsigned r = 0; r < n; ++r) {
    if (prev[r] != none) continue;
    unsigned len = 0;
    for (unsigned u = r; u != none; u = next[u]) ++len;
    const unsigned pieces = (len + seg_max - 1u) / seg_max;
    unsigned k = 0;
    for (unsigned u = r; u != none; u = next[u], ++k) seg_of[u] = nseg_total + (unsigned)((uint64_t)k * pieces / len);
    nseg_total += pieces;
  }
  // offers (layer, rank), smallest first; layer_of[r]: the lowest layer r was offered at in this tile.
  // A row is offered once, when its last unassigned dependency joins the tile (unassigned[r] reaches 0).
  using Offer = std::pair<unsigned, unsigned>;
  std::priority_queue<Offer, std::vector<Offer>, std::greater<Offer>> heap;
  std::vector<unsigned> layer_of(n, none), offered;  // offered: rows whose layer_of is set in this tile
  std::vector<unsigned> width, seg_tile(nseg_total, none), unassigned(n);
  for (unsigned i = 0; i < n; ++i) {
    unsigned s0, s1;
    dep_range(i, s0, s1);
    unassigned[i] = s1 - s0;
  }
  unsigned cursor = 0, t = 0;
  for (;;) {
    while (cursor < n && tile_of[order[cursor]] != none) ++cursor;
    if (cursor >= n) break;
    const unsigned seed = order[cursor];
    for (unsigned r : offered) layer_of[r] = none;
    offered.clear();
    while (!heap.empty()) heap.pop();
    heap.push(Offer(0u, pos[seed]));
    layer_of[seed] = 0;
    offered.push_back(seed);
    width.assign(max_rows + 1u, 0u);
    unsigned count = 0, nseg = 0;
    while (!heap.empty() && count < max_rows) {
      const Offer o = heap.top();
      heap.pop();
      const unsigned r = order[o.second];
      if (tile_of[r] != none) continue;
      const bool new_seg = seg_tile[seg_of[r]] != t;
      if (new_seg && nseg >= max_width) continue;
      unsigned s0, s1;
      dep_range(r, s0, s1);
      unsigned lv = 0;  // every dependency is assigned (the row was offered when the last one joined)
      for (unsigned s = s0; s < s1; ++s) {
        const unsigned d = col[s];
        if (tile_of[d] == t) lv = std::max(lv, lev[d] + 1u);
      }
      if (width[lv] >= max_width) continue;  // left to a later tile
      tile_of[r] = t;
      lev[r] = lv;
      width[lv]++;
      ++count;
      if (new_seg) {
        seg_tile[seg_of[r]] = t;
        ++nseg;
      }
      for (unsigned k = sptr[r]; k < sptr[r + 1]; ++k) {
        const unsigned u = succ[k];
        // same segment: same layer; another strand: one layer further; the
        // strand's next segment: after every other segment in reach
        const unsigned lay = o.first + (seg_of[u] == seg_of[r] ? 0u : prev[u] == r ? kTiSegFar : 1u);
        if (layer_of[u] == none) offered.push_back(u);
        layer_of[u] = std::min(layer_of[u], lay);
        if (--unassigned[u] == 0) heap.push(Offer(layer_of[u], pos[u]));
      }
    }
    ++t;
  }
  ntiles = t;
}

namespace {

// Register rounds of the kernel: dependency slots rounded up to 4 (codes are
// loaded in fours), 8 or 16.
unsigned tile_rounds(unsigned m) { return round4u(m) <= 8 ? 8u : 16u; }

// The host part of a direction's tile schedule (no CUDA calls, so the two
// directions can be built at once on two host threads): partition, rows of
// each tile by local level, group records (row ids, codes), per-step halo
// lists, tile and step descriptors.
struct TileHost {
  bool ok = false;
  unsigned ntiles = 0, nsteps = 0, M = 0, max_groups = 0, max_halo = 0;
  size_t ngroups = 0;
  std::vector<uint4> tiles, steps;
  std::vector<unsigned> rec_of, gmeta, halo;
};

// Tiles of at most max_rows rows (unused dependency slots point to local row
// max_rows, the all-zero row).
void tile_host_build(unsigned n, const std::vector<unsigned> &rs, const std::vector<unsigned> &col,
                     const std::vector<unsigned> &dia, const std::vector<unsigned> &order, bool fwd,
                     unsigned max_rows, TileHost &out) {
  out.ok = false;
  std::vector<unsigned> tile_of, lev;
  unsigned ntiles = 0, m = 0;
  tile_partition(n, rs.data(), dia.data(), col.data(), order.data(), fwd, max_rows, kTiSegs, tile_of, lev, ntiles,
                 m);
  if (m > 16) return;  // rows too long for the register rounds
  const unsigned M = std::max(m, 1u);
  // rows of each tile by (local level, level order)
  std::vector<unsigned> tstart(ntiles + 1, 0u), trows(n);
  for (unsigned i = 0; i < n; ++i) tstart[tile_of[i] + 1]++;
  for (unsigned t = 0; t < ntiles; ++t) tstart[t + 1] += tstart[t];
  {
    std::vector<unsigned> fill(tstart.begin(), tstart.end() - 1);
    for (unsigned k = 0; k < n; ++k) trows[fill[tile_of[order[k]]]++] = order[k];
  }
  std::vector<unsigned> local(n);
  for (unsigned t = 0; t < ntiles; ++t) {
    unsigned *b = trows.data() + tstart[t], *e = trows.data() + tstart[t + 1];
    std::stable_sort(b, e, [&](unsigned x, unsigned y) { return lev[x] < lev[y]; });
    const unsigned nr = (unsigned)(e - b);
    for (unsigned k = 0; k < nr; ++k) local[b[k]] = k;
  }
  // group records (row ids, codes) and per-step halo lists; rows whose 32-byte
  // copy (FP32 or FP64) would pass the end of the vector are read in global
  // memory instead (kTiGlobal codes), as are halo rows beyond kTiHalo
  const unsigned Mc = round4u(M);
  const size_t words = (size_t)kTiG * (Mc + 1u);
  auto copyable = [&](unsigned d) {
    return (((size_t)d * 12u) & ~(size_t)15) + 32u <= (size_t)n * 12u &&
           (((size_t)d * 24u) & ~(size_t)15) + 32u <= (size_t)n * 24u;
  };
  std::vector<uint4> tiles(2 * (size_t)ntiles), steps;
  std::vector<unsigned> rec_of(n), gmeta, halo, hidx(n, ~0u), hrows;
  size_t ngroups = 0;
  unsigned max_groups = 0, max_halo = 0;
  for (unsigned t = 0; t < ntiles; ++t) {
    const unsigned *b = trows.data() + tstart[t];
    const unsigned nr = tstart[t + 1] - tstart[t];
    tiles[2 * t] = make_uint4((unsigned)(steps.size() / 2), 0u, (unsigned)ngroups, 0u);
    tiles[2 * t + 1] = make_uint4((unsigned)halo.size(), 0u, 0u, 0u);
    unsigned k = 0;
    while (k < nr) {
      unsigned k1 = k;
      while (k1 < nr && lev[b[k1]] == lev[b[k]]) ++k1;
      const unsigned w = k1 - k, ng = (w + kTiG - 1) / kTiG;
      hrows.clear();
      for (unsigned u = k; u < k1; ++u) {
        const unsigned i = b[u];
        const unsigned s0 = fwd ? rs[i] : dia[i], s1 = fwd ? dia[i] : rs[i + 1];
        for (unsigned s = s0; s < s1; ++s) {
          const unsigned d = col[s];
          if (tile_of[d] != t && hidx[d] == ~0u && copyable(d) && hrows.size() < kTiHalo) {
            hidx[d] = (unsigned)hrows.size();
            hrows.push_back(d);
          }
        }
      }
      const unsigned hoff = (unsigned)halo.size(), hc = (unsigned)hrows.size();
      for (unsigned h = 0; h < hc; ++h) halo.push_back(hrows[h]);
      while (halo.size() % 4u) halo.push_back(0u);
      max_halo = std::max(max_halo, hc);
      gmeta.resize((ngroups + ng) * words, 0u);
      for (size_t g = ngroups; g < ngroups + ng; ++g)
        for (unsigned q = 0; q < kTiG; ++q) {
          gmeta[g * words + q] = ~0u;
          for (unsigned bb = 0; bb < Mc; ++bb) gmeta[g * words + kTiG + q * Mc + bb] = kTiLocal | max_rows;
        }
      for (unsigned u = 0; u < w; ++u) {
        const unsigned i = b[k + u];
        const size_t g = ngroups + u / kTiG;
        const unsigned q = u % kTiG;
        rec_of[i] = (unsigned)(g * kTiG + q);
        gmeta[g * words + q] = i;
        const unsigned s0 = fwd ? rs[i] : dia[i], s1 = fwd ? dia[i] : rs[i + 1];
        for (unsigned s = s0; s < s1; ++s) {
          const unsigned d = col[s];
          unsigned code;
          if (tile_of[d] == t) {
            code = kTiLocal | local[d];
          } else if (hidx[d] != ~0u) {
            const unsigned o32 = (unsigned)(((size_t)d * 12u) & 15u) / 4u;
            const unsigned o64 = (unsigned)(((size_t)d * 24u) & 15u) / 8u;
            code = hidx[d] | (o32 << 8) | (o64 << 10);
          } else {
            code = kTiGlobal | d;
          }
          gmeta[g * words + kTiG + q * Mc + (s - s0)] = code;
        }
      }
      for (unsigned d : hrows) hidx[d] = ~0u;
      steps.push_back(make_uint4((unsigned)ngroups, w, k, ng));
      steps.push_back(make_uint4(hoff, hc, 0u, 0u));
      max_groups = std::max(max_groups, ng);
      ngroups += ng;
      k = k1;
    }
    tiles[2 * t].y = (unsigned)(steps.size() / 2) - tiles[2 * t].x;
    tiles[2 * t].w = (unsigned)ngroups - tiles[2 * t].z;
    tiles[2 * t + 1].y = (unsigned)halo.size() - tiles[2 * t + 1].x;
  }
  if ((ngroups + 1) * kTiG >= 0xFFFFFFFFull || halo.size() >= 0xFFFFFFFFull) return;
  out.ntiles = ntiles;
  out.nsteps = (unsigned)(steps.size() / 2);
  out.M = M;
  out.max_groups = max_groups;
  out.max_halo = max_halo;
  out.ngroups = ngroups;
  out.tiles = std::move(tiles);
  out.steps = std::move(steps);
  out.rec_of = std::move(rec_of);
  out.gmeta = std::move(gmeta);
  out.halo = std::move(halo);
  out.ok = true;
}

int tile_upload(unsigned n, const TileHost &h, TileSched &ts) {
  ts.ok = false;
  if (!h.ok) return DFM2G_OK;
  ts.ntiles = h.ntiles;
  ts.nsteps = h.nsteps;
  ts.rows_per_step = ts.nsteps ? (double)n / ts.nsteps : 0.0;
  ts.ngroups = h.ngroups;
  ts.max_groups = h.max_groups;
  ts.max_halo = h.max_halo;
  ts.M = h.M;
  DFM2G_TRY(ts.tiles.resize(h.tiles.size() + 2));
  DFM2G_TRY(ts.steps.resize(h.steps.size() + 2));
  DFM2G_TRY(ts.rec_of.resize((size_t)n + 1));
  DFM2G_TRY(ts.gmeta.resize(h.gmeta.size() + 1));
  DFM2G_TRY(ts.halo.resize(h.halo.size() + 4));
  DFM2G_TRY(ts.ctr.resize(2));
  DFM2G_CUDA(cudaMemcpy(ts.tiles.p, h.tiles.data(), sizeof(uint4) * h.tiles.size(), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(ts.steps.p, h.steps.data(), sizeof(uint4) * h.steps.size(), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(ts.rec_of.p, h.rec_of.data(), sizeof(unsigned) * n, cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(ts.gmeta.p, h.gmeta.data(), sizeof(unsigned) * h.gmeta.size(), cudaMemcpyHostToDevice));
  if (!h.halo.empty())
    DFM2G_CUDA(cudaMemcpy(ts.halo.p, h.halo.data(), sizeof(unsigned) * h.halo.size(), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemset(ts.ctr.p, 0, 2 * sizeof(unsigned)));
  ts.ok = true;
  return DFM2G_OK;
}

// Builds the tile schedules that are not built yet, of both value types and
// both directions (the FP64 ones on first use of the FP32 ones and the other
// way round, so that a first solve in the other precision finds them): the
// host partitions on one thread each.
int tile_build(dfm2g_ilu_s *p) {
  const unsigned n = p->nblk;
  bool need[2][2], any = false, need_dir[2] = {false, false};
  for (int f = 0; f < 2; ++f)
    for (int d = 0; d < 2; ++d) {
      TileSched &ts = p->tiles[f][d];
      need[f][d] = !ts.built;
      ts.built = true;
      if (need[f][d]) ts.ok = false;
      any |= need[f][d];
      need_dir[d] |= need[f][d];
    }
  if (!any) return DFM2G_OK;
  if (n >= kTiGlobal) return DFM2G_OK;  // row ids must fit the codes' 30 bits
  std::vector<unsigned> rs, col, dia, order[2];
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  DFM2G_TRY(tile_to_host(rs, p->row_start.p, (size_t)n + 1));
  DFM2G_TRY(tile_to_host(col, p->col.p, p->nnz));
  DFM2G_TRY(tile_to_host(dia, p->dia_ind.p, n));
  if (need_dir[0]) DFM2G_TRY(tile_to_host(order[0], p->order_f.p, n));
  if (need_dir[1]) DFM2G_TRY(tile_to_host(order[1], p->order_b.p, n));
  TileHost h[2][2];
  // an exception inside a worker (out of host memory) is caught there: it
  // leaves that schedule unusable and the call reports DFM2G_ERR_HOST
  std::atomic<bool> failed{false};
  std::vector<std::thread> workers;
  try {
    for (int f = 0; f < 2; ++f)
      for (int d = 0; d < 2; ++d)
        if (need[f][d])
          workers.emplace_back([&, f, d]() {
            try {
              tile_host_build(n, rs, col, dia, order[d], d == 0, tile_rows(f ? 8u : 4u), h[f][d]);
            } catch (...) {
              h[f][d].ok = false;
              failed = true;
            }
          });
  } catch (...) {  // a thread that could not start: join the others before leaving
    for (std::thread &w : workers) w.join();
    throw;
  }
  for (std::thread &w : workers) w.join();
  if (failed) return fail(DFM2G_ERR_HOST, "tile schedule: out of host memory while partitioning");
  for (int f = 0; f < 2; ++f)
    for (int d = 0; d < 2; ++d)
      if (need[f][d]) DFM2G_TRY(tile_upload(n, h[f][d], p->tiles[f][d]));
  return DFM2G_OK;
}

template <typename T, bool FWD>
void *tile_kernel(unsigned MR) {
  if (MR <= 8) return (void *)k_sweep_tiles<T, FWD, 8>;
  return (void *)k_sweep_tiles<T, FWD, 16>;
}

// Lets `kernel` launch with `smem` bytes of dynamic shared memory. The
// attribute belongs to the kernel, not to a pattern, so it only ever grows
// (per kernel and device).
int tile_allow_smem(void *kernel, size_t smem) {
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

}  // namespace

// Builds the tiles of one direction (first use), rewrites the records of the
// value type after each decomposition, gathers the right-hand side into the
// records' row order and launches the sweep; false in *usable when the
// pattern does not suit the schedule (rows with more than 16 dependencies, or
// a ring that does not fit), or when !may_alloc and the tiles or records do
// not exist yet.
template <typename T>
int tile_sweep(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia, const int *skip,
               unsigned long long timeout, bool may_alloc, bool pick, bool *usable) {
  const bool f64 = sizeof(T) == 8;
  TileSched &ts = p->tiles[f64 ? 1 : 0][forward ? 0 : 1];
  *usable = false;
  if (p->ndim != 3) return DFM2G_OK;
  // DFM2G_SWEEP_AUTO takes no tiles for rows of more than kTiAutoDeps blocks
  // (ILU(k > 0) of voxel blocks: the chains are 1.5x faster even where its
  // FP32 tiles hold 25-30 rows per step), so their tiles are not built
  if (pick && (forward ? p->max_lower : p->max_upper) > kTiAutoDeps) return DFM2G_OK;
  if (!may_alloc && (!ts.built || !ts.ok || !ts.bytes.p)) return DFM2G_OK;
  if (!ts.built) DFM2G_TRY(tile_build(p));  // both directions and value types
  if (!ts.ok) return DFM2G_OK;
  // DFM2G_SWEEP_AUTO: tiles only where their steps are full (ILU(0) of voxel
  // blocks: 33-40 rows per step; cloth sheets 9-15, where the chains are
  // 1.1-1.3x faster; FP64 on 26 tiles of a 32^3 block: the chains by 7%)
  if (pick && (ts.rows_per_step < kTiAutoRows || (f64 && 2u * ts.ntiles < (unsigned)ctx().num_sms)))
    return DFM2G_OK;
  const unsigned S = (unsigned)sizeof(T);
  const TileGeom g = tile_geom(ts.M, S, forward);
  const SlotGeom sg = slot_geom(ts.max_groups, g.gbytes, S);
  // ring slots: as many as fit (at most kTiMaxSlots, at least kTiMinLead + 2);
  // the halo lead: kTiHaloLead where the ring has two slots more (a step's
  // records land at least two issues before its halo copies start)
  unsigned nslots = kTiMaxSlots;
  while (nslots > kTiMinLead + 2 && tile_smem(S, nslots, sg.bytes) > kTiSmemCap) --nslots;
  unsigned lead = std::min(kTiHaloLead, nslots - 2u);
  const size_t smem = tile_smem(S, nslots, sg.bytes);
  if (smem > kTiSmemCap) return DFM2G_OK;
  DevBuf<unsigned char> &bytes = ts.bytes;
  unsigned &ver = ts.ver;
  if (!bytes.p) {
    DFM2G_TRY(bytes.resize(ts.ngroups * g.gbytes + 16));
    DFM2G_CUDA(cudaMemsetAsync(bytes.p, 0, ts.ngroups * g.gbytes + 16, stream()));
    ver = ~0u;
  }
  if (ver != p->factor_version) {
    const unsigned blocks = ctx().num_sms * 16;
    if (forward)
      k_tile_fill<T, true><<<blocks, 256, 0, stream()>>>(p->nblk, ts.ngroups, p->row_start.p, p->dia_ind.p, vcrs,
                                                          vdia, ts.rec_of.p, ts.gmeta.p, ts.M, g.Mc, g.vo,
                                                          g.gbytes, bytes.p);
    else
      k_tile_fill<T, false><<<blocks, 256, 0, stream()>>>(p->nblk, ts.ngroups, p->row_start.p, p->dia_ind.p, vcrs,
                                                           vdia, ts.rec_of.p, ts.gmeta.p, ts.M, g.Mc, g.vo,
                                                           g.gbytes, bytes.p);
    DFM2G_LAUNCH_CHECK();
    note_launches(1);
    ver = p->factor_version;
  }
  const unsigned MR = tile_rounds(ts.M);
  void *kernel = forward ? tile_kernel<T, true>(MR) : tile_kernel<T, false>(MR);
  DFM2G_TRY(tile_allow_smem(kernel, smem));
  int &cap = ts.coop;
  if (cap <= 0) {
    int per_sm = 0;
    DFM2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTiThreads, smem));
    if (per_sm <= 0) return DFM2G_OK;
    cap = per_sm * ctx().num_sms;
  }
  const unsigned blocks = std::min<unsigned>((unsigned)cap, ts.ntiles);
  unsigned ntiles = ts.ntiles, M = ts.M, vo = g.vo, gb = g.gbytes;
  const uint4 *tiles = ts.tiles.p;
  const uint4 *steps = ts.steps.p;
  const unsigned char *bp = bytes.p;
  const unsigned *hl = ts.halo.p;
  unsigned *ctr = ts.ctr.p;
  int *err = p->err.p;
  SlotGeom sgv = sg;
  void *args[] = {(void *)&ntiles, (void *)&tiles, (void *)&steps, (void *)&bp,   (void *)&in,
                  (void *)&hl,     (void *)&M,     (void *)&vo,    (void *)&gb,   (void *)&nslots,
                  (void *)&lead,   (void *)&sgv,   (void *)&out,   (void *)&ctr,  (void *)&err,
                  (void *)&timeout, (void *)&skip};
  DFM2G_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(blocks), dim3(kTiThreads), args, smem, stream()));
  note_launches(1);
  *usable = true;
  return DFM2G_OK;
}

template int tile_sweep<float>(dfm2g_ilu_s *, bool, const float *, float *, const float *, const float *,
                               const int *, unsigned long long, bool, bool, bool *);
template int tile_sweep<double>(dfm2g_ilu_s *, bool, const double *, double *, const double *, const double *,
                                const int *, unsigned long long, bool, bool, bool *);

// Drops the tiles and records (a new pattern); rebuilt on first use.
void tile_schedules_reset(dfm2g_ilu_s *p) {
  for (TileSched *ts : {&p->tiles[0][0], &p->tiles[0][1], &p->tiles[1][0], &p->tiles[1][1]}) {
    ts->built = ts->ok = false;
    ts->ntiles = ts->nsteps = ts->M = ts->max_groups = ts->max_halo = 0;
    ts->rows_per_step = 0;
    ts->ngroups = 0;
    ts->ver = ~0u;
    ts->coop = 0;
    ts->tiles.release();
    ts->steps.release();
    ts->rec_of.release();
    ts->gmeta.release();
    ts->halo.release();
    ts->bytes.release();
    ts->ctr.release();
  }
}

}  // namespace dfm2g

using namespace dfm2g;

extern "C" {

// Host-only: the tile partition the tile schedule uses. No device work.
int dfm2g_tile_partition(unsigned n, const unsigned *row_start, const unsigned *col, const unsigned *dia_ind,
                         const unsigned *order, int backward, unsigned max_rows, unsigned max_width,
                         unsigned *tile_of, unsigned *level, unsigned *ntiles, unsigned *max_deps) try {
  if (n && (!row_start || !col || !dia_ind || !order || !tile_of || !level))
    return fail(DFM2G_ERR_ARG, "tile_partition: null array");
  if (max_rows == 0 || max_width == 0) return fail(DFM2G_ERR_ARG, "tile_partition: zero tile size");
  std::vector<unsigned> t, lv;
  unsigned nt = 0, m = 0;
  tile_partition(n, row_start, dia_ind, col, order, backward == 0, max_rows, max_width, t, lv, nt, m);
  if (n) {
    std::copy(t.begin(), t.end(), tile_of);
    std::copy(lv.begin(), lv.end(), level);
  }
  if (ntiles) *ntiles = nt;
  if (max_deps) *max_deps = m;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

}  // extern "C"

// Cluster-scheduled triangular sweep (DFM2G_SWEEP_CLUSTER), 3x3 blocks, FP32
// and FP64, for patterns whose solution vector fits in one CTA's shared
// memory (at most 9,400 block rows in FP64, 18,900 in FP32).
//
// One thread-block cluster of kClCtas CTAs walks the level sets in order and
// meets at a cluster barrier after each level. Every CTA keeps the whole
// solution vector in its shared memory: a row's result goes to global memory
// and to every CTA's copy (distributed shared memory), so after the level's
// barrier each CTA reads every dependency from its own shared memory. The rows
// of a level go round-robin to the cluster's kClCtas * kClWarps warps; a warp
// computes a row with one lane per block (a warp sum per component), and loads
// the data of its next row (block columns and values, right-hand side, D^-1)
// while it computes the current one, with the row descriptor one row further
// ahead. The level sets and their per-position descriptors are the ones every
// schedule uses, so nothing is built for this schedule and it allocates
// nothing.
//
// Against the chain and tile schedules this trades the global-memory hand-off
// between warps (a store, its visibility in L2 and a poll) for a distributed
// shared-memory store and a cluster barrier per level. Measured on GB300 it
// costs about 1.3 us per level in FP32 and 2.9 us in FP64 (cloth sheets of
// 32-96 cells, voxel blocks of 16^3-20^3), more than the chains' hand-offs:
// the automatic choice does not take it; it is faster only on the smallest
// systems (an 8^3 voxel block in FP32).
//
// Progress: every thread of every CTA runs the same number of cluster barriers
// (one per level, one before the first and one after the last), whatever rows
// it has; there are no waits on data.
#include "common.cuh"
#include "tma.cuh"

namespace dfm2g {

namespace {

constexpr unsigned kClCtas = 8;   // CTAs per cluster (the portable maximum)
constexpr unsigned kClWarps = 8;  // warps per CTA
constexpr unsigned kClThreads = 32 * kClWarps;
constexpr unsigned kClSlots = kClCtas * kClWarps;
constexpr size_t kClSmemCap = 227u * 1024u;

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// shared-memory address `addr` of this CTA mapped to CTA `rank` of the cluster
__device__ __forceinline__ unsigned mapa_shared(unsigned addr, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_cluster(unsigned addr, float v) {
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}
__device__ __forceinline__ void st_cluster(unsigned addr, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(addr), "d"(v) : "memory");
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// One lane's share of a row: its block (lane k holds block k of the row's
// first 32) and, on lanes 0-2, the row's right-hand side component and row of
// D^-1 (forward).
template <typename T>
struct ClRow {
  unsigned row, s0, s1, c;  // c: the lane's block column (~0u: none)
  T b[9];
  T in, d0, d1, d2;
};

// dynamic shared memory: level starts (nlev + 1 u32), then x (3 n values)
__host__ __device__ inline size_t cl_x_off(unsigned nlev) { return ((size_t)(nlev + 1) * 4u + 15u) & ~(size_t)15; }

template <typename T, bool FWD>
__global__ void __cluster_dims__(kClCtas, 1, 1) __launch_bounds__(kClThreads, 1)
    k_sweep_cluster(unsigned nlev, const unsigned *__restrict__ lstart, const uint4 *__restrict__ meta,
                    const unsigned *__restrict__ col, const T *__restrict__ vcrs, const T *__restrict__ vdia,
                    const T *__restrict__ in, T *__restrict__ out, const int *skip) {
  extern __shared__ __align__(16) unsigned char cl_smem[];
  if (skip && *skip) return;  // every CTA reads the same value before any barrier
  unsigned *ls = reinterpret_cast<unsigned *>(cl_smem);
  T *xs = reinterpret_cast<T *>(cl_smem + cl_x_off(nlev));
  for (unsigned k = threadIdx.x; k <= nlev; k += blockDim.x) ls[k] = lstart[k];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const unsigned slot = cluster_rank() * kClWarps + warp;
  unsigned remote[kClCtas];
#pragma unroll
  for (unsigned r = 0; r < kClCtas; ++r) remote[r] = mapa_shared(smem_u32(xs), r);
  __syncthreads();
  cluster_sync();  // every CTA's shared memory is live before the first remote store

  // this warp's rows: position `slot` of each level, then every kClSlots-th
  struct It {
    unsigned L, j;  // level, position in the level order (L == nlev: none)
  };
  auto advance = [&](It it) -> It {
    if (it.L >= nlev) return it;
    if (it.j + kClSlots < ls[it.L + 1]) return It{it.L, it.j + kClSlots};
    for (unsigned L = it.L + 1; L < nlev; ++L)
      if (ls[L] + slot < ls[L + 1]) return It{L, ls[L] + slot};
    return It{nlev, 0u};
  };
  auto load = [&](ClRow<T> &R, const uint4 &m) {
    R.row = m.x;
    R.s0 = m.y;
    R.s1 = m.z;
    const unsigned s = m.y + lane;
    R.c = ~0u;
    if (s < m.z) {
      R.c = col[s];
#pragma unroll
      for (unsigned k = 0; k < 9; ++k) R.b[k] = vcrs[(size_t)s * 9 + k];
    }
    if (lane < 3) {
      R.in = in[(size_t)m.x * 3 + lane];
      if constexpr (FWD) {
        R.d0 = vdia[(size_t)m.x * 9 + lane * 3 + 0];
        R.d1 = vdia[(size_t)m.x * 9 + lane * 3 + 1];
        R.d2 = vdia[(size_t)m.x * 9 + lane * 3 + 2];
      }
    }
  };
  auto compute = [&](const ClRow<T> &R) {
    T p0 = T(0), p1 = T(0), p2 = T(0);
    if (R.c != ~0u) {
      const T x0 = xs[(size_t)R.c * 3 + 0], x1 = xs[(size_t)R.c * 3 + 1], x2 = xs[(size_t)R.c * 3 + 2];
      p0 = R.b[0] * x0 + R.b[1] * x1 + R.b[2] * x2;
      p1 = R.b[3] * x0 + R.b[4] * x1 + R.b[5] * x2;
      p2 = R.b[6] * x0 + R.b[7] * x1 + R.b[8] * x2;
    }
    for (unsigned s = R.s0 + 32u + lane; s < R.s1; s += 32u) {  // rows of more than 32 blocks
      const unsigned c = col[s];
      const T *B = vcrs + (size_t)s * 9;
      const T x0 = xs[(size_t)c * 3 + 0], x1 = xs[(size_t)c * 3 + 1], x2 = xs[(size_t)c * 3 + 2];
      p0 += B[0] * x0 + B[1] * x1 + B[2] * x2;
      p1 += B[3] * x0 + B[4] * x1 + B[5] * x2;
      p2 += B[6] * x0 + B[7] * x1 + B[8] * x2;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      p0 += __shfl_xor_sync(0xffffffffu, p0, o);
      p1 += __shfl_xor_sync(0xffffffffu, p1, o);
      p2 += __shfl_xor_sync(0xffffffffu, p2, o);
    }
    const T acc = R.in - (lane == 0u ? p0 : (lane == 1u ? p1 : p2));  // meaningful on lanes 0-2
    T z;
    if constexpr (FWD) {
      const T a0 = __shfl_sync(0xffffffffu, acc, 0), a1 = __shfl_sync(0xffffffffu, acc, 1),
              a2 = __shfl_sync(0xffffffffu, acc, 2);
      z = R.d0 * a0 + R.d1 * a1 + R.d2 * a2;
    } else {
      z = acc;
    }
    if (lane < 3) {
      const size_t k = (size_t)R.row * 3 + lane;
      out[k] = z;
      const unsigned off = (unsigned)(k * sizeof(T));
#pragma unroll
      for (unsigned r = 0; r < kClCtas; ++r) st_cluster(remote[r] + off, z);
    }
  };

  It a{nlev, 0u};  // the warp's first row: position `slot` of the first level that has it
  for (unsigned L = 0; L < nlev; ++L)
    if (ls[L] + slot < ls[L + 1]) {
      a = It{L, ls[L] + slot};
      break;
    }
  It b = advance(a), c = advance(b);
  ClRow<T> cur, nxt;
  uint4 mb = make_uint4(0u, 0u, 0u, 0u);
  if (a.L < nlev) load(cur, meta[a.j]);
  if (b.L < nlev) mb = meta[b.j];
  for (unsigned L = 0; L < nlev; ++L) {
    while (a.L == L) {
      // the next row's data and the one after's descriptor, in flight while this row is computed
      if (b.L < nlev) load(nxt, mb);
      const uint4 mc = c.L < nlev ? meta[c.j] : make_uint4(0u, 0u, 0u, 0u);
      compute(cur);
      a = b;
      b = c;
      c = advance(c);
      cur = nxt;
      mb = mc;
    }
    cluster_sync();
  }
}

}  // namespace

// Sweeps over the cluster schedule when the pattern is 3x3 and its solution
// vector fits in shared memory; *usable = false otherwise.
template <typename T>
int cluster_sweep(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia, const int *skip,
                  bool *usable) {
  *usable = false;
  if (p->ndim != 3 || p->nblk == 0) return DFM2G_OK;
  const unsigned nlev = forward ? p->nlev_f : p->nlev_b;
  const size_t smem = cl_x_off(nlev) + (size_t)p->nblk * 3u * sizeof(T);
  if (smem > kClSmemCap) return DFM2G_OK;
  void *kernel = forward ? (void *)k_sweep_cluster<T, true> : (void *)k_sweep_cluster<T, false>;
  static size_t allowed[2][2] = {{0, 0}, {0, 0}};  // largest size set per kernel (the attribute only grows)
  static int allowed_dev = -1;
  if (allowed_dev != ctx().device) {
    allowed[0][0] = allowed[0][1] = allowed[1][0] = allowed[1][1] = 0;
    allowed_dev = ctx().device;
  }
  size_t &al = allowed[sizeof(T) == 8 ? 1 : 0][forward ? 1 : 0];
  if (smem > al) {
    DFM2G_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    al = smem;
  }
  const unsigned *ls = forward ? p->lstart_f.p : p->lstart_b.p;
  const uint4 *meta = forward ? p->meta_f.p : p->meta_b.p;
  if (forward)
    k_sweep_cluster<T, true><<<kClCtas, kClThreads, smem, stream()>>>(nlev, ls, meta, p->col.p, vcrs, vdia, in, out,
                                                                      skip);
  else
    k_sweep_cluster<T, false><<<kClCtas, kClThreads, smem, stream()>>>(nlev, ls, meta, p->col.p, vcrs, vdia, in, out,
                                                                       skip);
  DFM2G_LAUNCH_CHECK();
  note_launches(1);
  *usable = true;
  return DFM2G_OK;
}

template int cluster_sweep<float>(dfm2g_ilu_s *, bool, const float *, float *, const float *, const float *,
                                  const int *, bool *);
template int cluster_sweep<double>(dfm2g_ilu_s *, bool, const double *, double *, const double *, const double *,
                                   const int *, bool *);

}  // namespace dfm2g

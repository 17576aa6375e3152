// Shared internals of libdfm2g: error plumbing, the library stream, handle
// layouts and small device helpers. Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/dfm2g.h"

namespace dfm2g {

// ---- errors ----------------------------------------------------------------
void set_error(const char *fmt, ...);
int fail(int status, const char *fmt, ...);
// From a catch block of an entry point: records what was thrown and returns
// DFM2G_ERR_HOST (no exception crosses the C ABI).
int host_failure() noexcept;

#define DFM2G_CUDA(call)                                                              \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return ::dfm2g::fail(DFM2G_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, \
                           cudaGetErrorString(e_));                                   \
  } while (0)

#define DFM2G_TRY(call)            \
  do {                             \
    int s_ = (call);               \
    if (s_ != DFM2G_OK) return s_; \
  } while (0)

#define DFM2G_LAUNCH_CHECK() DFM2G_CUDA(cudaGetLastError())

// ---- instrumentation -----------------------------------------------------------
void note_launches(unsigned n);
void note_alloc();  // one device allocation (cudaMalloc) made by the library
// Times the launches between construction and destruction as one `kind`
// sample when profiling is on; counts them always.
struct ProfScope {
  int kind;
  unsigned n;
  bool on;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(int kind, unsigned launches);
  ~ProfScope();
};

// ---- context ---------------------------------------------------------------
struct Context {
  cudaStream_t stream = nullptr;
  cudaStream_t own = nullptr;
  int device = -1;
  int num_sms = 0;
};
Context &ctx();
int ensure_context();
inline cudaStream_t stream() { return ctx().stream; }

// ---- device buffers ----------------------------------------------------------
template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  int resize(size_t count) {
    if (count == n && p) return DFM2G_OK;
    release();
    if (count == 0) return DFM2G_OK;
    note_alloc();
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(DFM2G_ERR_CUDA, "cudaMalloc(%zu bytes): %s", count * sizeof(T),
                  cudaGetErrorString(e));
    }
    n = count;
    return DFM2G_OK;
  }
  int ensure(size_t count) { return (n >= count && p) ? DFM2G_OK : resize(count); }
};

// Stage a host or device vector argument: `dev()` is a device pointer holding
// the caller's data; copy_back() returns results to a host caller.
template <typename T>
struct VecArg {
  T *user = nullptr;
  size_t n = 0;
  int mem = DFM2G_MEM_DEVICE;
  DevBuf<T> tmp;
  int in(const T *u, size_t count, int m, bool copy_in) {
    user = const_cast<T *>(u);
    n = count;
    mem = m;
    if (m == DFM2G_MEM_DEVICE) return DFM2G_OK;
    if (m != DFM2G_MEM_HOST) return fail(DFM2G_ERR_ARG, "mem flag must be 0 (host) or 1 (device)");
    DFM2G_TRY(tmp.resize(count));
    if (copy_in && count)
      DFM2G_CUDA(cudaMemcpyAsync(tmp.p, u, count * sizeof(T), cudaMemcpyHostToDevice, stream()));
    return DFM2G_OK;
  }
  T *dev() const { return mem == DFM2G_MEM_DEVICE ? user : tmp.p; }
  int copy_back() {
    if (mem == DFM2G_MEM_HOST && n) {
      DFM2G_CUDA(cudaMemcpyAsync(user, tmp.p, n * sizeof(T), cudaMemcpyDeviceToHost, stream()));
      DFM2G_CUDA(cudaStreamSynchronize(stream()));
    }
    return DFM2G_OK;
  }
};

// ---- grid sizing -------------------------------------------------------------
inline unsigned blocks_for(size_t work, unsigned per_block, unsigned cap = 0xFFFFFFFFu) {
  size_t b = (work + per_block - 1) / per_block;
  if (b == 0) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

// ---- device helpers ------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float ld_relaxed(const float *p) {
  float v;
  asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ double ld_relaxed(const double *p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(float *p, float v) {
  asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(double *p, double v) {
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// "Not yet written" marker for values produced by the sync-free sweeps: an
// all-ones NaN. Arithmetic on the GPU only produces the canonical NaN
// (0x7fffffff / 0x7fffffffffffffff), so a computed value never equals it.
__device__ __forceinline__ bool is_pending(float v) { return __float_as_uint(v) == 0xffffffffu; }
__device__ __forceinline__ bool is_pending(double v) {
  return __double_as_longlong(v) == (long long)-1;
}
template <typename T>
__device__ __forceinline__ T pending_value() {
  if constexpr (sizeof(T) == 8)
    return __longlong_as_double(-1ll);
  else
    return __uint_as_float(0xffffffffu);
}

// Default bound on every device-side wait.
constexpr unsigned long long kWaitTimeoutNs = 1000000000ull;  // 1 s

// Block-wide FP64 sum; valid in thread 0. `sh` holds >= blockDim.x/32 doubles.
__device__ __forceinline__ double block_sum(double v, double *sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? sh[lane] : 0.0;
    v = warp_sum(v);
  }
  return v;
}

// Deterministic grid reduction: every block writes its partial sum, the last
// block to arrive (ticket) adds the partials in block order. Returns true in
// thread 0 of the last block, with *total set; the ticket is reset there.
__device__ __forceinline__ bool grid_sum_last(double partial, double *partials,
                                              unsigned *ticket, double *sh, double *total) {
  __shared__ bool am_last;
  double v = block_sum(partial, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = v;
    __threadfence();
    const unsigned t = atomicAdd(ticket, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double s = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) s += ld_relaxed(partials + b);
  // fixed-order combination: per-thread strided sums then a fixed tree
  s = block_sum(s, sh);
  if (threadIdx.x == 0) {
    *total = s;
    *ticket = 0;
  }
  return threadIdx.x == 0;
}

// Barrier of all CTAs of a cooperative launch: bar[0] counts arrivals, bar[1]
// is the generation the last arrival advances (both start at 0 and the count
// returns to 0, so one pair serves any number of barriers of successive
// launches on a stream). Bounded: false, with DFM2G_ERR_WAIT_TIMEOUT in
// *err, when the other CTAs do not all arrive within timeout_ns.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *err, unsigned long long timeout_ns) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned *gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const unsigned long long t0 = globaltimer_ns();
      while (*gen == g) {
        if (globaltimer_ns() - t0 > timeout_ns) {
          atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// Sum of partials[0, nparts) in a fixed order, the same in every CTA that
// calls it (all threads of the CTA receive it).
__device__ __forceinline__ double sum_partials_all(const double *partials, unsigned nparts, double *sh) {
  __shared__ double total_s;
  double s = 0.0;
  for (unsigned b = threadIdx.x; b < nparts; b += blockDim.x) s += ld_relaxed(partials + b);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) total_s = s;
  __syncthreads();
  return total_s;
}

}  // namespace dfm2g

// ---- handle layouts -----------------------------------------------------------------
struct dfm2g_bsr_s {
  unsigned nblk = 0;
  unsigned ndim = 3;  // block size: 3x3 (TMA SpMV, every sweep schedule), 1x1 or 2x2 (nd.cuh kernels)
  size_t nnz = 0;
  bool has_pattern = false;
  std::vector<unsigned> h_row_start, h_col;  // host copy of the pattern
  dfm2g::DevBuf<unsigned> row_start, col;
  dfm2g::DevBuf<double> vcrs, vdia;
  dfm2g::DevBuf<float> vcrs32, vdia32;
  bool f32_valid = false;
  unsigned pattern_version = 0;
  // row tiles of the TMA-staged SpMV (FP32: component layout, TileCfgC; FP64: TileCfg<double>); tiles_ok is
  // false when a row alone exceeds a tile
  dfm2g::DevBuf<unsigned> tiles32, tiles64;
  unsigned ntiles32 = 0, ntiles64 = 0;
  bool tiles_ok = false;
  dfm2g::DevBuf<int> err;  // bounded-wait error word of the SpMV kernels
};

// Blob schedule of one sweep direction (FP32): rows partitioned into compact
// groups, one CTA per group; see groups.cu.
struct GroupSched {
  bool ok = false;
  unsigned ngroups = 0, max_rows = 0, slot_bytes = 0, threads = 0, ring = 0;
  size_t smem = 0, nvblocks = 0;
  dfm2g::DevBuf<uint4> units;          // {byte offset, byte length, rows, 0}
  dfm2g::DevBuf<unsigned> gunit;       // ngroups+1: first unit of each group
  dfm2g::DevBuf<unsigned> growptr;     // ngroups+1: first position of each group in prow
  dfm2g::DevBuf<unsigned> prow;        // rows in processing order
  dfm2g::DevBuf<unsigned char> bytes;  // unit records (headers, dependency codes, values)
  dfm2g::DevBuf<unsigned> vsrc, vdst;  // value blocks: source (slot, or nnz+row for D^-1), destination
  bool values_ok = false;
};

// Row-range partition of one sweep direction (parts.cu): per part, its rows in
// the sweep's level order as position metadata {row, s0, s1, 0}.
struct PartSched {
  dfm2g::DevBuf<uint4> meta;
  dfm2g::DevBuf<unsigned> pstart;  // nparts+1 offsets into meta
};

// Level-ordered record stream of one sweep direction and value type
// (stream.cu): unit descriptors, records, and where each factor block goes.
struct StreamSched {
  bool built = false, ok = false;
  unsigned nunits = 0;
  size_t nvblocks = 0;
  unsigned values_version = ~0u;  // factor_version the values were copied from
  dfm2g::DevBuf<unsigned char> bytes;
  dfm2g::DevBuf<uint4> units;     // 2 per unit
  dfm2g::DevBuf<unsigned> vsrc;   // factor block: slot, or nnz + row for D^-1
  dfm2g::DevBuf<size_t> vdst;     // its first value in the stream
};

// Chains of one sweep direction (chain.cu): descriptors, the record of each
// row, and the row records per value type (rewritten after each decomposition).
struct ChainSched {
  bool built = false, ok = false;
  unsigned nchain = 0, m = 0;       // chains; longest cross list (blocks)
  unsigned ver32 = ~0u, ver64 = ~0u; // factor_version the records were written from
  int coop[2] = {0, 0};             // resident CTAs of the sweep kernel [f64]
  dfm2g::DevBuf<uint4> chains;      // {first row, rows, record of the first row, 0}
  dfm2g::DevBuf<unsigned> rec_of;   // record index of each row
  dfm2g::DevBuf<unsigned char> linked;  // 1 when the row continues its predecessor's chain
  dfm2g::DevBuf<unsigned char> bytes32, bytes64;
  dfm2g::DevBuf<unsigned> ctr;      // chain counter and done-ticket of the launch
};

// Tiles of one sweep direction and value type (tiles.cu; FP32 and FP64 tiles
// differ in size): tile and step descriptors, the record of each row, group
// headers and codes, per-step halo lists, and the records (rewritten after
// each decomposition).
struct TileSched {
  bool built = false, ok = false;
  unsigned ntiles = 0, nsteps = 0, M = 0, max_groups = 0, max_halo = 0;  // M: dependency slots per row
  double rows_per_step = 0;           // rows / steps: how full the tiles' steps are
  size_t ngroups = 0;
  unsigned ver = ~0u;                 // factor_version the records were written from
  int coop = 0;                       // resident CTAs of the sweep kernel
  dfm2g::DevBuf<uint4> tiles;         // 2 per tile: {first step, steps, first group, groups}, {halo words}
  dfm2g::DevBuf<uint4> steps;         // 2 per step: {first group, rows, local base, groups}, {halo list}
  dfm2g::DevBuf<unsigned> halo;       // per step: the rows of other tiles it reads
  dfm2g::DevBuf<unsigned> rec_of;     // 10 * group + position of each row
  dfm2g::DevBuf<unsigned> gmeta;      // per group: 10 row ids, then codes [10][Mc]
  dfm2g::DevBuf<unsigned char> bytes; // the records
  dfm2g::DevBuf<unsigned> ctr;        // tile counter and done-ticket of the launch
};

struct dfm2g_ilu_s {
  unsigned nblk = 0;
  unsigned ndim = 3;  // block size of the matrix the pattern was taken from
  size_t nnz = 0;
  bool has_pattern = false, has_factor = false, f32_valid = false;
  int sweep_mode = DFM2G_SWEEP_SYNCFREE;
  dfm2g::DevBuf<unsigned> row_start, col, dia_ind;
  dfm2g::DevBuf<double> vcrs, vdia;
  dfm2g::DevBuf<float> vcrs32, vdia32;
  // level sets: level[i], order (rows by (level,row)), level_start (nlev+1)
  dfm2g::DevBuf<unsigned> level_f, order_f, lstart_f, level_b, order_b, lstart_b;
  dfm2g::DevBuf<uint4> meta_f, meta_b;  // per position of the level order: {row, s0, s1, 0}
  dfm2g::DevBuf<unsigned> pos_f, pos_b; // position of each row in the level order
  GroupSched gs_f, gs_b;                // FP32 blob schedules (forward, backward)
  PartSched parts_f, parts_b;           // row-range partitions (forward, backward)
  StreamSched ss32_f, ss32_b, ss64_f, ss64_b;  // level streams of the single-CTA sweep
  ChainSched cs_f, cs_b;                // chain schedules (forward, backward)
  TileSched tiles[2][2];                // tile schedules [f64][backward]
  dfm2g::DevBuf<double> in_lv64;        // right-hand side gathered in level order
  dfm2g::DevBuf<float> in_lv32;
  unsigned factor_version = 0;          // incremented by each decomposition
  bool parts_ok = false;
  unsigned parts_rpp = 0, parts_n = 0;  // rows per part, number of parts
  std::vector<unsigned> group_of;       // blob of each row
  unsigned nlev_f = 0, nlev_b = 0;
  std::vector<unsigned> h_lstart_f, h_lstart_b;
  // scratch for the sweeps (sentinel-filled outputs) and the device error word
  dfm2g::DevBuf<double> tmp64a, tmp64b;
  dfm2g::DevBuf<float> tmp32a, tmp32b;
  dfm2g::DevBuf<int> err;
  dfm2g::DevBuf<int> nsing;
  int coop_cache[2][2][2] = {};         // resident blocks of the sync-free kernel [f64][fwd][wide]
  unsigned max_lower = 0, max_upper = 0; // longest triangle rows (blocks)
  int last_sched[2][2] = {{-1, -1}, {-1, -1}};  // schedule of the last sweep [f64][backward]
};

struct dfm2g_tetmesh_s {
  size_t np = 0, ntet = 0;
  unsigned nblk = 0;
  unsigned pattern_version = 0;
  const dfm2g_bsr_s *bsr = nullptr;
  dfm2g::DevBuf<double> xyz;
  dfm2g::DevBuf<unsigned> tet;        // ntet*4, original order
  dfm2g::DevBuf<unsigned> slot;       // ntet*16 slot ids (diagonal: 0xffffffff)
  dfm2g::DevBuf<unsigned> by_color;   // tets sorted by colour (stable)
  std::vector<unsigned> color_start;  // ncolor+1
};

namespace dfm2g {
// cross-file internals
int ilu_sweep(dfm2g_ilu_s *p, int prec, bool forward, const void *in, void *out);
int ilu_sweep_guarded(dfm2g_ilu_s *p, int prec, bool forward, const void *in, void *out, const int *skip);
int color_elements(const unsigned *elem, size_t nelem, unsigned nno, size_t np, std::vector<unsigned> &by_color,
                   std::vector<unsigned> &color_start);
void to_f32(size_t n, const double *in, float *out);
int build_slot_map(const unsigned *d_elem, size_t nelem, unsigned nno, const dfm2g_bsr_s *m, unsigned *d_slot);
int group_schedules_build(dfm2g_ilu_s *p);
int group_values_fill(dfm2g_ilu_s *p);
int group_sweep(dfm2g_ilu_s *p, bool forward, const float *in, float *out, const int *skip);
int part_schedules_build(dfm2g_ilu_s *p);
template <typename T>
int stream_sweep(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia, const int *skip,
                 unsigned long long timeout, bool may_alloc, bool *usable);
void stream_schedules_reset(dfm2g_ilu_s *p);
template <typename T>
int chain_sweep(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia, const int *skip,
                unsigned long long timeout, bool may_alloc, bool *usable);
void chain_schedules_reset(dfm2g_ilu_s *p);
template <typename T>
int tile_sweep(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia, const int *skip,
               unsigned long long timeout, bool may_alloc, bool pick, bool *usable);
void tile_schedules_reset(dfm2g_ilu_s *p);
template <typename T>
int cluster_sweep(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia, const int *skip,
                  bool *usable);
void tile_partition(unsigned n, const unsigned *rs, const unsigned *dia, const unsigned *col, const unsigned *order,
                    bool fwd, unsigned max_rows, unsigned max_width, std::vector<unsigned> &tile_of,
                    std::vector<unsigned> &lev, unsigned &ntiles, unsigned &m);
template <typename T>
int part_sweep(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia, const int *skip,
               unsigned long long timeout);
int bsr_spmv(dfm2g_bsr_s *m, int prec, void *y, double alpha, const void *x, double beta);
// Fails with DFM2G_ERR_UNSUPPORTED unless the matrix has 3x3 blocks (entry
// points whose kernels are written for 3x3 blocks call it first).
int require_3x3(const dfm2g_bsr_s *m, const char *what);
int bsr_tiles_build(dfm2g_bsr_s *m);
int bsr_check_err(dfm2g_bsr_s *m);
int ilu_ensure_f32(dfm2g_ilu_s *p);
int bsr_ensure_f32(dfm2g_bsr_s *m);
}  // namespace dfm2g

// Single-CTA level-stream triangular sweep (DFM2G_SWEEP_BLOCK), for patterns
// with few rows per level (the cloth sheet: ~64 rows on each of 1,021 levels).
//
// Each sweep direction is encoded once, per value type, as a byte stream of
// the rows in (level, row) order, cut into units of at most kUnitBytes bytes
// and kUnitRows rows that never span two levels. Unit layout (16-byte aligned):
//   [16 B: nrows, 0, 0, 0][nrows x u32 record offsets, padded to 16 B]
//   record: [16 B: row i, nb, position q, 0]
//           [nb x {column j, position p} (u32 pairs), padded to 16 B]
//           [nb x 9 factor values (+ 9 of D^-1 forward), row-major, padded to 16 B]
// The values are refreshed from the factors after each decomposition. A unit
// descriptor (global, read-only) gives its byte range, first position, row
// count, the end position of its level and whether it ends the level.
//
// One CTA of 32 warps: warp 31 streams the units and the matching slice of
// the level-ordered right-hand side (gathered by a separate kernel) into a
// kStages-deep shared-memory ring with cp.async.bulk (full/empty mbarriers).
// Warps 0..30 compute the unit's rows (lane layout of rowkern.cuh, two rows
// per warp at a time) and keep every result in a shared-memory ring indexed by
// position. A dependency at position p comes from that ring while no row of
// the current level can have reused its slot (p >= level end - kSlots), else
// from the global output, which this CTA wrote before the last level barrier.
// After a level's last unit the 31 consumer warps meet at a named barrier.
//
// Every mbarrier wait is bounded. The first timeout sets a shared abort flag:
// later waits return at once, the producer stops issuing and drains (bounded)
// what it issued, and the consumers still pass every level barrier (their
// sequence depends only on the descriptors), so the kernel always ends.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "rowkern.cuh"
#include "tma.cuh"

namespace dfm2g {

namespace {

constexpr unsigned kStThreads = 1024;
constexpr unsigned kStConsumers = kStThreads / 32 - 1;
constexpr unsigned kStStages = 4;
constexpr unsigned kUnitBytes = 16 * 1024;
constexpr unsigned kUnitRows = 62;  // one pass of 31 warps x 2 rows

template <typename T>
struct StreamCfg {
  static constexpr unsigned kInBytes = (kUnitRows * 3 * sizeof(T) + 32 + 15) / 16 * 16;
  static constexpr unsigned kStageBytes = kUnitBytes + kInBytes;
  static constexpr unsigned kSlots = sizeof(T) == 8 ? 4096u : 8192u;  // 96 KiB of recent results
  static constexpr size_t kRingBytes = (size_t)kSlots * 3 * sizeof(T);
  static constexpr size_t kSmem = 128 + kRingBytes + (size_t)kStStages * kStageBytes;
  static_assert(kStageBytes % 16 == 0, "16-byte stages");
};

inline size_t pad16(size_t x) { return (x + 15) & ~size_t(15); }

__device__ __forceinline__ void consumers_barrier() {
  asm volatile("bar.sync 1, %0;" ::"r"(kStConsumers * 32) : "memory");
}

template <typename T, bool FWD>
__device__ __forceinline__ T stream_row_acc(const unsigned char *rec, const RowLane &L, unsigned lim,
                                            const T (*ring)[3], const T *out, unsigned slots) {
  const uint4 h = *reinterpret_cast<const uint4 *>(rec);
  const uint2 *codes = reinterpret_cast<const uint2 *>(rec + 16);
  const T *vals = reinterpret_cast<const T *>(rec + 16 + ((8u * h.y + 15u) & ~15u));
  T acc = T(0);
  if (L.active) {
#pragma unroll 4
    for (unsigned t = L.g; t < h.y; t += 3u) {
      const uint2 c = codes[t];
      const T x = (c.y >= lim) ? ring[c.y & (slots - 1)][L.c] : out[(size_t)c.x * 3 + L.c];
      acc += vals[(size_t)t * 9 + L.e] * x;
    }
  }
  return acc;
}

template <typename T, bool FWD>
__device__ __forceinline__ void stream_row_finish(const unsigned char *rec, const T s[3], const T *inl,
                                                  unsigned q0, unsigned lane, T (*ring)[3], T *out,
                                                  unsigned slots) {
  if (lane >= 3) return;
  const uint4 h = *reinterpret_cast<const uint4 *>(rec);
  const T *in3 = inl + (size_t)(h.z - q0) * 3;
  const T t0 = in3[0] - s[0], t1 = in3[1] - s[1], t2 = in3[2] - s[2];
  T z;
  if (FWD) {
    const T *d = reinterpret_cast<const T *>(rec + 16 + ((8u * h.y + 15u) & ~15u)) + (size_t)h.y * 9 + lane * 3;
    z = d[0] * t0 + d[1] * t1 + d[2] * t2;
  } else {
    z = lane == 0 ? t0 : (lane == 1 ? t1 : t2);
  }
  ring[h.z & (slots - 1)][lane] = z;
  out[(size_t)h.x * 3 + lane] = z;
}

// Unit descriptor: {byte offset, byte length, first position, rows} and
// {end position of its level, 1 if it ends the level, 0, 0}.
template <typename T, bool FWD>
__global__ void __launch_bounds__(kStThreads, 1) k_sweep_stream(const uint4 *__restrict__ units, unsigned nunits,
                                                                const unsigned char *__restrict__ bytes,
                                                                const T *__restrict__ in_lv, T *out, int *err,
                                                                unsigned long long timeout_ns, const int *skip) {
  using C = StreamCfg<T>;
  extern __shared__ __align__(128) unsigned char st_smem[];
  if (skip && *skip) return;
  uint64_t *full = reinterpret_cast<uint64_t *>(st_smem);
  uint64_t *empty = full + kStStages;
  volatile unsigned *abort_flag = reinterpret_cast<volatile unsigned *>(empty + kStStages);
  T(*ring)[3] = reinterpret_cast<T(*)[3]>(st_smem + 128);
  unsigned char *stages = st_smem + 128 + C::kRingBytes;
  const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  if (threadIdx.x == 0) {
    for (unsigned s = 0; s < kStStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kStConsumers);
    }
    *abort_flag = 0u;
    mbar_fence_init();
  }
  __syncthreads();
  if (warp == kStConsumers) {
    if (lane != 0) return;
    // descriptors kStStages units ahead are requested before they are needed
    uint4 pre[kStStages];
#pragma unroll
    for (unsigned j = 0; j < kStStages; ++j) pre[j] = j < nunits ? units[2 * (size_t)j] : make_uint4(0u, 0u, 0u, 0u);
    unsigned u = 0;
    for (; u < nunits; ++u) {
      const unsigned s = u % kStStages;
      if (u >= kStStages &&
          (*abort_flag || !mbar_wait_bounded(&empty[s], ((u / kStStages) - 1) & 1u, timeout_ns))) {
        *abort_flag = 1u;
        atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
        break;
      }
      uint4 U = pre[0];
#pragma unroll
      for (unsigned j = 0; j + 1 < kStStages; ++j) pre[j] = pre[j + 1];
      pre[kStStages - 1] =
          u + kStStages < nunits ? units[2 * (size_t)(u + kStStages)] : make_uint4(0u, 0u, 0u, 0u);
      const size_t i0 = (size_t)U.z * 3 * sizeof(T), i1 = (size_t)(U.z + U.w) * 3 * sizeof(T);
      const size_t ia = i0 & ~size_t(15);
      const unsigned il = (unsigned)(((i1 + 15) & ~size_t(15)) - ia);
      unsigned char *st = stages + (size_t)s * C::kStageBytes;
      mbar_arrive_expect_tx(&full[s], U.y + il);
      tma_load_1d(st, bytes + U.x, U.y, &full[s]);
      tma_load_1d(st + kUnitBytes, reinterpret_cast<const unsigned char *>(in_lv) + ia, il, &full[s]);
    }
    const unsigned first = u > kStStages ? u - kStStages : 0u;
    for (unsigned j = first; j < u; ++j) mbar_wait_bounded(&full[j % kStStages], (j / kStStages) & 1u, timeout_ns);
    return;
  }
  const RowLane L(lane);
  uint4 U = nunits ? units[0] : make_uint4(0u, 0u, 0u, 0u), V = nunits ? units[1] : make_uint4(0u, 0u, 0u, 0u);
  for (unsigned u = 0; u < nunits; ++u) {
    const unsigned s = u % kStStages;
    // next unit's descriptor, requested before this unit's work
    const uint4 Un = u + 1 < nunits ? units[2 * (size_t)u + 2] : U;
    const uint4 Vn = u + 1 < nunits ? units[2 * (size_t)u + 3] : V;
    bool ok = !*abort_flag && mbar_wait_bounded(&full[s], (u / kStStages) & 1u, timeout_ns);
    if (!ok) {
      *abort_flag = 1u;
      atomicCAS(err, 0, DFM2G_ERR_WAIT_TIMEOUT);
    }
    if (ok) {
      const unsigned char *st = stages + (size_t)s * C::kStageBytes;
      const unsigned *offs = reinterpret_cast<const unsigned *>(st + 16);
      const T *inl = reinterpret_cast<const T *>(st + kUnitBytes + (((size_t)U.z * 3 * sizeof(T)) & 15));
      const unsigned lim = V.x > C::kSlots ? V.x - C::kSlots : 0u;
      for (unsigned r = warp; r < U.w; r += 2 * kStConsumers) {
        const unsigned r2 = r + kStConsumers;
        const unsigned char *ra = st + offs[r];
        const unsigned char *rb = r2 < U.w ? st + offs[r2] : ra;
        const T acc_a = stream_row_acc<T, FWD>(ra, L, lim, ring, out, C::kSlots);
        const T acc_b = r2 < U.w ? stream_row_acc<T, FWD>(rb, L, lim, ring, out, C::kSlots) : T(0);
        T sa[3], sb[3];
        row_reduce(acc_a, sa);
        row_reduce(acc_b, sb);
        stream_row_finish<T, FWD>(ra, sa, inl, U.z, lane, ring, out, C::kSlots);
        if (r2 < U.w) stream_row_finish<T, FWD>(rb, sb, inl, U.z, lane, ring, out, C::kSlots);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
    if (V.y) consumers_barrier();
    U = Un;
    V = Vn;
  }
}

template <typename T>
__global__ void k_gather_level_order(unsigned n, const unsigned *__restrict__ order, const T *__restrict__ in,
                                     T *__restrict__ in_lv) {
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const unsigned i = order[q];
    in_lv[(size_t)q * 3 + 0] = in[(size_t)i * 3 + 0];
    in_lv[(size_t)q * 3 + 1] = in[(size_t)i * 3 + 1];
    in_lv[(size_t)q * 3 + 2] = in[(size_t)i * 3 + 2];
  }
}

template <typename T>
__global__ void k_stream_values(size_t nvb, const unsigned *__restrict__ vsrc, const size_t *__restrict__ vdst,
                                size_t nnz, const T *__restrict__ vcrs, const T *__restrict__ vdia,
                                T *__restrict__ dst) {
  const size_t total = nvb * 9;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const size_t b = t / 9, e = t - b * 9;
    const size_t s = vsrc[b];
    dst[vdst[b] + e] = s < nnz ? vcrs[s * 9 + e] : vdia[(s - nnz) * 9 + e];
  }
}

template <typename V>
int to_host_vec(std::vector<V> &h, const V *d, size_t n) {
  h.resize(n);
  if (n) DFM2G_CUDA(cudaMemcpy(h.data(), d, n * sizeof(V), cudaMemcpyDeviceToHost));
  return DFM2G_OK;
}

// Encodes one direction for value size `vs` (4 or 8 bytes).
int build_stream(dfm2g_ilu_s *p, bool fwd, size_t vs, StreamSched &ss) {
  ss.ok = false;
  const unsigned n = p->nblk;
  std::vector<unsigned> rs, col, dia, order, pos;
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  DFM2G_TRY(to_host_vec(rs, p->row_start.p, (size_t)n + 1));
  DFM2G_TRY(to_host_vec(col, p->col.p, p->nnz));
  DFM2G_TRY(to_host_vec(dia, p->dia_ind.p, n));
  DFM2G_TRY(to_host_vec(order, fwd ? p->order_f.p : p->order_b.p, n));
  DFM2G_TRY(to_host_vec(pos, fwd ? p->pos_f.p : p->pos_b.p, n));
  const std::vector<unsigned> &ls = fwd ? p->h_lstart_f : p->h_lstart_b;
  auto rec_bytes = [&](unsigned i) {
    const size_t nb = fwd ? dia[i] - rs[i] : rs[i + 1] - dia[i];
    return 16 + pad16(8 * nb) + pad16((nb + (fwd ? 1 : 0)) * 9 * vs);
  };
  std::vector<unsigned char> bytes;
  std::vector<uint4> units;
  std::vector<unsigned> vsrc;
  std::vector<size_t> vdst;
  for (size_t l = 0; l + 1 < ls.size(); ++l) {
    unsigned q = ls[l];
    const unsigned qend = ls[l + 1];
    while (q < qend) {
      // rows [q, q1) form the next unit
      unsigned q1 = q;
      size_t body = 0;
      while (q1 < qend && q1 - q < kUnitRows) {
        const size_t rb = rec_bytes(order[q1]);
        if (pad16(16 + 4 * (size_t)(q1 - q + 1)) + body + rb > kUnitBytes) break;
        body += rb;
        ++q1;
      }
      if (q1 == q) return DFM2G_OK;  // one row alone exceeds a unit: schedule unavailable
      const unsigned nr = q1 - q;
      const size_t base = bytes.size(), head = pad16(16 + 4 * (size_t)nr), len = head + body;
      if (base + len > 0xFFFFFFF0ull) return DFM2G_OK;  // offsets are 32-bit
      bytes.resize(base + len, 0);
      unsigned char *u = bytes.data() + base;
      reinterpret_cast<unsigned *>(u)[0] = nr;
      size_t off = head;
      for (unsigned k = 0; k < nr; ++k) {
        const unsigned i = order[q + k];
        reinterpret_cast<unsigned *>(u + 16)[k] = (unsigned)off;
        const unsigned s0 = fwd ? rs[i] : dia[i], s1 = fwd ? dia[i] : rs[i + 1], nb = s1 - s0;
        unsigned *h = reinterpret_cast<unsigned *>(u + off);
        h[0] = i;
        h[1] = nb;
        h[2] = q + k;
        h[3] = 0;
        unsigned *codes = reinterpret_cast<unsigned *>(u + off + 16);
        for (unsigned t = 0; t < nb; ++t) {
          codes[2 * t] = col[s0 + t];
          codes[2 * t + 1] = pos[col[s0 + t]];
        }
        const size_t vbase = (base + off + 16 + pad16(8 * (size_t)nb)) / vs;  // in values
        for (unsigned t = 0; t < nb; ++t) {
          vsrc.push_back(s0 + t);
          vdst.push_back(vbase + (size_t)t * 9);
        }
        if (fwd) {
          vsrc.push_back((unsigned)(p->nnz + i));
          vdst.push_back(vbase + (size_t)nb * 9);
        }
        off += rec_bytes(i);
      }
      units.push_back(make_uint4((unsigned)base, (unsigned)len, q, nr));
      units.push_back(make_uint4(qend, q1 == qend ? 1u : 0u, 0u, 0u));
      q = q1;
    }
  }
  if (p->nnz + n >= 0xFFFFFFFFull) return DFM2G_OK;
  ss.nunits = (unsigned)(units.size() / 2);
  ss.nvblocks = vsrc.size();
  DFM2G_TRY(ss.bytes.resize(bytes.size() + 16));
  DFM2G_TRY(ss.units.resize(units.size() + 2));
  DFM2G_TRY(ss.vsrc.resize(vsrc.size() + 1));
  DFM2G_TRY(ss.vdst.resize(vdst.size() + 1));
  DFM2G_CUDA(cudaMemcpy(ss.bytes.p, bytes.data(), bytes.size(), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(ss.units.p, units.data(), sizeof(uint4) * units.size(), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(ss.vsrc.p, vsrc.data(), sizeof(unsigned) * vsrc.size(), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(ss.vdst.p, vdst.data(), sizeof(size_t) * vdst.size(), cudaMemcpyHostToDevice));
  ss.values_version = ~0u;
  ss.ok = true;
  return DFM2G_OK;
}

StreamSched &sched_of(dfm2g_ilu_s *p, bool fwd, double) { return fwd ? p->ss64_f : p->ss64_b; }
StreamSched &sched_of(dfm2g_ilu_s *p, bool fwd, float) { return fwd ? p->ss32_f : p->ss32_b; }
DevBuf<double> &in_lv_of(dfm2g_ilu_s *p, double) { return p->in_lv64; }
DevBuf<float> &in_lv_of(dfm2g_ilu_s *p, float) { return p->in_lv32; }

}  // namespace

// Builds (first use) and refreshes (after each decomposition) the stream of
// one direction and value type; false in *usable when the pattern does not fit,
// or when !may_alloc and the stream or its level-ordered input buffer does not
// exist yet (building them allocates).
template <typename T>
int stream_sweep(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia, const int *skip,
                 unsigned long long timeout, bool may_alloc, bool *usable) {
  StreamSched &ss = sched_of(p, forward, T(0));
  *usable = false;
  if (!may_alloc &&
      (!ss.built || !ss.ok || !in_lv_of(p, T(0)).p || in_lv_of(p, T(0)).n < (size_t)p->nblk * 3 + 16))
    return DFM2G_OK;
  if (!ss.built) {
    ss.built = true;
    DFM2G_TRY(build_stream(p, forward, sizeof(T), ss));
    if (ss.ok) {
      auto kernel = forward ? k_sweep_stream<T, true> : k_sweep_stream<T, false>;
      DFM2G_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)StreamCfg<T>::kSmem));
    }
  }
  if (!ss.ok) return DFM2G_OK;
  const unsigned n = p->nblk;
  if (ss.values_version != p->factor_version) {
    k_stream_values<T><<<blocks_for(ss.nvblocks * 9, 256, ctx().num_sms * 16), 256, 0, stream()>>>(
        ss.nvblocks, ss.vsrc.p, ss.vdst.p, p->nnz, vcrs, vdia, reinterpret_cast<T *>(ss.bytes.p));
    note_launches(1);
    DFM2G_LAUNCH_CHECK();
    ss.values_version = p->factor_version;
  }
  DevBuf<T> &in_lv = in_lv_of(p, T(0));
  DFM2G_TRY(in_lv.ensure((size_t)n * 3 + 16));
  k_gather_level_order<T><<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(
      n, forward ? p->order_f.p : p->order_b.p, in, in_lv.p);
  if (forward)
    k_sweep_stream<T, true><<<1, kStThreads, StreamCfg<T>::kSmem, stream()>>>(
        ss.units.p, ss.nunits, ss.bytes.p, in_lv.p, out, p->err.p, timeout, skip);
  else
    k_sweep_stream<T, false><<<1, kStThreads, StreamCfg<T>::kSmem, stream()>>>(
        ss.units.p, ss.nunits, ss.bytes.p, in_lv.p, out, p->err.p, timeout, skip);
  note_launches(2);
  DFM2G_LAUNCH_CHECK();
  *usable = true;
  return DFM2G_OK;
}

template int stream_sweep<float>(dfm2g_ilu_s *, bool, const float *, float *, const float *, const float *,
                                 const int *, unsigned long long, bool, bool *);
template int stream_sweep<double>(dfm2g_ilu_s *, bool, const double *, double *, const double *, const double *,
                                  const int *, unsigned long long, bool, bool *);

}  // namespace dfm2g

namespace dfm2g {
// Drops the streams (a new pattern); they are rebuilt on first use.
void stream_schedules_reset(dfm2g_ilu_s *p) {
  for (StreamSched *ss : {&p->ss32_f, &p->ss32_b, &p->ss64_f, &p->ss64_b}) {
    ss->built = ss->ok = false;
    ss->values_version = ~0u;
    ss->bytes.release();
    ss->units.release();
    ss->vsrc.release();
    ss->vdst.release();
  }
}
}  // namespace dfm2g

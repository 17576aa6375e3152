// Blob-scheduled FP32 triangular sweeps (sweep mode DFM2G_SWEEP_GROUPS).
//
// The rows are partitioned into compact blobs of the matrix graph (BFS region
// growing), at most as many blobs as CTAs that can be resident at once. One
// CTA owns one blob for the whole sweep (cooperative launch: all resident).
// It keeps the blob's right-hand side in shared memory and overwrites it in
// place with the solution, visiting its rows in (level, row) order in units
// of at most kRowsPerUnit rows of one level, with one __syncthreads per unit.
// A dependency inside the blob is read from shared memory; one outside waits
// (bounded) on the global output until it is no longer the pending marker.
// Deadlock-free: the lowest unfinished level can always proceed, because
// every blob is resident and sweeps its levels in increasing order.
//
// Each unit's data - row headers, dependency codes and factor values in
// processing order - is one contiguous, 16-byte-aligned byte range that the
// CTA streams into a kRing-slot shared-memory ring with cp.async, two units
// ahead of the one it computes. Unit layout:
//   [16 B: nrows][nrows x u16 record offsets, padded to 16 B]
//   records: [16 B: row, blocks incl. D^-1, off-diagonal blocks, blob position]
//            [off-diagonal dependency codes, i32, padded to 16 B]
//            [blocks x 9 values (row-major 3x3), f32, padded to 16 B]
// A dependency code d >= 0 is the blob position of the column row; d < 0 is
// -(column row) - 1 (outside the blob). The forward sweep's last block is D^-1.
#include <algorithm>
#include <climits>
#include <cstring>
#include <numeric>

#include "common.cuh"
#include "rowkern.cuh"

namespace dfm2g {

constexpr unsigned kGThreads = 256;
constexpr unsigned kRowsPerUnit = kGThreads / 4;  // 4 lanes per row: components 0..2 (+1 helper lane)
constexpr unsigned kRing = 3;
constexpr unsigned kCtasPerSm = 2;
constexpr size_t kUnitBytesCap = 16 * 1024;  // 3 slots + the blob vector fit twice per SM
constexpr size_t kSmemPerSm = 227 * 1024;

static inline size_t pad16(size_t x) { return (x + 15) & ~size_t(15); }

// ---- partition -------------------------------------------------------------------
// Breadth-first region growing from seeds in row order; blobs of `target` rows.
static unsigned grow_blobs(unsigned n, const std::vector<unsigned> &rs, const std::vector<unsigned> &col,
                           unsigned target, std::vector<unsigned> &gof) {
  gof.assign(n, UINT_MAX);
  unsigned ng = 0;
  std::vector<unsigned> q;
  q.reserve((size_t)target + 64);
  for (unsigned seed = 0; seed < n; ++seed) {
    if (gof[seed] != UINT_MAX) continue;
    const unsigned g = ng++;
    q.clear();
    q.push_back(seed);
    gof[seed] = g;
    for (size_t h = 0; h < q.size() && q.size() < target; ++h) {
      const unsigned i = q[h];
      for (unsigned s = rs[i]; s < rs[i + 1] && q.size() < target; ++s) {
        const unsigned j = col[s];
        if (gof[j] == UINT_MAX) {
          gof[j] = g;
          q.push_back(j);
        }
      }
    }
  }
  return ng;
}

// Merge the smallest blob into its smallest neighbouring blob (or the smallest
// blob overall when it has no neighbour) until at most `cap` blobs remain.
static unsigned merge_blobs(unsigned n, const std::vector<unsigned> &rs, const std::vector<unsigned> &col,
                            std::vector<unsigned> &gof, unsigned ng, unsigned cap) {
  std::vector<std::vector<unsigned>> mem(ng);
  for (unsigned i = 0; i < n; ++i) mem[gof[i]].push_back(i);
  std::vector<char> alive(ng, 1);
  unsigned live = ng;
  while (live > cap) {
    unsigned s = UINT_MAX;
    for (unsigned g = 0; g < ng; ++g)
      if (alive[g] && (s == UINT_MAX || mem[g].size() < mem[s].size())) s = g;
    unsigned t = UINT_MAX;
    for (unsigned i : mem[s])
      for (unsigned k = rs[i]; k < rs[i + 1]; ++k) {
        const unsigned g = gof[col[k]];
        if (g != s && (t == UINT_MAX || mem[g].size() < mem[t].size())) t = g;
      }
    if (t == UINT_MAX)
      for (unsigned g = 0; g < ng; ++g)
        if (alive[g] && g != s && (t == UINT_MAX || mem[g].size() < mem[t].size())) t = g;
    for (unsigned i : mem[s]) gof[i] = t;
    mem[t].insert(mem[t].end(), mem[s].begin(), mem[s].end());
    mem[s].clear();
    alive[s] = 0;
    --live;
  }
  std::vector<unsigned> relabel(ng, UINT_MAX);
  unsigned k = 0;
  for (unsigned g = 0; g < ng; ++g)
    if (alive[g]) relabel[g] = k++;
  for (unsigned i = 0; i < n; ++i) gof[i] = relabel[gof[i]];
  return k;
}

// ---- schedule of one direction --------------------------------------------------------
static int build_direction(GroupSched &gs, bool fwd, unsigned n, size_t nnz, unsigned ng,
                           const std::vector<unsigned> &gof, const std::vector<unsigned> &rs,
                           const std::vector<unsigned> &col, const std::vector<unsigned> &dia,
                           const std::vector<unsigned> &level) {
  gs.ok = false;
  std::vector<unsigned> gptr(ng + 1, 0), prow(n);
  for (unsigned i = 0; i < n; ++i) gptr[gof[i] + 1]++;
  for (unsigned g = 0; g < ng; ++g) gptr[g + 1] += gptr[g];
  {
    std::vector<unsigned> cur(gptr.begin(), gptr.end() - 1);
    for (unsigned i = 0; i < n; ++i) prow[cur[gof[i]]++] = i;
  }
  std::vector<unsigned> pos(n);
  unsigned max_rows = 0;
  for (unsigned g = 0; g < ng; ++g) {
    auto b = prow.begin() + gptr[g], e = prow.begin() + gptr[g + 1];
    std::sort(b, e, [&](unsigned x, unsigned y) { return level[x] != level[y] ? level[x] < level[y] : x < y; });
    for (unsigned p = gptr[g]; p < gptr[g + 1]; ++p) pos[prow[p]] = p - gptr[g];
    max_rows = std::max(max_rows, gptr[g + 1] - gptr[g]);
  }
  auto off_range = [&](unsigned i, unsigned &s0, unsigned &s1) {
    s0 = fwd ? rs[i] : dia[i];
    s1 = fwd ? dia[i] : rs[i + 1];
  };
  auto record_bytes = [&](unsigned i) {
    unsigned s0, s1;
    off_range(i, s0, s1);
    const size_t nbo = s1 - s0, nbt = nbo + (fwd ? 1 : 0);
    return 16 + pad16(nbo * 4) + pad16(nbt * 9 * sizeof(float));
  };
  // units: runs of one level within a blob, <= kRowsPerUnit rows, <= kUnitBytesCap bytes
  std::vector<uint4> units;
  std::vector<unsigned> gunit(ng + 1, 0);
  size_t total = 0, slot = 0;
  struct UnitRows {
    unsigned p0, p1;
  };
  std::vector<UnitRows> urows;
  for (unsigned g = 0; g < ng; ++g) {
    gunit[g] = (unsigned)units.size();
    unsigned p = gptr[g];
    while (p < gptr[g + 1]) {
      const unsigned lv = level[prow[p]];
      size_t bytes = 16 + pad16(2 * kRowsPerUnit);
      unsigned q = p;
      while (q < gptr[g + 1] && level[prow[q]] == lv && q - p < kRowsPerUnit) {
        const size_t rb = record_bytes(prow[q]);
        if (q > p && bytes + rb > kUnitBytesCap) break;
        bytes += rb;
        ++q;
      }
      if (bytes > 0xFFFF) return fail(DFM2G_ERR_UNSUPPORTED, "blob schedule: a unit exceeds 64 KiB");
      units.push_back(make_uint4((unsigned)total, (unsigned)bytes, q - p, 0u));
      urows.push_back({p, q});
      total += bytes;
      slot = std::max(slot, bytes);
      p = q;
    }
  }
  gunit[ng] = (unsigned)units.size();
  if (total > 0xFFFFFFF0ull) return fail(DFM2G_ERR_UNSUPPORTED, "blob schedule larger than 4 GiB");
  // bytes + value maps
  std::vector<unsigned char> bytes(total, 0);
  std::vector<unsigned> vsrc, vdst;
  vsrc.reserve(nnz / 2 + n);
  vdst.reserve(nnz / 2 + n);
  for (size_t u = 0; u < units.size(); ++u) {
    unsigned char *base = bytes.data() + units[u].x;
    const unsigned nr = units[u].z;
    std::memcpy(base, &nr, 4);
    unsigned short *rowoff = reinterpret_cast<unsigned short *>(base + 16);
    size_t off = 16 + pad16(2 * kRowsPerUnit);
    for (unsigned k = 0; k < nr; ++k) {
      const unsigned p = urows[u].p0 + k, i = prow[p];
      const unsigned g = gof[i];
      unsigned s0, s1;
      off_range(i, s0, s1);
      const unsigned nbo = s1 - s0, nbt = nbo + (fwd ? 1 : 0);
      rowoff[k] = (unsigned short)off;
      const unsigned hdr[4] = {i, nbt, nbo, p - gptr[g]};
      std::memcpy(base + off, hdr, 16);
      int *deps = reinterpret_cast<int *>(base + off + 16);
      for (unsigned b = 0; b < nbo; ++b) {
        const unsigned j = col[s0 + b];
        deps[b] = gof[j] == g ? (int)pos[j] : -(int)j - 1;
      }
      const size_t voff = units[u].x + off + 16 + pad16((size_t)nbo * 4);
      for (unsigned b = 0; b < nbt; ++b) {
        vsrc.push_back(b < nbo ? s0 + b : (unsigned)(nnz + i));
        vdst.push_back((unsigned)(voff / sizeof(float)) + b * 9);
      }
      off += record_bytes(i);
    }
  }
  gs.threads = kGThreads;
  gs.ring = kRing;
  gs.max_rows = max_rows;
  gs.slot_bytes = (unsigned)pad16(slot);
  gs.smem = pad16((size_t)max_rows * 3 * sizeof(float)) + (size_t)kRing * gs.slot_bytes;
  if (gs.smem * kCtasPerSm > kSmemPerSm)
    return fail(DFM2G_ERR_UNSUPPORTED, "blob schedule needs %zu B of shared memory per CTA", gs.smem);
  gs.ngroups = ng;
  gs.nvblocks = vsrc.size();
  DFM2G_TRY(gs.units.resize(units.size() + 1));
  DFM2G_TRY(gs.gunit.resize(ng + 1));
  DFM2G_TRY(gs.growptr.resize(ng + 1));
  DFM2G_TRY(gs.prow.resize(n + 1));
  DFM2G_TRY(gs.bytes.resize(total + 16));
  DFM2G_TRY(gs.vsrc.resize(vsrc.size() + 1));
  DFM2G_TRY(gs.vdst.resize(vdst.size() + 1));
  DFM2G_CUDA(cudaMemcpy(gs.units.p, units.data(), units.size() * sizeof(uint4), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(gs.gunit.p, gunit.data(), gunit.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(gs.growptr.p, gptr.data(), gptr.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(gs.prow.p, prow.data(), n * sizeof(unsigned), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(gs.bytes.p, bytes.data(), total, cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(gs.vsrc.p, vsrc.data(), vsrc.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
  DFM2G_CUDA(cudaMemcpy(gs.vdst.p, vdst.data(), vdst.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
  gs.values_ok = false;
  gs.ok = true;
  return DFM2G_OK;
}

template <typename V>
static int to_host(std::vector<V> &h, const V *d, size_t n) {
  h.resize(n);
  if (n) DFM2G_CUDA(cudaMemcpy(h.data(), d, n * sizeof(V), cudaMemcpyDeviceToHost));
  return DFM2G_OK;
}

// Builds both directions' schedules (FP32) after set_pattern0. Leaves the
// schedules disabled (and the sync-free sweeps in use) when the blobs do not
// fit the shared memory of kCtasPerSm CTAs per SM.
int group_schedules_build(dfm2g_ilu_s *p) {
  p->gs_f.ok = p->gs_b.ok = false;
  const unsigned n = p->nblk;
  if (n == 0) return DFM2G_OK;
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  std::vector<unsigned> rs, col, dia, lf, lb;
  DFM2G_TRY(to_host(rs, p->row_start.p, (size_t)n + 1));
  DFM2G_TRY(to_host(col, p->col.p, p->nnz));
  DFM2G_TRY(to_host(dia, p->dia_ind.p, n));
  DFM2G_TRY(to_host(lf, p->level_f.p, n));
  DFM2G_TRY(to_host(lb, p->level_b.p, n));
  const unsigned cap = (unsigned)ctx().num_sms * kCtasPerSm;
  const unsigned target = std::max(32u, (unsigned)((n + cap - 1) / cap));
  unsigned ng = grow_blobs(n, rs, col, target, p->group_of);
  if (ng > cap) ng = merge_blobs(n, rs, col, p->group_of, ng, cap);
  const int sf = build_direction(p->gs_f, true, n, p->nnz, ng, p->group_of, rs, col, dia, lf);
  const int sb = sf == DFM2G_OK ? build_direction(p->gs_b, false, n, p->nnz, ng, p->group_of, rs, col, dia, lb) : sf;
  if (sf != DFM2G_OK || sb != DFM2G_OK) {  // not an error: the sync-free schedule serves
    p->gs_f.ok = p->gs_b.ok = false;
    if (sf == DFM2G_ERR_CUDA || sb == DFM2G_ERR_CUDA) return DFM2G_ERR_CUDA;
  }
  return DFM2G_OK;
}

// ---- values ------------------------------------------------------------------------
__global__ void k_group_values(size_t nvb, const unsigned *__restrict__ vsrc, const unsigned *__restrict__ vdst,
                               size_t nnz, const float *__restrict__ vcrs, const float *__restrict__ vdia,
                               float *__restrict__ dst) {
  const size_t total = nvb * 9;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const size_t b = t / 9, e = t - b * 9;
    const size_t s = vsrc[b];
    dst[(size_t)vdst[b] + e] = s < nnz ? vcrs[s * 9 + e] : vdia[(s - nnz) * 9 + e];
  }
}

// Copies the FP32 factors into both schedules (after each decomposition).
int group_values_fill(dfm2g_ilu_s *p) {
  for (GroupSched *gs : {&p->gs_f, &p->gs_b}) {
    if (!gs->ok) continue;
    k_group_values<<<blocks_for(gs->nvblocks * 9, 256, ctx().num_sms * 16), 256, 0, stream()>>>(
        gs->nvblocks, gs->vsrc.p, gs->vdst.p, p->nnz, p->vcrs32.p, p->vdia32.p,
        reinterpret_cast<float *>(gs->bytes.p));
    note_launches(1);
    DFM2G_LAUNCH_CHECK();
    gs->values_ok = true;
  }
  return DFM2G_OK;
}

// ---- the sweep --------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void copy_unit(const uint4 U, const unsigned char *sched, unsigned char *dst) {
  const unsigned char *src = sched + U.x;
  for (unsigned o = threadIdx.x * 16u; o < U.y; o += blockDim.x * 16u) cp_async16(dst + o, src + o);
}

template <bool FWD>
__global__ void __launch_bounds__(kGThreads) k_sweep_groups(const uint4 *__restrict__ units,
                                                            const unsigned *__restrict__ gunit,
                                                            const unsigned *__restrict__ growptr,
                                                            const unsigned *__restrict__ prow,
                                                            const unsigned char *__restrict__ sched, const float *in,
                                                            float *out, int *err, unsigned long long timeout_ns,
                                                            const int *skip, unsigned xs_bytes, unsigned slot_bytes) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem[];
  float *xs = reinterpret_cast<float *>(smem);
  unsigned char *ring = smem + xs_bytes;
  const unsigned g = blockIdx.x, tid = threadIdx.x;
  const unsigned rb = growptr[g], nrow = growptr[g + 1] - rb;
  const unsigned u0 = gunit[g], u1 = gunit[g + 1];
#pragma unroll
  for (unsigned s = 0; s + 1 < kRing; ++s) {
    if (u0 + s < u1) copy_unit(units[u0 + s], sched, ring + s * slot_bytes);
    cp_async_commit();
  }
  for (unsigned t = tid; t < nrow * 3; t += blockDim.x) {
    const unsigned k = t / 3;
    xs[t] = in[(size_t)prow[rb + k] * 3 + (t - k * 3)];
  }
  const unsigned q = tid >> 2, r = tid & 3, lane = tid & 31;
  const unsigned gbase = lane & 28u, gmask = 0xFu << gbase;
  for (unsigned u = u0; u < u1; ++u) {
    cp_async_wait<kRing - 2>();
    __syncthreads();  // unit u staged by every thread; unit u-1 finished (its slot is free)
    {
      const unsigned un = u + kRing - 1;
      if (un < u1) copy_unit(units[un], sched, ring + ((un - u0) % kRing) * slot_bytes);
      cp_async_commit();
    }
    const unsigned char *slot = ring + ((u - u0) % kRing) * slot_bytes;
    const unsigned nr = *reinterpret_cast<const unsigned *>(slot);
    if (q < nr) {
      const unsigned short *rowoff = reinterpret_cast<const unsigned short *>(slot + 16);
      const unsigned char *rec = slot + rowoff[q];
      const uint4 h = *reinterpret_cast<const uint4 *>(rec);  // row, blocks, off-diagonal blocks, position
      const int *deps = reinterpret_cast<const int *>(rec + 16);
      const float *vals = reinterpret_cast<const float *>(rec + 16 + ((h.z * 4u + 15u) & ~15u));
      float t = 0.f;
      if (r < 3) {
        float acc = 0.f;
        for (unsigned b = 0; b < h.z; ++b) {
          const int d = deps[b];
          float x0, x1, x2;
          if (d >= 0) {
            x0 = xs[d * 3 + 0];
            x1 = xs[d * 3 + 1];
            x2 = xs[d * 3 + 2];
          } else {
            const float *px = out + (size_t)(-(d + 1)) * 3;
            x0 = wait_value(px + 0, err, timeout_ns);
            x1 = wait_value(px + 1, err, timeout_ns);
            x2 = wait_value(px + 2, err, timeout_ns);
          }
          const float *a = vals + b * 9 + r * 3;
          acc += a[0] * x0 + a[1] * x1 + a[2] * x2;
        }
        t = xs[h.w * 3 + r] - acc;
      }
      const float t0 = __shfl_sync(gmask, t, gbase + 0);
      const float t1 = __shfl_sync(gmask, t, gbase + 1);
      const float t2 = __shfl_sync(gmask, t, gbase + 2);
      if (r < 3) {
        float z;
        if (FWD) {
          const float *dv = vals + h.z * 9 + r * 3;
          z = dv[0] * t0 + dv[1] * t1 + dv[2] * t2;
        } else {
          z = r == 0 ? t0 : (r == 1 ? t1 : t2);
        }
        xs[h.w * 3 + r] = z;
        st_relaxed(out + (size_t)h.x * 3 + r, z);
      }
    }
  }
  cp_async_wait<0>();
}

int group_sweep(dfm2g_ilu_s *p, bool forward, const float *in, float *out, const int *skip) {
  GroupSched &gs = forward ? p->gs_f : p->gs_b;
  if (!gs.ok || !gs.values_ok) return fail(DFM2G_ERR_STATE, "blob schedule not ready");
  void *kernel = forward ? (void *)k_sweep_groups<true> : (void *)k_sweep_groups<false>;
  DFM2G_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gs.smem));
  const unsigned xs_bytes = (unsigned)pad16((size_t)gs.max_rows * 3 * sizeof(float));
  const unsigned nlev = forward ? p->nlev_f : p->nlev_b;
  unsigned long long timeout = kWaitTimeoutNs + 20000ull * nlev;
  int *err = p->err.p;
  const uint4 *units = gs.units.p;
  const unsigned *gunit = gs.gunit.p, *growptr = gs.growptr.p, *prow = gs.prow.p;
  const unsigned char *sched = gs.bytes.p;
  unsigned slot_bytes = gs.slot_bytes;
  void *args[] = {(void *)&units, (void *)&gunit, (void *)&growptr, (void *)&prow, (void *)&sched, (void *)&in,
                  (void *)&out, (void *)&err, (void *)&timeout, (void *)&skip, (void *)&xs_bytes,
                  (void *)&slot_bytes};
  DFM2G_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(gs.ngroups), dim3(gs.threads), args, gs.smem, stream()));
  note_launches(1);
  return DFM2G_OK;
}

}  // namespace dfm2g

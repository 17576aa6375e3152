// CPreconditionerILU<double> for 3x3 blocks on the device: SetPattern0,
// CopyValue, level-scheduled Decompose, and the forward/backward sweeps.
//
// Level sets. Forward level: 0 for a row with no column j < i, else
// 1 + max over its columns j < i; backward: the same over columns j > i. Rows of
// one level are independent in the sweep (and in the factorisation, which has
// the forward dependency structure). `order` lists rows by (level, row id);
// `level_start[l]` is the first position of level l. Everything is computed on
// the device (iterative level assignment + a stable LSD radix sort) and is
// bit-exact against a serial CPU recomputation.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "nd.cuh"
#include "rowkern.cuh"

namespace dfm2g {

// ---------------------------------------------------------------------------
// SetPattern0: sort each row's columns ascending (thread per row, insertion
// sort - rows hold a handful of entries) and find dia_ind = first col > i.
__global__ void k_sort_rows_diaind(unsigned nblk, const unsigned *__restrict__ row_start, unsigned *col,
                                   unsigned *__restrict__ dia_ind) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < nblk; i += gridDim.x * blockDim.x) {
    const unsigned s0 = row_start[i], s1 = row_start[i + 1];
    for (unsigned a = s0 + 1; a < s1; ++a) {
      const unsigned v = col[a];
      unsigned b = a;
      while (b > s0 && col[b - 1] > v) {
        col[b] = col[b - 1];
        --b;
      }
      col[b] = v;
    }
    unsigned d = s1;
    for (unsigned s = s0; s < s1; ++s)
      if (col[s] > i) {
        d = s;
        break;
      }
    dia_ind[i] = d;
  }
}

// One relaxation sweep of the level assignment. A row gets its level once all
// of its dependencies have one; a level, once written, is final, so reading a
// stale "unassigned" only postpones the row to a later sweep.
__global__ void k_level_sweep(unsigned nblk, const unsigned *__restrict__ row_start,
                              const unsigned *__restrict__ col, const unsigned *__restrict__ dia_ind,
                              int backward, int *level, unsigned *n_assigned, unsigned *max_level) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned stride = gridDim.x * blockDim.x;
  for (unsigned t0 = blockIdx.x * blockDim.x; t0 < nblk; t0 += stride) {
    const unsigned t = t0 + threadIdx.x;
    bool newly = false;
    int lv = 0;
    if (t < nblk) {
      const unsigned i = backward ? nblk - 1 - t : t;
      if (level[i] < 0) {
        const unsigned s0 = backward ? dia_ind[i] : row_start[i];
        const unsigned s1 = backward ? row_start[i + 1] : dia_ind[i];
        bool ready = true;
        for (unsigned s = s0; s < s1; ++s) {
          const int lj = ld_relaxed(level + col[s]);
          if (lj < 0) {
            ready = false;
            break;
          }
          lv = max(lv, lj + 1);
        }
        if (ready) {
          level[i] = lv;
          newly = true;
        }
      }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, newly);
    if (newly) atomicMax(max_level, (unsigned)lv);
    if (lane == 0 && bal) atomicAdd(n_assigned, (unsigned)__popc(bal));
  }
}

// ---- stable LSD radix sort of (key, value) pairs, 8-bit digits ----------------
constexpr int kRsThreads = 256;
constexpr int kRsRounds = 8;
constexpr int kRsTile = kRsThreads * kRsRounds;

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(unsigned n, const unsigned *__restrict__ keys, int shift,
                                                        unsigned *__restrict__ counts, unsigned ntiles) {
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsRounds; ++r) {
    const size_t idx = base + (size_t)r * kRsThreads + threadIdx.x;
    if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
  }
  __syncthreads();
  counts[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// In-place exclusive scan of a[0..n) by one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan_exclusive(unsigned *a, size_t n) {
  __shared__ unsigned warp_tot[32];
  __shared__ unsigned carry;
  const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (size_t base = 0; base < n; base += blockDim.x) {
    const size_t i = base + threadIdx.x;
    const unsigned v = i < n ? a[i] : 0u;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
      unsigned tw = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, tw, o);
        if (lane >= (unsigned)o) tw += y;
      }
      warp_tot[lane] = tw;
    }
    __syncthreads();
    const unsigned excl = (w ? warp_tot[w - 1] : 0u) + x - v;
    const unsigned c = carry;
    if (i < n) a[i] = c + excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = c + excl + v;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(unsigned n, const unsigned *__restrict__ kin,
                                                           const unsigned *__restrict__ vin,
                                                           unsigned *__restrict__ kout, unsigned *__restrict__ vout,
                                                           int shift, const unsigned *__restrict__ offsets,
                                                           unsigned ntiles) {
  __shared__ unsigned run[256];
  __shared__ unsigned wc[kRsThreads / 32][256];
  const unsigned tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  run[tid] = offsets[(size_t)tid * ntiles + blockIdx.x];
  const size_t base = (size_t)blockIdx.x * kRsTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kRsRounds; ++r) {
    for (unsigned k = tid; k < (kRsThreads / 32) * 256; k += kRsThreads) (&wc[0][0])[k] = 0;
    __syncthreads();
    const size_t idx = base + (size_t)r * kRsThreads + tid;
    const bool ok = idx < n;
    const unsigned key = ok ? kin[idx] : 0u, val = ok ? vin[idx] : 0u;
    const unsigned d = (key >> shift) & 255u;
    const unsigned tag = ok ? d : 0x10000u + lane;  // invalid lanes match nobody
    const unsigned peers = __match_any_sync(0xffffffffu, tag);
    const unsigned rank = __popc(peers & lt_mask);
    if (ok && rank == 0) wc[w][d] = __popc(peers);
    __syncthreads();
    {
      unsigned acc = run[tid];
#pragma unroll
      for (int q = 0; q < kRsThreads / 32; ++q) {
        const unsigned c = wc[q][tid];
        wc[q][tid] = acc;
        acc += c;
      }
      run[tid] = acc;
    }
    __syncthreads();
    if (ok) {
      const unsigned pos = wc[w][d] + rank;
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
  }
}

__global__ void k_iota(unsigned n, unsigned *a) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}

__global__ void k_level_start(unsigned n, const unsigned *__restrict__ sorted_level, unsigned nlev,
                              unsigned *__restrict__ lstart) {
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const unsigned lq = sorted_level[q];
    const unsigned lp = q ? sorted_level[q - 1] : 0xFFFFFFFFu;
    if (lq != lp)
      for (unsigned l = lp + 1; l <= lq; ++l) lstart[l] = q;  // lp+1 wraps to 0 for q == 0
    if (q == n - 1) lstart[nlev] = n;
  }
}

// Sort rows by level (stable): returns order (values) in `order`.
static int radix_sort_levels(unsigned n, const unsigned *level, unsigned max_key, unsigned *order,
                             DevBuf<unsigned> &scratch_sorted_keys) {
  const unsigned ntiles = (n + kRsTile - 1) / kRsTile;
  DevBuf<unsigned> k0, k1, v0, v1, counts;
  DFM2G_TRY(k0.resize(n));
  DFM2G_TRY(k1.resize(n));
  DFM2G_TRY(v0.resize(n));
  DFM2G_TRY(v1.resize(n));
  DFM2G_TRY(counts.resize((size_t)256 * ntiles));
  DFM2G_CUDA(cudaMemcpyAsync(k0.p, level, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, stream()));
  k_iota<<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(n, v0.p);
  unsigned *ka = k0.p, *kb = k1.p, *va = v0.p, *vb = v1.p;
  int shift = 0;
  do {
    k_rs_hist<<<ntiles, kRsThreads, 0, stream()>>>(n, ka, shift, counts.p, ntiles);
    k_scan_exclusive<<<1, 1024, 0, stream()>>>(counts.p, (size_t)256 * ntiles);
    k_rs_scatter<<<ntiles, kRsThreads, 0, stream()>>>(n, ka, va, kb, vb, shift, counts.p, ntiles);
    DFM2G_LAUNCH_CHECK();
    std::swap(ka, kb);
    std::swap(va, vb);
    shift += 8;
  } while (shift < 32 && (max_key >> shift) != 0);
  DFM2G_CUDA(cudaMemcpyAsync(order, va, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, stream()));
  DFM2G_TRY(scratch_sorted_keys.resize(n));
  DFM2G_CUDA(cudaMemcpyAsync(scratch_sorted_keys.p, ka, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  return DFM2G_OK;
}

__global__ void k_sweep_meta(unsigned n, const unsigned *__restrict__ order, const unsigned *__restrict__ row_start,
                             const unsigned *__restrict__ dia_ind, int backward, uint4 *__restrict__ meta,
                             unsigned *__restrict__ pos);

static int compute_levels(dfm2g_ilu_s *p, bool backward) {
  const unsigned n = p->nblk;
  DevBuf<unsigned> &level = backward ? p->level_b : p->level_f;
  DevBuf<unsigned> &order = backward ? p->order_b : p->order_f;
  DevBuf<unsigned> &lstart = backward ? p->lstart_b : p->lstart_f;
  DFM2G_TRY(level.resize(n));
  DFM2G_TRY(order.resize(n));
  DevBuf<unsigned> counters;  // [0] assigned, [1] max level
  DFM2G_TRY(counters.resize(2));
  if (n) DFM2G_CUDA(cudaMemsetAsync(level.p, 0xFF, sizeof(unsigned) * n, stream()));
  DFM2G_CUDA(cudaMemsetAsync(counters.p, 0, sizeof(unsigned) * 2, stream()));
  unsigned h[2] = {0, 0};
  unsigned sweeps = 0;
  const unsigned blocks = blocks_for(n, 256, ctx().num_sms * 8);
  while (h[0] < n) {
    const unsigned before = h[0];
    for (int k = 0; k < 8; ++k)
      k_level_sweep<<<blocks, 256, 0, stream()>>>(n, p->row_start.p, p->col.p, p->dia_ind.p, backward ? 1 : 0,
                                                  (int *)level.p, counters.p, counters.p + 1);
    DFM2G_LAUNCH_CHECK();
    DFM2G_CUDA(cudaMemcpyAsync(h, counters.p, sizeof(h), cudaMemcpyDeviceToHost, stream()));
    DFM2G_CUDA(cudaStreamSynchronize(stream()));
    sweeps += 8;
    if (h[0] == before || sweeps > n + 16)
      return fail(DFM2G_ERR_PATTERN, "level sets: no progress (cyclic dependency?)");
  }
  const unsigned nlev = n ? h[1] + 1 : 0;
  DFM2G_TRY(lstart.resize(nlev + 1));
  std::vector<unsigned> &hl = backward ? p->h_lstart_b : p->h_lstart_f;
  if (n) {
    DevBuf<unsigned> sorted_keys;
    DFM2G_TRY(radix_sort_levels(n, level.p, h[1], order.p, sorted_keys));
    k_level_start<<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(n, sorted_keys.p, nlev, lstart.p);
    DFM2G_LAUNCH_CHECK();
    hl.resize(nlev + 1);
    DFM2G_CUDA(cudaMemcpyAsync(hl.data(), lstart.p, sizeof(unsigned) * (nlev + 1), cudaMemcpyDeviceToHost,
                               stream()));
    DFM2G_CUDA(cudaStreamSynchronize(stream()));
  } else {
    hl.assign(1, 0);
  }
  DevBuf<uint4> &meta = backward ? p->meta_b : p->meta_f;
  DevBuf<unsigned> &pos = backward ? p->pos_b : p->pos_f;
  DFM2G_TRY(meta.resize((size_t)n + 1));
  DFM2G_TRY(pos.resize((size_t)n + 1));
  if (n) {
    k_sweep_meta<<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(n, order.p, p->row_start.p, p->dia_ind.p,
                                                                              backward ? 1 : 0, meta.p, pos.p);
    DFM2G_LAUNCH_CHECK();
  }
  (backward ? p->nlev_b : p->nlev_f) = nlev;
  return DFM2G_OK;
}

// ---------------------------------------------------------------------------
// CopyValue: every matrix block goes to the ILU slot of the same column (binary
// search in the sorted ILU row); blocks without a slot are dropped.
template <unsigned BB>
__global__ void k_ilu_copy(unsigned nblk, const unsigned *__restrict__ m_row_start,
                           const unsigned *__restrict__ m_col, const double *__restrict__ m_vcrs,
                           const unsigned *__restrict__ p_row_start, const unsigned *__restrict__ p_col,
                           double *__restrict__ p_vcrs) {
  const unsigned lane = threadIdx.x & 31, nwarp = (gridDim.x * blockDim.x) >> 5;
  for (unsigned i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nblk; i += nwarp) {
    const unsigned q0 = p_row_start[i], q1 = p_row_start[i + 1];
    for (unsigned s = m_row_start[i] + lane; s < m_row_start[i + 1]; s += 32) {
      const unsigned j = m_col[s];
      unsigned lo = q0, hi = q1;
      while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if (p_col[mid] < j) lo = mid + 1; else hi = mid;
      }
      if (lo < q1 && p_col[lo] == j) {
#pragma unroll
        for (unsigned k = 0; k < BB; ++k) p_vcrs[(size_t)lo * BB + k] = m_vcrs[(size_t)s * BB + k];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Decompose, one level at a time, one warp per row. For each k < i of row i
// (ascending, sequential): A_ik is read fresh (earlier k's may have updated
// it), and the lanes split the (j in U(k)) x (3x3 entry) updates
// A_ij -= A_ik A_kj, each touching a distinct entry. Then D_i is inverted by
// the cofactor formula (|det| <= 1e-30 counts a singular pivot and leaves it),
// then U_ij <- D_i^-1 U_ij (one lane per block).
__global__ void __launch_bounds__(256) k_ilu_factor_level(const unsigned *__restrict__ rows, unsigned nrows,
                                                          const unsigned *__restrict__ row_start,
                                                          const unsigned *__restrict__ col,
                                                          const unsigned *__restrict__ dia_ind, double *vcrs,
                                                          double *vdia, int *nsing) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= nrows) return;
  const unsigned i = rows[w];
  const unsigned s0 = row_start[i], s1 = row_start[i + 1], sd = dia_ind[i];
  for (unsigned sk = s0; sk < sd; ++sk) {
    const unsigned k = col[sk];
    double aik[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) aik[q] = vcrs[(size_t)sk * 9 + q];
    const unsigned u0 = dia_ind[k], u1 = row_start[k + 1];
    const unsigned ntask = (u1 - u0) * 9;
    for (unsigned t = lane; t < ntask; t += 32) {
      const unsigned uu = t / 9u, e = t - uu * 9u, r = e / 3u, c = e - r * 3u;
      const unsigned sj = u0 + uu;
      const unsigned j = col[sj];
      double *dst;
      if (j == i) {
        dst = vdia + (size_t)i * 9;
      } else {
        unsigned lo = s0, hi = s1;
        while (lo < hi) {
          const unsigned mid = (lo + hi) >> 1;
          if (col[mid] < j) lo = mid + 1; else hi = mid;
        }
        if (lo >= s1 || col[lo] != j) continue;
        dst = vcrs + (size_t)lo * 9;
      }
      const double *akj = vcrs + (size_t)sj * 9;
      dst[e] -= aik[r * 3 + 0] * akj[0 * 3 + c] + aik[r * 3 + 1] * akj[1 * 3 + c] + aik[r * 3 + 2] * akj[2 * 3 + c];
    }
    __syncwarp();
  }
  double d[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) d[q] = vdia[(size_t)i * 9 + q];
  const double det = d[0] * (d[4] * d[8] - d[5] * d[7]) - d[1] * (d[3] * d[8] - d[5] * d[6]) +
                     d[2] * (d[3] * d[7] - d[4] * d[6]);
  double v[9];
  if (fabs(det) > 1.0e-30) {
    const double s = 1.0 / det;
    v[0] = s * (d[4] * d[8] - d[5] * d[7]);
    v[1] = s * (d[2] * d[7] - d[1] * d[8]);
    v[2] = s * (d[1] * d[5] - d[2] * d[4]);
    v[3] = s * (d[5] * d[6] - d[3] * d[8]);
    v[4] = s * (d[0] * d[8] - d[2] * d[6]);
    v[5] = s * (d[2] * d[3] - d[0] * d[5]);
    v[6] = s * (d[3] * d[7] - d[4] * d[6]);
    v[7] = s * (d[1] * d[6] - d[0] * d[7]);
    v[8] = s * (d[0] * d[4] - d[1] * d[3]);
  } else {
#pragma unroll
    for (int q = 0; q < 9; ++q) v[q] = d[q];
    if (lane == 0) atomicAdd(nsing, 1);
  }
  __syncwarp();
  if (lane < 9) vdia[(size_t)i * 9 + lane] = v[lane];
  for (unsigned s = sd + lane; s < s1; s += 32) {
    double *u = vcrs + (size_t)s * 9;
    double t[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) t[q] = u[q];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        u[r * 3 + c] = v[r * 3 + 0] * t[0 * 3 + c] + v[r * 3 + 1] * t[1 * 3 + c] + v[r * 3 + 2] * t[2 * 3 + c];
  }
}

// The same for 1x1 and 2x2 blocks, in the reference's arithmetic
// (ls_ilu_block_sparse.cpp:168-285): every product and sum is rounded on its
// own (no fused multiply-add), in the reference's order, so the factors equal
// the reference's bit for bit. A_ij -= A_ik A_kj; the pivot is inverted when
// |d| (1x1) or |det| (2x2) exceeds 1e-30, else counted and left; then
// U_ij <- D_i^-1 U_ij.
template <int B>
__global__ void __launch_bounds__(256) k_ilu_factor_level_nd(const unsigned *__restrict__ rows, unsigned nrows,
                                                             const unsigned *__restrict__ row_start,
                                                             const unsigned *__restrict__ col,
                                                             const unsigned *__restrict__ dia_ind, double *vcrs,
                                                             double *vdia, int *nsing) {
  constexpr unsigned BB = B * B;
  const unsigned lane = threadIdx.x & 31;
  const unsigned w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= nrows) return;
  const unsigned i = rows[w];
  const unsigned s0 = row_start[i], s1 = row_start[i + 1], sd = dia_ind[i];
  for (unsigned sk = s0; sk < sd; ++sk) {
    const unsigned k = col[sk];
    double aik[BB];
#pragma unroll
    for (unsigned q = 0; q < BB; ++q) aik[q] = vcrs[(size_t)sk * BB + q];
    const unsigned u0 = dia_ind[k], u1 = row_start[k + 1];
    const unsigned ntask = (u1 - u0) * BB;
    for (unsigned t = lane; t < ntask; t += 32) {
      const unsigned uu = t / BB, e = t - uu * BB, r = e / B, c = e - r * B;
      const unsigned sj = u0 + uu;
      const unsigned j = col[sj];
      double *dst;
      if (j == i) {
        dst = vdia + (size_t)i * BB;
      } else {
        unsigned lo = s0, hi = s1;
        while (lo < hi) {
          const unsigned mid = (lo + hi) >> 1;
          if (col[mid] < j) lo = mid + 1; else hi = mid;
        }
        if (lo >= s1 || col[lo] != j) continue;
        dst = vcrs + (size_t)lo * BB;
      }
      const double *akj = vcrs + (size_t)sj * BB;
      double sum = __dmul_rn(aik[r * B], akj[c]);
#pragma unroll
      for (int q = 1; q < B; ++q) sum = __dadd_rn(sum, __dmul_rn(aik[r * B + q], akj[q * B + c]));
      dst[e] = __dsub_rn(dst[e], sum);
    }
    __syncwarp();
  }
  double d[BB], v[BB];
#pragma unroll
  for (unsigned q = 0; q < BB; ++q) v[q] = d[q] = vdia[(size_t)i * BB + q];  // a singular pivot stays as it is
  bool singular;
  if constexpr (B == 1) {
    singular = !(fabs(d[0]) > 1.0e-30);
    if (!singular) v[0] = 1.0 / d[0];
  } else {
    const double det = __dsub_rn(__dmul_rn(d[0], d[3]), __dmul_rn(d[1], d[2]));
    singular = !(fabs(det) > 1.0e-30);
    if (!singular) {
      const double inv_det = 1.0 / det;
      v[0] = __dmul_rn(inv_det, d[3]);
      v[1] = __dmul_rn(-inv_det, d[1]);
      v[2] = __dmul_rn(-inv_det, d[2]);
      v[3] = __dmul_rn(inv_det, d[0]);
    }
  }
  if (singular && lane == 0) atomicAdd(nsing, 1);
  __syncwarp();
  if (lane < BB) {
    double o = v[0];
#pragma unroll
    for (unsigned q = 1; q < BB; ++q)
      if (q == lane) o = v[q];
    vdia[(size_t)i * BB + lane] = o;
  }
  for (unsigned s = sd + lane; s < s1; s += 32) {
    double *u = vcrs + (size_t)s * BB;
    if constexpr (B == 1) {
      u[0] = __dmul_rn(u[0], v[0]);
    } else {
      const double t0 = u[0], t1 = u[1], t2 = u[2], t3 = u[3];
      u[0] = __dadd_rn(__dmul_rn(v[0], t0), __dmul_rn(v[1], t2));
      u[1] = __dadd_rn(__dmul_rn(v[0], t1), __dmul_rn(v[1], t3));
      u[2] = __dadd_rn(__dmul_rn(v[2], t0), __dmul_rn(v[3], t2));
      u[3] = __dadd_rn(__dmul_rn(v[2], t1), __dmul_rn(v[3], t3));
    }
  }
}

// ---------------------------------------------------------------------------
// Sweeps. Forward: out_i = D_i^-1 (in_i - sum_{j<i} L_ij out_j). Backward:
// out_i = in_i - sum_{j>i} U'_ij out_j. One warp per row in the lane layout of
// rowkern.cuh. Rows are visited in level order through per-position
// metadata meta[q] = {row, first block, end block} (one 16-byte load), so a
// warp can request its next row's blocks and right-hand side before it starts
// waiting for the current row's dependencies.
__global__ void k_sweep_meta(unsigned n, const unsigned *__restrict__ order, const unsigned *__restrict__ row_start,
                             const unsigned *__restrict__ dia_ind, int backward, uint4 *__restrict__ meta,
                             unsigned *__restrict__ pos) {
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const unsigned i = order[q];
    const unsigned s0 = backward ? dia_ind[i] : row_start[i];
    const unsigned s1 = backward ? row_start[i + 1] : dia_ind[i];
    meta[q] = make_uint4(i, s0, s1, 0u);
    pos[i] = q;
  }
}

// R rounds (3R blocks of one triangle) in registers: 4 for ILU(0) patterns,
// 8 for fill-in patterns whose longest triangle row has 13..24 blocks.
template <typename T, unsigned R = 4>
struct SweepRow {
  static constexpr unsigned kRounds = R;
  RowFrag<T, kRounds> f;
  unsigned i, s0, s1;
  T in[3];  // lanes 0..2: the row's right-hand side
  T d[3];   // lanes 0..2: row `lane` of D_i^-1 (forward only)
};

template <typename T, bool FWD, unsigned NR>
__device__ __forceinline__ void sweep_load(SweepRow<T, NR> &R, const RowLane &L, unsigned lane, uint4 m,
                                           const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                           const T *__restrict__ vdia, const T *in) {
  R.i = m.x;
  R.s0 = m.y;
  R.s1 = m.z;
  row_load(R.f, L, m.y, m.z, col, vcrs, ~0u, (const T *)nullptr);
  if (lane < 3) {
#pragma unroll
    for (int k = 0; k < 3; ++k) R.in[k] = in[(size_t)m.x * 3 + k];
    if (FWD) {
#pragma unroll
      for (int k = 0; k < 3; ++k) R.d[k] = vdia[(size_t)m.x * 9 + lane * 3 + k];
    }
  }
}

template <typename T, bool FWD, bool WAIT, unsigned NR>
__device__ __forceinline__ void sweep_finish(const SweepRow<T, NR> &R, const RowLane &L, unsigned lane,
                                             const unsigned *__restrict__ col, const T *__restrict__ vcrs, T *out,
                                             int *err, unsigned long long timeout_ns) {
  T acc;
  if (R.f.nb <= 3 * NR)
    acc = WAIT ? row_dot_wait(R.f, L, out, err, timeout_ns) : row_dot(R.f, L, out);
  else
    acc = WAIT ? row_dot_wait_long(L, R.s0, R.s1, col, vcrs, out, err, timeout_ns)
               : row_dot_long(L, R.s0, R.s1, col, vcrs, ~0u, (const T *)nullptr, out);
  T s[3];
  row_reduce(acc, s);
  if (lane < 3) {
    const T t0 = R.in[0] - s[0], t1 = R.in[1] - s[1], t2 = R.in[2] - s[2];
    T z;
    if (FWD)
      z = R.d[0] * t0 + R.d[1] * t1 + R.d[2] * t2;
    else
      z = lane == 0 ? t0 : (lane == 1 ? t1 : t2);
    if (WAIT)
      st_relaxed(out + (size_t)R.i * 3 + lane, z);
    else
      out[(size_t)R.i * 3 + lane] = z;
  }
}

// One level: rows meta[0..nrows) are independent; `out` holds the input for
// rows not yet swept (in place), the results of earlier levels otherwise.
template <typename T, bool FWD>
__global__ void __launch_bounds__(256) k_sweep_level(const uint4 *__restrict__ meta, unsigned nrows,
                                                     const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                                     const T *__restrict__ vdia, T *out, const int *skip) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= nrows || (skip && *skip)) return;
  const RowLane L(lane);
  SweepRow<T> R;
  sweep_load<T, FWD>(R, L, lane, meta[w], col, vcrs, vdia, out);
  sweep_finish<T, FWD, false>(R, L, lane, col, vcrs, out, nullptr, 0);
}

// Sync-free sweep: one persistent, co-resident (cooperative) grid; warp w
// takes positions w, w+W, ... of the level order, and waits (bounded) on each
// needed out_j until it is no longer the pending marker. Every row depends only
// on rows earlier in the order and each warp walks its positions in order, so
// the earliest unfinished position can always proceed. Pipelined: the next
// position's row is loaded before the current one's wait, and the metadata
// of the one after that before the current row is finished.
template <typename T, bool FWD, unsigned NR>
__global__ void __launch_bounds__(256) k_sweep_syncfree(unsigned n, const uint4 *__restrict__ meta,
                                                        const unsigned *__restrict__ col,
                                                        const T *__restrict__ vcrs, const T *__restrict__ vdia,
                                                        const T *in, T *out, int *err,
                                                        unsigned long long timeout_ns, const int *skip) {
  if (skip && *skip) return;
  const unsigned lane = threadIdx.x & 31;
  const RowLane L(lane);
  const unsigned nwarp = (gridDim.x * blockDim.x) >> 5;
  unsigned q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= n) return;
  SweepRow<T, NR> cur, nxt;
  sweep_load<T, FWD>(cur, L, lane, meta[q], col, vcrs, vdia, in);
  uint4 m1 = (q + nwarp < n) ? meta[q + nwarp] : make_uint4(0u, 0u, 0u, 0u);
  for (;;) {
    const unsigned q1 = q + nwarp;
    if (q1 < n) sweep_load<T, FWD>(nxt, L, lane, m1, col, vcrs, vdia, in);
    const unsigned q2 = q1 + nwarp;
    const uint4 m2 = (q2 < n) ? meta[q2] : make_uint4(0u, 0u, 0u, 0u);
    sweep_finish<T, FWD, true>(cur, L, lane, col, vcrs, out, err, timeout_ns);
    if (q1 >= n) break;
    q = q1;
    cur = nxt;
    m1 = m2;
  }
}

// Sweeps for 1x1 and 2x2 blocks (nd.cuh): one warp per row, the lanes over
// the row's triangle blocks. The level kernel works in place on `out` (rows of
// one level are independent); the sync-free kernel is the same co-resident
// grid as k_sweep_syncfree, waiting (bounded) on each needed out_j.
template <typename T, bool FWD, int B>
__device__ __forceinline__ T nd_sweep_value(const uint4 m, unsigned lane, const T t[B], const T *__restrict__ vdia) {
  if constexpr (FWD) {
    const T *d = vdia + (size_t)m.x * (B * B) + (size_t)lane * B;
    T z = d[0] * t[0];
#pragma unroll
    for (int c = 1; c < B; ++c) z += d[c] * t[c];
    return z;
  } else {
    return nd_pick<T, B>(t, lane);
  }
}

template <typename T, bool FWD, int B>
__global__ void __launch_bounds__(256) k_sweep_level_nd(const uint4 *__restrict__ meta, unsigned nrows,
                                                        const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                                        const T *__restrict__ vdia, T *out, const int *skip) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= nrows || (skip && *skip)) return;
  const uint4 m = meta[w];
  T t[B];
#pragma unroll
  for (int r = 0; r < B; ++r) t[r] = out[(size_t)m.x * B + r];
  T acc[B];
  nd_row_sum<T, B, false>(lane, m.y, m.z, col, vcrs, out, acc, nullptr, 0);
#pragma unroll
  for (int r = 0; r < B; ++r) t[r] -= acc[r];
  __syncwarp();  // every lane has read row m.x's input before it is overwritten
  if (lane < (unsigned)B) out[(size_t)m.x * B + lane] = nd_sweep_value<T, FWD, B>(m, lane, t, vdia);
}

// One row of the pipelined sync-free sweep, held in registers: lane l keeps
// block s0 + l of the row's triangle (column and values), lanes < B the row's
// right-hand side entry and, forward, row `lane` of D_i^-1. Blocks past the
// first 32 of a long row are read when the row finishes.
template <typename T, int B>
struct NdSweepRow {
  unsigned i, s0, s1, j;  // j = ~0u: no block for this lane
  T a[B * B];
  T in;
  T d[B];
};

template <typename T, bool FWD, int B>
__device__ __forceinline__ void nd_sweep_load(NdSweepRow<T, B> &R, unsigned lane, uint4 m,
                                              const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                              const T *__restrict__ vdia, const T *in) {
  R.i = m.x;
  R.s0 = m.y;
  R.s1 = m.z;
  const unsigned s = m.y + lane;
  R.j = ~0u;
  if (s < m.z) {
    R.j = col[s];
#pragma unroll
    for (int q = 0; q < B * B; ++q) R.a[q] = vcrs[(size_t)s * (B * B) + q];
  }
  if (lane < (unsigned)B) {
    R.in = in[(size_t)m.x * B + lane];
    if constexpr (FWD) {
#pragma unroll
      for (int c = 0; c < B; ++c) R.d[c] = vdia[(size_t)m.x * (B * B) + lane * B + c];
    }
  }
}

template <typename T, bool FWD, int B>
__device__ __forceinline__ void nd_sweep_finish(const NdSweepRow<T, B> &R, unsigned lane,
                                                const unsigned *__restrict__ col, const T *__restrict__ vcrs, T *out,
                                                int *err, unsigned long long timeout_ns) {
  T acc[B];
#pragma unroll
  for (int r = 0; r < B; ++r) acc[r] = T(0);
  if (R.j != ~0u) {
    T xj[B];
#pragma unroll
    for (int c = 0; c < B; ++c) xj[c] = wait_value(out + (size_t)R.j * B + c, err, timeout_ns);
#pragma unroll
    for (int r = 0; r < B; ++r) {
      T t = R.a[r * B] * xj[0];
#pragma unroll
      for (int c = 1; c < B; ++c) t += R.a[r * B + c] * xj[c];
      acc[r] += t;
    }
  }
  if (R.s1 > R.s0 + 32) nd_row_partial<T, B, true>(lane, R.s0 + 32, R.s1, col, vcrs, out, acc, err, timeout_ns);
#pragma unroll
  for (int r = 0; r < B; ++r) acc[r] = warp_sum(acc[r]);
  if (lane < (unsigned)B) {
    const T t = R.in - nd_pick<T, B>(acc, lane);  // this lane's entry of in_i - sum
    T z;
    if constexpr (FWD) {
      // z = row `lane` of D_i^-1 times (in_i - sum): gather the other entries from lanes 0..B-1
      z = T(0);
#pragma unroll
      for (int c = 0; c < B; ++c) z += R.d[c] * __shfl_sync((1u << B) - 1u, t, c);
    } else {
      z = t;
    }
    st_relaxed(out + (size_t)R.i * B + lane, z);
  }
}

// Sync-free sweep for 1x1 and 2x2 blocks: the co-resident grid of
// k_sweep_syncfree, warp w taking positions w, w + W, ... of the level order.
// Pipelined: the next position's row is loaded before the current row waits
// for its dependencies, and the metadata of the one after that before the
// current row is finished.
template <typename T, bool FWD, int B>
__global__ void __launch_bounds__(256) k_sweep_syncfree_nd(unsigned n, const uint4 *__restrict__ meta,
                                                           const unsigned *__restrict__ col,
                                                           const T *__restrict__ vcrs, const T *__restrict__ vdia,
                                                           const T *in, T *out, int *err,
                                                           unsigned long long timeout_ns, const int *skip) {
  if (skip && *skip) return;
  const unsigned lane = threadIdx.x & 31;
  const unsigned nwarp = (gridDim.x * blockDim.x) >> 5;
  unsigned q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= n) return;
  NdSweepRow<T, B> cur, nxt;
  nd_sweep_load<T, FWD, B>(cur, lane, meta[q], col, vcrs, vdia, in);
  uint4 m1 = (q + nwarp < n) ? meta[q + nwarp] : make_uint4(0u, 0u, 0u, 0u);
  for (;;) {
    const unsigned q1 = q + nwarp;
    if (q1 < n) nd_sweep_load<T, FWD, B>(nxt, lane, m1, col, vcrs, vdia, in);
    const unsigned q2 = q1 + nwarp;
    const uint4 m2 = (q2 < n) ? meta[q2] : make_uint4(0u, 0u, 0u, 0u);
    nd_sweep_finish<T, FWD, B>(cur, lane, col, vcrs, out, err, timeout_ns);
    if (q1 >= n) break;
    q = q1;
    cur = nxt;
    m1 = m2;
  }
}

template <typename T>
__global__ void k_copy_guarded(size_t n, const T *__restrict__ in, T *__restrict__ out, const int *skip) {
  if (skip && *skip) return;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

// CTAs per SM of the 1x1 / 2x2 sync-free sweep. Their rows are cheap, so
// every resident warp mostly polls, and past 32 warps per SM the polls slow
// the handoff between levels. Measured on GB300 at 1,081,665 scalar rows
// (321 levels), forward / backward ms: FP32 1.14 / 1.02 at the 6-8 CTAs that
// fit, 0.76 / 0.68 at 4, 0.86 / 0.74 at 3; FP64 1.45 / 2.03, 1.28 / 1.30,
// 1.27 / 1.28. (The 3x3 sweep is register-limited to 4 CTAs per SM, and
// fewer are slower there.)
constexpr unsigned kNdSweepCtasPerSm = 4;

template <typename T>
static int coop_blocks(const void *kernel, int *cache) {
  if (*cache > 0) return DFM2G_OK;
  int per_sm = 0;
  DFM2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0));
  if (per_sm <= 0) return fail(DFM2G_ERR_CUDA, "sweep kernel cannot be resident");
  *cache = per_sm * ctx().num_sms;
  return DFM2G_OK;
}

template <typename T, int B>
static int nd_sweep_impl(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia,
                         const int *skip, bool prefilled, bool may_alloc) {
  int &ran = p->last_sched[sizeof(T) == 8 ? 1 : 0][forward ? 0 : 1];
  const unsigned n = p->nblk;
  const uint4 *meta = forward ? p->meta_f.p : p->meta_b.p;
  if (p->sweep_mode == DFM2G_SWEEP_LEVELS) {
    if (in != out) {
      k_copy_guarded<T><<<blocks_for((size_t)n * B, 256, ctx().num_sms * 4), 256, 0, stream()>>>((size_t)n * B, in,
                                                                                                 out, skip);
      DFM2G_LAUNCH_CHECK();
    }
    const std::vector<unsigned> &ls = forward ? p->h_lstart_f : p->h_lstart_b;
    for (size_t l = 0; l + 1 < ls.size(); ++l) {
      const unsigned nrows = ls[l + 1] - ls[l];
      const unsigned blocks = blocks_for((size_t)nrows * 32, 256);
      if (forward)
        k_sweep_level_nd<T, true, B><<<blocks, 256, 0, stream()>>>(meta + ls[l], nrows, p->col.p, vcrs, vdia, out,
                                                                  skip);
      else
        k_sweep_level_nd<T, false, B><<<blocks, 256, 0, stream()>>>(meta + ls[l], nrows, p->col.p, vcrs, vdia, out,
                                                                   skip);
    }
    note_launches((unsigned)(ls.size() - 1) + (in != out ? 1u : 0u));
    DFM2G_LAUNCH_CHECK();
    ran = DFM2G_SWEEP_LEVELS;
    return DFM2G_OK;
  }
  if ((const void *)in == (const void *)out) return fail(DFM2G_ERR_ARG, "sync-free sweep needs in != out");
  if (!prefilled) DFM2G_CUDA(cudaMemsetAsync(out, 0xFF, sizeof(T) * n * B, stream()));
  if (p->sweep_mode == DFM2G_SWEEP_CHAINS || p->sweep_mode == DFM2G_SWEEP_AUTO) {
    const unsigned nlev_c = forward ? p->nlev_f : p->nlev_b;
    bool usable = false;
    DFM2G_TRY(chain_sweep<T>(p, forward, in, out, vcrs, vdia, skip, kWaitTimeoutNs + 20000ull * nlev_c, may_alloc,
                             &usable));
    if (usable) {
      ran = DFM2G_SWEEP_CHAINS;
      return DFM2G_OK;
    }  // else (records too long for the ring): the sync-free schedule below
  }
  void *kernel = forward ? (void *)k_sweep_syncfree_nd<T, true, B> : (void *)k_sweep_syncfree_nd<T, false, B>;
  int *cache = &p->coop_cache[sizeof(T) == 8 ? 1 : 0][forward ? 1 : 0][0];
  DFM2G_TRY(coop_blocks<T>(kernel, cache));
  const unsigned want = blocks_for((size_t)n * 32, 256);
  const unsigned blocks =
      std::min<unsigned>(std::min<unsigned>(want, (unsigned)*cache), kNdSweepCtasPerSm * (unsigned)ctx().num_sms);
  const unsigned nlev = forward ? p->nlev_f : p->nlev_b;
  unsigned long long timeout = kWaitTimeoutNs + 20000ull * nlev;
  int *err = p->err.p;
  void *args[] = {(void *)&n, (void *)&meta, (void *)&p->col.p, (void *)&vcrs, (void *)&vdia, (void *)&in,
                  (void *)&out, (void *)&err, (void *)&timeout, (void *)&skip};
  DFM2G_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(blocks), dim3(256), args, 0, stream()));
  note_launches(1);
  ran = DFM2G_SWEEP_SYNCFREE;
  return DFM2G_OK;
}

template <typename T>
static int sweep_impl(dfm2g_ilu_s *p, bool forward, const T *in, T *out, const T *vcrs, const T *vdia,
                      const int *skip, bool prefilled, bool may_alloc = true) {
  const unsigned n = p->nblk;
  if (n == 0) return DFM2G_OK;
  if (p->ndim == 1) return nd_sweep_impl<T, 1>(p, forward, in, out, vcrs, vdia, skip, prefilled, may_alloc);
  if (p->ndim == 2) return nd_sweep_impl<T, 2>(p, forward, in, out, vcrs, vdia, skip, prefilled, may_alloc);
  int &ran = p->last_sched[sizeof(T) == 8 ? 1 : 0][forward ? 0 : 1];
  if (p->sweep_mode == DFM2G_SWEEP_LEVELS) {
    // levels in order; rows of one level are independent (in == out allowed)
    if (in != out) {
      k_copy_guarded<T><<<blocks_for((size_t)n * 3, 256, ctx().num_sms * 4), 256, 0, stream()>>>((size_t)n * 3, in,
                                                                                                 out, skip);
      DFM2G_LAUNCH_CHECK();
    }
    const std::vector<unsigned> &ls = forward ? p->h_lstart_f : p->h_lstart_b;
    const uint4 *meta = forward ? p->meta_f.p : p->meta_b.p;
    for (size_t l = 0; l + 1 < ls.size(); ++l) {
      const unsigned nrows = ls[l + 1] - ls[l];
      const unsigned blocks = blocks_for((size_t)nrows * 32, 256);
      if (forward)
        k_sweep_level<T, true><<<blocks, 256, 0, stream()>>>(meta + ls[l], nrows, p->col.p, vcrs, vdia, out, skip);
      else
        k_sweep_level<T, false><<<blocks, 256, 0, stream()>>>(meta + ls[l], nrows, p->col.p, vcrs, vdia, out, skip);
    }
    note_launches((unsigned)(ls.size() - 1) + (in != out ? 1u : 0u));
    DFM2G_LAUNCH_CHECK();
    ran = DFM2G_SWEEP_LEVELS;
    return DFM2G_OK;
  }
  if ((const void *)in == (const void *)out) return fail(DFM2G_ERR_ARG, "sync-free sweep needs in != out");
  if (p->sweep_mode == DFM2G_SWEEP_CLUSTER) {
    bool usable = false;
    DFM2G_TRY(cluster_sweep<T>(p, forward, in, out, vcrs, vdia, skip, &usable));
    if (usable) {
      ran = DFM2G_SWEEP_CLUSTER;
      return DFM2G_OK;
    }  // else (the vector exceeds shared memory): the automatic choice below
  }
  if (p->sweep_mode == DFM2G_SWEEP_BLOCK) {
    const unsigned nlev = forward ? p->nlev_f : p->nlev_b;
    bool usable = false;
    DFM2G_TRY(stream_sweep<T>(p, forward, in, out, vcrs, vdia, skip, kWaitTimeoutNs + 20000ull * nlev, may_alloc,
                              &usable));
    if (usable) {
      ran = DFM2G_SWEEP_BLOCK;
      return DFM2G_OK;
    }  // else (a row too long for a unit, or not built): the sync-free schedule below
  }
  if (p->sweep_mode == DFM2G_SWEEP_PARTS && p->parts_ok) {
    if (!prefilled) DFM2G_CUDA(cudaMemsetAsync(out, 0xFF, sizeof(T) * n * 3, stream()));
    const unsigned nlev = forward ? p->nlev_f : p->nlev_b;
    ran = DFM2G_SWEEP_PARTS;
    return part_sweep<T>(p, forward, in, out, vcrs, vdia, skip, kWaitTimeoutNs + 20000ull * nlev);
  }
  // sync-free, tile, chain and blob schedules: `out` is filled with the pending marker
  if (!prefilled) DFM2G_CUDA(cudaMemsetAsync(out, 0xFF, sizeof(T) * n * 3, stream()));
  const bool auto_pick = p->sweep_mode == DFM2G_SWEEP_AUTO || p->sweep_mode == DFM2G_SWEEP_CLUSTER;
  if (p->sweep_mode == DFM2G_SWEEP_TILES || auto_pick) {
    const unsigned nlev = forward ? p->nlev_f : p->nlev_b;
    bool usable = false;
    DFM2G_TRY(tile_sweep<T>(p, forward, in, out, vcrs, vdia, skip, kWaitTimeoutNs + 20000ull * nlev, may_alloc,
                            auto_pick, &usable));
    if (usable) {
      ran = DFM2G_SWEEP_TILES;
      return DFM2G_OK;
    }  // else (rows too long for the tiles, not built, or not picked): the chains below
  }
  if (p->sweep_mode == DFM2G_SWEEP_CHAINS || p->sweep_mode == DFM2G_SWEEP_TILES || auto_pick) {
    const unsigned nlev = forward ? p->nlev_f : p->nlev_b;
    bool usable = false;
    DFM2G_TRY(chain_sweep<T>(p, forward, in, out, vcrs, vdia, skip, kWaitTimeoutNs + 20000ull * nlev, may_alloc,
                             &usable));
    if (usable) {
      ran = DFM2G_SWEEP_CHAINS;
      return DFM2G_OK;
    }  // else (records too long for the ring): the sync-free schedule below
  }
  if constexpr (sizeof(T) == 4) {
    const GroupSched &gs = forward ? p->gs_f : p->gs_b;
    if (p->sweep_mode == DFM2G_SWEEP_GROUPS && gs.ok && gs.values_ok) {
      ran = DFM2G_SWEEP_GROUPS;
      return group_sweep(p, forward, (const float *)in, (float *)out, skip);
    }
  }
  const unsigned longest = forward ? p->max_lower : p->max_upper;
  const bool wide = longest > 12 && longest <= 24;
  void *kernel = wide ? (forward ? (void *)k_sweep_syncfree<T, true, 8> : (void *)k_sweep_syncfree<T, false, 8>)
                      : (forward ? (void *)k_sweep_syncfree<T, true, 4> : (void *)k_sweep_syncfree<T, false, 4>);
  int *cache = &p->coop_cache[sizeof(T) == 8 ? 1 : 0][forward ? 1 : 0][wide ? 1 : 0];
  DFM2G_TRY(coop_blocks<T>(kernel, cache));
  const unsigned want = blocks_for((size_t)n * 32, 256);
  const unsigned blocks = std::min<unsigned>(want, (unsigned)*cache);
  const uint4 *meta = forward ? p->meta_f.p : p->meta_b.p;
  const unsigned nlev = forward ? p->nlev_f : p->nlev_b;
  unsigned long long timeout = kWaitTimeoutNs + 20000ull * nlev;
  int *err = p->err.p;
  void *args[] = {(void *)&n, (void *)&meta, (void *)&p->col.p, (void *)&vcrs, (void *)&vdia, (void *)&in,
                  (void *)&out, (void *)&err, (void *)&timeout, (void *)&skip};
  DFM2G_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(blocks), dim3(256), args, 0, stream()));
  note_launches(1);
  ran = DFM2G_SWEEP_SYNCFREE;
  return DFM2G_OK;
}

int ilu_sweep(dfm2g_ilu_s *p, int prec, bool forward, const void *in, void *out) {
  if (prec == DFM2G_F64)
    return sweep_impl<double>(p, forward, (const double *)in, (double *)out, p->vcrs.p, p->vdia.p, nullptr, false);
  DFM2G_TRY(ilu_ensure_f32(p));
  return sweep_impl<float>(p, forward, (const float *)in, (float *)out, p->vcrs32.p, p->vdia32.p, nullptr, false);
}

// A sweep that allocates nothing: the chain schedule is used only when its
// records already exist, otherwise the sync-free one. The FP32 factors must exist.
static int ilu_sweep_noalloc(dfm2g_ilu_s *p, int prec, bool forward, const void *in, void *out) {
  if (prec == DFM2G_F64)
    return sweep_impl<double>(p, forward, (const double *)in, (double *)out, p->vcrs.p, p->vdia.p, nullptr, false,
                              false);
  return sweep_impl<float>(p, forward, (const float *)in, (float *)out, p->vcrs32.p, p->vdia32.p, nullptr, false,
                           false);
}

// Variant for the solver loops: the sweep is skipped once *skip != 0, and in
// sync-free mode `out` must already hold the pending marker.
int ilu_sweep_guarded(dfm2g_ilu_s *p, int prec, bool forward, const void *in, void *out, const int *skip) {
  if (prec == DFM2G_F64)
    return sweep_impl<double>(p, forward, (const double *)in, (double *)out, p->vcrs.p, p->vdia.p, skip, true);
  return sweep_impl<float>(p, forward, (const float *)in, (float *)out, p->vcrs32.p, p->vdia32.p, skip, true);
}

int ilu_ensure_f32(dfm2g_ilu_s *p) {
  if (p->f32_valid) return DFM2G_OK;
  if (!p->has_factor) return fail(DFM2G_ERR_STATE, "ILU not decomposed");
  const size_t bb = (size_t)p->ndim * p->ndim;
  DFM2G_TRY(p->vcrs32.ensure(p->nnz * bb + 1));
  DFM2G_TRY(p->vdia32.ensure((size_t)p->nblk * bb + 1));
  to_f32(p->nnz * bb, p->vcrs.p, p->vcrs32.p);
  to_f32((size_t)p->nblk * bb, p->vdia.p, p->vdia32.p);
  DFM2G_LAUNCH_CHECK();
  DFM2G_TRY(group_values_fill(p));
  p->f32_valid = true;
  return DFM2G_OK;
}

static int read_err(dfm2g_ilu_s *p) {
  int h = 0;
  DFM2G_CUDA(cudaMemcpyAsync(&h, p->err.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  if (h != 0) {
    DFM2G_CUDA(cudaMemsetAsync(p->err.p, 0, sizeof(int), stream()));
    return fail(h, "ILU sweep: device-side wait timed out");
  }
  return DFM2G_OK;
}

}  // namespace dfm2g

using namespace dfm2g;

// Level-of-fill symbolic ILU(k) on the host (Initialize_ILUk,
// include/delfem2/ls_ilu_block_sparse.cpp:849-999). Row i starts as its sorted
// matrix row (level 0); for each k < i of the row in ascending order with
// lev(i,k) + 1 <= fill_level, every j of row k's upper part with
// lev(k,j) + 1 <= fill_level and j != i that row i lacks is inserted with level
// max(lev(i,k), lev(k,j)) + 1. An entry already present keeps its level (as the
// reference does). fill_level == -1 keeps every fill.
static int ilu_symbolic_k(unsigned n, const std::vector<unsigned> &mrs, const std::vector<unsigned> &mcol,
                          int fill_level, std::vector<unsigned> &rs, std::vector<unsigned> &col) {
  rs.assign((size_t)n + 1, 0u);
  col.clear();
  std::vector<unsigned> lev, dia(n);
  std::vector<std::pair<unsigned, unsigned>> row;  // (column, level), ascending
  auto too_deep = [fill_level](unsigned l) { return fill_level != -1 && (int)l + 1 > fill_level; };
  for (unsigned i = 0; i < n; ++i) {
    row.clear();
    for (unsigned s = mrs[i]; s < mrs[i + 1]; ++s) row.emplace_back(mcol[s], 0u);
    std::sort(row.begin(), row.end());
    for (size_t kk = 0; kk < row.size(); ++kk) {
      const unsigned k = row[kk].first, lik = row[kk].second;
      if (too_deep(lik)) continue;
      if (k >= i) break;
      size_t pos = kk;
      for (unsigned s = dia[k]; s < rs[k + 1]; ++s) {
        const unsigned lkj = lev[s], j = col[s];
        if (too_deep(lkj) || j == i) continue;
        while (pos + 1 < row.size() && row[pos + 1].first < j) ++pos;
        if (pos + 1 < row.size() && row[pos + 1].first == j) continue;
        row.insert(row.begin() + (std::ptrdiff_t)pos + 1, std::make_pair(j, std::max(lik, lkj) + 1));
        ++pos;
      }
    }
    if (col.size() + row.size() > 0xFFFFFFF0ull)
      return fail(DFM2G_ERR_UNSUPPORTED, "set_pattern_k: fill exceeds 32-bit offsets");
    dia[i] = (unsigned)(col.size() + row.size());
    for (size_t t = 0; t < row.size(); ++t) {
      if (row[t].first > i && dia[i] == col.size() + row.size()) dia[i] = (unsigned)(col.size() + t);
    }
    for (const auto &e : row) {
      col.push_back(e.first);
      lev.push_back(e.second);
    }
    rs[i + 1] = (unsigned)col.size();
  }
  return DFM2G_OK;
}

// Installs an ILU pattern (row offsets and columns, rows sorted or not):
// device copies, row sort + dia_ind, level sets and sweep schedules.
static int ilu_install_pattern(dfm2g_ilu p, unsigned n, unsigned ndim, size_t nnz, const unsigned *rs_src,
                               const unsigned *col_src, cudaMemcpyKind kind) {
  p->nblk = n;
  p->ndim = ndim;
  p->nnz = nnz;
  p->has_pattern = p->has_factor = p->f32_valid = false;
  const size_t bb = (size_t)ndim * ndim;
  DFM2G_TRY(p->row_start.resize(n + 1));
  DFM2G_TRY(p->col.resize(nnz + 1));
  DFM2G_TRY(p->dia_ind.resize(n + 1));
  DFM2G_TRY(p->vcrs.resize(nnz * bb + 4));
  DFM2G_TRY(p->vdia.resize((size_t)n * bb + 4));
  DFM2G_CUDA(cudaMemcpyAsync(p->row_start.p, rs_src, sizeof(unsigned) * (n + 1), kind, stream()));
  if (nnz) DFM2G_CUDA(cudaMemcpyAsync(p->col.p, col_src, sizeof(unsigned) * nnz, kind, stream()));
  if (n) {
    k_sort_rows_diaind<<<blocks_for(n, 128, ctx().num_sms * 16), 128, 0, stream()>>>(n, p->row_start.p, p->col.p,
                                                                                    p->dia_ind.p);
    DFM2G_LAUNCH_CHECK();
  }
  {  // longest lower / upper triangle row (picks the sweep's register fragment)
    std::vector<unsigned> hrs(n + 1), hdia(n);
    if (n) {
      DFM2G_CUDA(cudaMemcpyAsync(hrs.data(), p->row_start.p, sizeof(unsigned) * (n + 1), cudaMemcpyDeviceToHost,
                                 stream()));
      DFM2G_CUDA(cudaMemcpyAsync(hdia.data(), p->dia_ind.p, sizeof(unsigned) * n, cudaMemcpyDeviceToHost, stream()));
      DFM2G_CUDA(cudaStreamSynchronize(stream()));
    }
    p->max_lower = p->max_upper = 0;
    for (unsigned i = 0; i < n; ++i) {
      p->max_lower = std::max(p->max_lower, hdia[i] - hrs[i]);
      p->max_upper = std::max(p->max_upper, hrs[i + 1] - hdia[i]);
    }
  }
  for (auto &a : p->coop_cache)
    for (auto &b : a)
      for (int &c : b) c = 0;
  DFM2G_TRY(compute_levels(p, false));
  DFM2G_TRY(compute_levels(p, true));
  stream_schedules_reset(p);
  chain_schedules_reset(p);
  tile_schedules_reset(p);
  if (ndim == 3) {  // the blob and row-range schedules are written for 3x3 blocks
    DFM2G_TRY(group_schedules_build(p));
    DFM2G_TRY(part_schedules_build(p));
  } else {
    p->gs_f.ok = p->gs_b.ok = false;
    p->parts_ok = false;
  }
  // Default: tiles or chains, picked per pattern and precision (3.24M DOF on
  // GB300, FP32 / FP64 forward sweep: 0.47 / 0.88 ms over tiles against 0.58
  // / 1.23 ms over chains and 0.91 / 2.19 ms sync-free; scalar Poisson on the
  // same mesh, chains: mixed solve 165 ms against 225 ms sync-free).
  p->sweep_mode = DFM2G_SWEEP_AUTO;
  const size_t nvec = (size_t)n * ndim + 1;
  DFM2G_TRY(p->tmp64a.resize(nvec));
  DFM2G_TRY(p->tmp64b.resize(nvec));
  DFM2G_TRY(p->tmp32a.resize(nvec));
  DFM2G_TRY(p->tmp32b.resize(nvec));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  p->has_pattern = true;
  return DFM2G_OK;
}

static int check_ilu(dfm2g_ilu p, bool pattern, bool factor) {
  if (!p) return fail(DFM2G_ERR_ARG, "null ILU handle");
  if (pattern && !p->has_pattern) return fail(DFM2G_ERR_STATE, "ILU has no pattern (call set_pattern0)");
  if (factor && !p->has_factor) return fail(DFM2G_ERR_STATE, "ILU not decomposed (call decompose)");
  return DFM2G_OK;
}

extern "C" {

int dfm2g_ilu_create(dfm2g_ilu *out) try {
  if (!out) return fail(DFM2G_ERR_ARG, "ilu_create: null out");
  DFM2G_TRY(ensure_context());
  auto *p = new dfm2g_ilu_s();
  DFM2G_TRY(p->err.resize(1));
  DFM2G_TRY(p->nsing.resize(1));
  DFM2G_CUDA(cudaMemsetAsync(p->err.p, 0, sizeof(int), stream()));
  *out = p;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_destroy(dfm2g_ilu p) try {
  if (p) {
    cudaStreamSynchronize(stream());
    delete p;
  }
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_set_pattern0(dfm2g_ilu p, dfm2g_bsr m) try {
  DFM2G_TRY(check_ilu(p, false, false));
  if (!m || !m->has_pattern) return fail(DFM2G_ERR_STATE, "set_pattern0: matrix has no pattern");
  return ilu_install_pattern(p, m->nblk, m->ndim, m->nnz, m->row_start.p, m->col.p, cudaMemcpyDeviceToDevice);
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_set_pattern_k(dfm2g_ilu p, dfm2g_bsr m, int fill_level) try {
  DFM2G_TRY(check_ilu(p, false, false));
  if (!m || !m->has_pattern) return fail(DFM2G_ERR_STATE, "set_pattern_k: matrix has no pattern");
  if (fill_level == 0) return dfm2g_ilu_set_pattern0(p, m);
  std::vector<unsigned> rs, col;
  DFM2G_TRY(ilu_symbolic_k(m->nblk, m->h_row_start, m->h_col, fill_level, rs, col));
  return ilu_install_pattern(p, m->nblk, m->ndim, col.size(), rs.data(), col.data(), cudaMemcpyHostToDevice);
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_copy_value(dfm2g_ilu p, dfm2g_bsr m) try {
  DFM2G_TRY(check_ilu(p, true, false));
  if (!m || !m->has_pattern || m->nblk != p->nblk) return fail(DFM2G_ERR_ARG, "copy_value: matrix size mismatch");
  if (m->ndim != p->ndim)
    return fail(DFM2G_ERR_ARG, "copy_value: matrix blocks are %ux%u, the pattern's %ux%u", m->ndim, m->ndim, p->ndim,
                p->ndim);
  const size_t bb = (size_t)p->ndim * p->ndim;
  DFM2G_CUDA(cudaMemsetAsync(p->vcrs.p, 0, sizeof(double) * p->nnz * bb, stream()));
  if (p->nblk) {
    const unsigned blocks = blocks_for((size_t)p->nblk * 32, 256, ctx().num_sms * 16);
    if (p->ndim == 3)
      k_ilu_copy<9><<<blocks, 256, 0, stream()>>>(p->nblk, m->row_start.p, m->col.p, m->vcrs.p, p->row_start.p,
                                                  p->col.p, p->vcrs.p);
    else if (p->ndim == 2)
      k_ilu_copy<4><<<blocks, 256, 0, stream()>>>(p->nblk, m->row_start.p, m->col.p, m->vcrs.p, p->row_start.p,
                                                  p->col.p, p->vcrs.p);
    else
      k_ilu_copy<1><<<blocks, 256, 0, stream()>>>(p->nblk, m->row_start.p, m->col.p, m->vcrs.p, p->row_start.p,
                                                  p->col.p, p->vcrs.p);
    DFM2G_LAUNCH_CHECK();
    DFM2G_CUDA(cudaMemcpyAsync(p->vdia.p, m->vdia.p, sizeof(double) * bb * p->nblk, cudaMemcpyDeviceToDevice,
                               stream()));
  }
  p->has_factor = false;
  p->f32_valid = false;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_decompose(dfm2g_ilu p, int *n_singular) try {
  DFM2G_TRY(check_ilu(p, true, false));
  DFM2G_CUDA(cudaMemsetAsync(p->nsing.p, 0, sizeof(int), stream()));
  const std::vector<unsigned> &ls = p->h_lstart_f;
  for (size_t l = 0; l + 1 < ls.size(); ++l) {
    const unsigned nrows = ls[l + 1] - ls[l];
    const unsigned blocks = blocks_for((size_t)nrows * 32, 256);
    if (p->ndim == 3)
      k_ilu_factor_level<<<blocks, 256, 0, stream()>>>(p->order_f.p + ls[l], nrows, p->row_start.p, p->col.p,
                                                       p->dia_ind.p, p->vcrs.p, p->vdia.p, p->nsing.p);
    else if (p->ndim == 2)
      k_ilu_factor_level_nd<2><<<blocks, 256, 0, stream()>>>(p->order_f.p + ls[l], nrows, p->row_start.p, p->col.p,
                                                             p->dia_ind.p, p->vcrs.p, p->vdia.p, p->nsing.p);
    else
      k_ilu_factor_level_nd<1><<<blocks, 256, 0, stream()>>>(p->order_f.p + ls[l], nrows, p->row_start.p, p->col.p,
                                                             p->dia_ind.p, p->vcrs.p, p->vdia.p, p->nsing.p);
  }
  DFM2G_LAUNCH_CHECK();
  int ns = 0;
  DFM2G_CUDA(cudaMemcpyAsync(&ns, p->nsing.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  if (n_singular) *n_singular = ns;
  p->has_factor = true;
  p->f32_valid = false;
  p->factor_version++;
  if (ns > 10) return fail(DFM2G_ERR_SINGULAR_PIVOT, "ILU: %d pivots with |det| <= 1e-30", ns);
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

static int precond_host(dfm2g_ilu p, int prec, void *vec, int mem, int which /*1 fwd, 2 bwd, 3 both*/) {
  DFM2G_TRY(check_ilu(p, true, true));
  if (!vec) return fail(DFM2G_ERR_ARG, "null vector");
  if (prec != DFM2G_F64 && prec != DFM2G_F32) return fail(DFM2G_ERR_ARG, "prec must be F64 or F32");
  const size_t n = (size_t)p->nblk * p->ndim;
  const size_t es = prec == DFM2G_F64 ? 8 : 4;
  void *a = prec == DFM2G_F64 ? (void *)p->tmp64a.p : (void *)p->tmp32a.p;
  void *b = prec == DFM2G_F64 ? (void *)p->tmp64b.p : (void *)p->tmp32b.p;
  if (mem == DFM2G_MEM_HOST) {
    DFM2G_CUDA(cudaMemcpyAsync(a, vec, n * es, cudaMemcpyHostToDevice, stream()));
  } else {
    DFM2G_CUDA(cudaMemcpyAsync(a, vec, n * es, cudaMemcpyDeviceToDevice, stream()));
  }
  void *res = a;
  if (which & 1) {
    DFM2G_TRY(ilu_sweep(p, prec, true, res, b));
    res = b;
  }
  if (which & 2) {
    void *dst = (res == a) ? b : a;
    DFM2G_TRY(ilu_sweep(p, prec, false, res, dst));
    res = dst;
  }
  DFM2G_CUDA(cudaMemcpyAsync(vec, res, n * es, mem == DFM2G_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                             stream()));
  return read_err(p);
}

// ---------------------------------------------------------------------------
// SolvePrecond without any allocation.
//
// The forward sweep needs somewhere to put its result while the backward
// sweep reads it. Here that intermediate vector is this fixed device array
// instead of memory the library allocates. It is loaded with the library
// (with CUDA's lazy module loading, on first use) and every GPU that loads the
// library keeps it until the process exits. Its size caps the problem:
// 3 * nblk <= kNoAllocMaxScalars.
constexpr size_t kNoAllocMaxScalars = size_t(1) << 20;  // 8 MiB as FP64
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxScalars];

// Device address of g_noalloc_scratch per device, looked up once per device
// with that device current (the host-side name is only a stand-in).
static void *g_noalloc_addr[64];
static std::mutex g_noalloc_mutex;

static int noalloc_scratch(void **out) {
  int dev = 0;
  DFM2G_CUDA(cudaGetDevice(&dev));
  // The library's stream and handles live on ctx().device; a sweep launched
  // there must get that device's copy of the array.
  if (dev != ctx().device)
    return fail(DFM2G_ERR_STATE, "solve_precond_noalloc: current device %d is not the library's device %d", dev,
                ctx().device);
  if (dev < 0 || dev >= 64) return fail(DFM2G_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(DFM2G_ERR_CUDA, "cudaGetSymbolAddress(scratch) on device %d: %s", dev, cudaGetErrorString(e));
    g_noalloc_addr[dev] = ptr;
  }
  *out = g_noalloc_addr[dev];
  return DFM2G_OK;
}

int dfm2g_ilu_solve_precond_noalloc(dfm2g_ilu p, int prec, void *vec) try {
  DFM2G_TRY(check_ilu(p, true, true));
  if (!vec) return fail(DFM2G_ERR_ARG, "solve_precond_noalloc: null vector");
  if (prec != DFM2G_F64 && prec != DFM2G_F32) return fail(DFM2G_ERR_ARG, "prec must be F64 or F32");
  const size_t n = (size_t)p->nblk * p->ndim;
  if (n > kNoAllocMaxScalars)
    return fail(DFM2G_ERR_ARG,
                "solve_precond_noalloc: %zu unknowns exceed the fixed scratch of %zu (at most %zu %ux%u block rows); "
                "use dfm2g_ilu_solve_precond for larger systems",
                n, kNoAllocMaxScalars, kNoAllocMaxScalars / p->ndim, p->ndim, p->ndim);
  if (prec == DFM2G_F32 && !p->f32_valid)
    return fail(DFM2G_ERR_STATE,
                "solve_precond_noalloc: no FP32 factors yet (creating them allocates); call "
                "dfm2g_ilu_solve_precond once with DFM2G_F32 first");
  void *scratch = nullptr;
  DFM2G_TRY(ensure_context());
  DFM2G_TRY(noalloc_scratch(&scratch));
  // forward: vec -> scratch; backward: scratch -> vec. Each sweep first fills
  // its own output (the pending marker in the sync-free schedule, a copy of
  // its input in the level schedule), so no scratch content carries over
  // from an earlier call.
  DFM2G_TRY(ilu_sweep_noalloc(p, prec, true, vec, scratch));
  DFM2G_TRY(ilu_sweep_noalloc(p, prec, false, scratch, vec));
  return read_err(p);
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_forward(dfm2g_ilu p, int prec, void *vec, int mem) try {
  return precond_host(p, prec, vec, mem, 1);
} catch (...) {
  return host_failure();
}
int dfm2g_ilu_backward(dfm2g_ilu p, int prec, void *vec, int mem) try {
  return precond_host(p, prec, vec, mem, 2);
} catch (...) {
  return host_failure();
}
int dfm2g_ilu_solve_precond(dfm2g_ilu p, int prec, void *vec, int mem) try {
  return precond_host(p, prec, vec, mem, 3);
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_set_sweep_mode(dfm2g_ilu p, int mode) try {
  DFM2G_TRY(check_ilu(p, false, false));
  if (mode != DFM2G_SWEEP_SYNCFREE && mode != DFM2G_SWEEP_LEVELS && mode != DFM2G_SWEEP_GROUPS &&
      mode != DFM2G_SWEEP_BLOCK && mode != DFM2G_SWEEP_PARTS && mode != DFM2G_SWEEP_CHAINS &&
      mode != DFM2G_SWEEP_TILES && mode != DFM2G_SWEEP_AUTO && mode != DFM2G_SWEEP_CLUSTER)
    return fail(DFM2G_ERR_ARG, "unknown sweep mode");
  if (p->ndim != 3 && mode != DFM2G_SWEEP_SYNCFREE && mode != DFM2G_SWEEP_LEVELS && mode != DFM2G_SWEEP_CHAINS &&
      mode != DFM2G_SWEEP_AUTO)
    return fail(DFM2G_ERR_UNSUPPORTED, "sweep mode %d needs 3x3 blocks (the pattern has ndim %u)", mode, p->ndim);
  if (mode == DFM2G_SWEEP_PARTS && !p->parts_ok)
    return fail(DFM2G_ERR_UNSUPPORTED, "row-range partition unavailable for this pattern");
  if (mode == DFM2G_SWEEP_GROUPS && !(p->gs_f.ok && p->gs_b.ok))
    return fail(DFM2G_ERR_UNSUPPORTED, "blob schedule unavailable for this pattern");
  p->sweep_mode = mode;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_get_sweep_mode(dfm2g_ilu p, int *mode) try {
  DFM2G_TRY(check_ilu(p, false, false));
  if (!mode) return fail(DFM2G_ERR_ARG, "get_sweep_mode: null out");
  *mode = p->sweep_mode;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_last_schedule(dfm2g_ilu p, int prec, int backward, int *mode) try {
  DFM2G_TRY(check_ilu(p, false, false));
  if (!mode) return fail(DFM2G_ERR_ARG, "last_schedule: null out");
  if (prec != DFM2G_F64 && prec != DFM2G_F32) return fail(DFM2G_ERR_ARG, "last_schedule: bad precision");
  *mode = p->last_sched[prec == DFM2G_F64 ? 1 : 0][backward ? 1 : 0];
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_info(dfm2g_ilu p, unsigned *nblk, size_t *nnz) try {
  DFM2G_TRY(check_ilu(p, true, false));
  if (nblk) *nblk = p->nblk;
  if (nnz) *nnz = p->nnz;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_get_row_start(dfm2g_ilu p, unsigned *row_start) try {
  DFM2G_TRY(check_ilu(p, true, false));
  if (!row_start) return fail(DFM2G_ERR_ARG, "get_row_start: null out");
  DFM2G_CUDA(cudaMemcpyAsync(row_start, p->row_start.p, sizeof(unsigned) * (p->nblk + 1), cudaMemcpyDeviceToHost,
                             stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_get_pattern(dfm2g_ilu p, unsigned *col, unsigned *dia_ind) try {
  DFM2G_TRY(check_ilu(p, true, false));
  if (col && p->nnz) DFM2G_CUDA(cudaMemcpyAsync(col, p->col.p, sizeof(unsigned) * p->nnz, cudaMemcpyDeviceToHost, stream()));
  if (dia_ind && p->nblk)
    DFM2G_CUDA(cudaMemcpyAsync(dia_ind, p->dia_ind.p, sizeof(unsigned) * p->nblk, cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_get_values(dfm2g_ilu p, double *vcrs, double *vdia, int mem) try {
  DFM2G_TRY(check_ilu(p, true, false));
  const cudaMemcpyKind k = mem == DFM2G_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  const size_t bb = (size_t)p->ndim * p->ndim;
  if (vcrs && p->nnz) DFM2G_CUDA(cudaMemcpyAsync(vcrs, p->vcrs.p, sizeof(double) * bb * p->nnz, k, stream()));
  if (vdia && p->nblk) DFM2G_CUDA(cudaMemcpyAsync(vdia, p->vdia.p, sizeof(double) * bb * p->nblk, k, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_ilu_get_levels(dfm2g_ilu p, int backward, unsigned *level, unsigned *order, unsigned *level_start,
                         unsigned *nlevels) try {
  DFM2G_TRY(check_ilu(p, true, false));
  const unsigned n = p->nblk;
  const unsigned nlev = backward ? p->nlev_b : p->nlev_f;
  if (level && n)
    DFM2G_CUDA(cudaMemcpyAsync(level, backward ? p->level_b.p : p->level_f.p, sizeof(unsigned) * n,
                               cudaMemcpyDeviceToHost, stream()));
  if (order && n)
    DFM2G_CUDA(cudaMemcpyAsync(order, backward ? p->order_b.p : p->order_f.p, sizeof(unsigned) * n,
                               cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  if (level_start) {
    const std::vector<unsigned> &hl = backward ? p->h_lstart_b : p->h_lstart_f;
    std::memcpy(level_start, hl.data(), sizeof(unsigned) * hl.size());
  }
  if (nlevels) *nlevels = nlev;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

}  // extern "C"

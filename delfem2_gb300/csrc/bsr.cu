// CMatrixSparse<double> on the device: pattern, values, fixed boundary
// conditions, MatVec, and the colour-scheduled Merge, for 3x3 blocks (the
// tuned path) and for 1x1 / 2x2 blocks (nd.cuh).
//
// Device layout: row_start[nblk+1] and col[nnz] (u32, the reference's
// col_ind_ / row_ptr_), vcrs[B*B*nnz] and vdia[B*B*nblk] (f64, row-major
// B x B, B = ndim), plus an FP32 mirror vcrs32/vdia32 used by the
// mixed-precision solver.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "nd.cuh"
#include "rowkern.cuh"
#include "spmv_tma.cuh"

namespace dfm2g {

int require_3x3(const dfm2g_bsr_s *m, const char *what) {
  if (m && m->ndim != 3) return fail(DFM2G_ERR_UNSUPPORTED, "%s: needs 3x3 blocks (matrix has ndim %u)", what, m->ndim);
  return DFM2G_OK;
}

// y = alpha*K*x + beta*y for 1x1 and 2x2 blocks, eight lanes per block row.
template <typename T, int B>
__global__ void __launch_bounds__(256) k_nd_spmv(unsigned nblk, const unsigned *__restrict__ row_start,
                                                 const unsigned *__restrict__ col, const T *__restrict__ vcrs,
                                                 const T *__restrict__ vdia, T *__restrict__ y, T alpha,
                                                 const T *__restrict__ x, T beta) {
  nd_spmv_rows<T, B>(nblk, row_start, col, vcrs, vdia, x, [&](unsigned row, const T s[B], unsigned sub) {
    if (sub < (unsigned)B) {
      T *py = y + (size_t)row * B + sub;
      *py = beta * *py + alpha * nd_pick<T, B>(s, sub);
    }
  });
}

// ---------------------------------------------------------------------------
// SpMV y = alpha*K*x + beta*y, one warp per block row (rows w, w+W, ...), in
// the lane layout of rowkern.cuh (off-diagonal blocks, then the diagonal as
// the row's last block). Software-pipelined: the next row's block columns and
// values are requested before the current row's x entries are gathered, and
// the row offsets two rows ahead before that.
template <typename T>
__global__ void __launch_bounds__(256) k_bsr_spmv(unsigned nblk, const unsigned *__restrict__ row_start,
                                                  const unsigned *__restrict__ col,
                                                  const T *__restrict__ vcrs, const T *__restrict__ vdia,
                                                  T *__restrict__ y, T alpha, const T *__restrict__ x, T beta) {
  const unsigned lane = threadIdx.x & 31;
  spmv_rows(nblk, row_start, col, vcrs, vdia, x, [&](unsigned row, const T s[3]) {
    if (lane < 3) {
      T *py = y + (size_t)row * 3 + lane;
      *py = beta * *py + alpha * pick3(s, lane);
    }
  });
}

// Same product in the component layout (spmv_tma_rows_c).
template <typename T>
__global__ void __launch_bounds__(TileCfgC<T>::kThreads, 1)
    k_bsr_spmv_tma_c(const unsigned *__restrict__ tiles, unsigned ntiles, const unsigned *__restrict__ row_start,
                     const unsigned *__restrict__ col, const T *__restrict__ vcrs, const T *__restrict__ vdia,
                     T *__restrict__ y, T alpha, const T *__restrict__ x, T beta, int *err,
                     unsigned long long timeout_ns) {
  extern __shared__ __align__(128) unsigned char tma_smem[];
  spmv_tma_rows_c<T>(tiles, ntiles, row_start, col, vcrs, vdia, x, err, timeout_ns, tma_smem,
                     [&](unsigned row, unsigned a, T v) {
                       T *py = y + (size_t)row * 3 + a;
                       *py = beta * *py + alpha * v;
                     });
}

// Tiles of consecutive rows with at most `maxb` off-diagonal blocks and `maxr`
// rows each; false when one row alone has more than `maxb` blocks.
static bool make_tiles(const std::vector<unsigned> &rs, unsigned nblk, unsigned maxb, unsigned maxr,
                       std::vector<unsigned> &t) {
  t.assign(1, 0u);
  unsigned r0 = 0;
  for (unsigned i = 0; i < nblk; ++i) {
    if (rs[i + 1] - rs[i] > maxb) return false;
    if (rs[i + 1] - rs[r0] > maxb || i + 1 - r0 > maxr) {
      t.push_back(i);
      r0 = i;
    }
  }
  if (nblk) t.push_back(nblk);
  return true;
}

int bsr_tiles_build(dfm2g_bsr_s *m) {
  m->tiles_ok = false;
  std::vector<unsigned> t32, t64;
  if (m->nblk == 0 ||
      !make_tiles(m->h_row_start, m->nblk, TileCfgC<float>::kBlocks, TileCfgC<float>::kRows, t32) ||
      !make_tiles(m->h_row_start, m->nblk, TileCfgC<double>::kBlocks, TileCfgC<double>::kRows, t64))
    return DFM2G_OK;
  DFM2G_TRY(m->tiles32.resize(t32.size()));
  DFM2G_TRY(m->tiles64.resize(t64.size()));
  DFM2G_TRY(m->err.resize(1));
  DFM2G_CUDA(cudaMemcpyAsync(m->tiles32.p, t32.data(), sizeof(unsigned) * t32.size(), cudaMemcpyHostToDevice,
                             stream()));
  DFM2G_CUDA(cudaMemcpyAsync(m->tiles64.p, t64.data(), sizeof(unsigned) * t64.size(), cudaMemcpyHostToDevice,
                             stream()));
  DFM2G_CUDA(cudaMemsetAsync(m->err.p, 0, sizeof(int), stream()));
  static int attr_device = -1;  // opt the kernels in to their shared memory once per device
  if (attr_device != ctx().device) {
    DFM2G_CUDA(cudaFuncSetAttribute(k_bsr_spmv_tma_c<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)TileCfgC<float>::kSmem));
    DFM2G_CUDA(cudaFuncSetAttribute(k_bsr_spmv_tma_c<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)TileCfgC<double>::kSmem));
    attr_device = ctx().device;
  }
  m->ntiles32 = (unsigned)t32.size() - 1;
  m->ntiles64 = (unsigned)t64.size() - 1;
  m->tiles_ok = true;
  return DFM2G_OK;
}

// Reads and clears the SpMV error word (a bounded wait that gave up).
int bsr_check_err(dfm2g_bsr_s *m) {
  if (!m->tiles_ok) return DFM2G_OK;
  int e = 0;
  DFM2G_CUDA(cudaMemcpyAsync(&e, m->err.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  if (e) {
    DFM2G_CUDA(cudaMemsetAsync(m->err.p, 0, sizeof(int), stream()));
    return fail(DFM2G_ERR_WAIT_TIMEOUT, "SpMV: a pipeline wait timed out");
  }
  return DFM2G_OK;
}

template <typename T>
static void nd_spmv_launch(dfm2g_bsr_s *m, const T *vcrs, const T *vdia, T *y, T alpha, const T *x, T beta) {
  const unsigned blocks = blocks_for((size_t)m->nblk * 32, 256, (unsigned)ctx().num_sms * 16);
  if (m->ndim == 1)
    k_nd_spmv<T, 1><<<blocks, 256, 0, stream()>>>(m->nblk, m->row_start.p, m->col.p, vcrs, vdia, y, alpha, x, beta);
  else
    k_nd_spmv<T, 2><<<blocks, 256, 0, stream()>>>(m->nblk, m->row_start.p, m->col.p, vcrs, vdia, y, alpha, x, beta);
}

int bsr_spmv(dfm2g_bsr_s *m, int prec, void *y, double alpha, const void *x, double beta) {
  if (m->ndim != 3) {
    if (prec == DFM2G_F64) {
      nd_spmv_launch<double>(m, m->vcrs.p, m->vdia.p, (double *)y, alpha, (const double *)x, beta);
    } else if (prec == DFM2G_F32) {
      DFM2G_TRY(bsr_ensure_f32(m));
      nd_spmv_launch<float>(m, m->vcrs32.p, m->vdia32.p, (float *)y, (float)alpha, (const float *)x, (float)beta);
    } else {
      return fail(DFM2G_ERR_ARG, "matvec: prec must be DFM2G_F64 or DFM2G_F32");
    }
    note_launches(1);
    DFM2G_LAUNCH_CHECK();
    return DFM2G_OK;
  }
  if (m->tiles_ok && (prec == DFM2G_F64 || prec == DFM2G_F32)) {
    const unsigned long long timeout = kWaitTimeoutNs;
    if (prec == DFM2G_F64) {
      const unsigned grid = std::min(m->ntiles64, (unsigned)ctx().num_sms);
      k_bsr_spmv_tma_c<double><<<grid, TileCfgC<double>::kThreads, TileCfgC<double>::kSmem, stream()>>>(
          m->tiles64.p, m->ntiles64, m->row_start.p, m->col.p, m->vcrs.p, m->vdia.p, (double *)y, alpha,
          (const double *)x, beta, m->err.p, timeout);
    } else {
      DFM2G_TRY(bsr_ensure_f32(m));
      const unsigned grid = std::min(m->ntiles32, (unsigned)ctx().num_sms);
      k_bsr_spmv_tma_c<float><<<grid, TileCfgC<float>::kThreads, TileCfgC<float>::kSmem, stream()>>>(
          m->tiles32.p, m->ntiles32, m->row_start.p, m->col.p, m->vcrs32.p, m->vdia32.p, (float *)y, (float)alpha,
          (const float *)x, (float)beta, m->err.p, timeout);
    }
    note_launches(1);
    DFM2G_LAUNCH_CHECK();
    return DFM2G_OK;
  }
  const unsigned blocks = blocks_for((size_t)m->nblk * 32, 256, (unsigned)ctx().num_sms * 16);
  if (prec == DFM2G_F64) {
    k_bsr_spmv<double><<<blocks, 256, 0, stream()>>>(m->nblk, m->row_start.p, m->col.p, m->vcrs.p,
                                                    m->vdia.p, (double *)y, alpha, (const double *)x, beta);
  } else if (prec == DFM2G_F32) {
    DFM2G_TRY(bsr_ensure_f32(m));
    k_bsr_spmv<float><<<blocks, 256, 0, stream()>>>(m->nblk, m->row_start.p, m->col.p, m->vcrs32.p,
                                                   m->vdia32.p, (float *)y, (float)alpha,
                                                   (const float *)x, (float)beta);
  } else {
    return fail(DFM2G_ERR_ARG, "matvec: prec must be DFM2G_F64 or DFM2G_F32");
  }
  note_launches(1);
  DFM2G_LAUNCH_CHECK();
  return DFM2G_OK;
}

// ---------------------------------------------------------------------------
__global__ void k_to_f32(size_t n, const double *__restrict__ in, float *__restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

void to_f32(size_t n, const double *in, float *out) {
  if (n) k_to_f32<<<blocks_for(n, 256, ctx().num_sms * 8), 256, 0, stream()>>>(n, in, out);
}

int bsr_ensure_f32(dfm2g_bsr_s *m) {
  if (m->f32_valid) return DFM2G_OK;
  // +8 floats: bulk copies round their byte range up to 16 B past the last element
  const size_t bb = (size_t)m->ndim * m->ndim;
  DFM2G_TRY(m->vcrs32.ensure(m->nnz * bb + 8));
  DFM2G_TRY(m->vdia32.ensure((size_t)m->nblk * bb + 8));
  const unsigned cap = (unsigned)ctx().num_sms * 8;
  if (m->nnz)
    k_to_f32<<<blocks_for(m->nnz * bb, 256, cap), 256, 0, stream()>>>(m->nnz * bb, m->vcrs.p, m->vcrs32.p);
  if (m->nblk)
    k_to_f32<<<blocks_for((size_t)m->nblk * bb, 256, cap), 256, 0, stream()>>>((size_t)m->nblk * bb, m->vdia.p,
                                                                             m->vdia32.p);
  DFM2G_LAUNCH_CHECK();
  m->f32_valid = true;
  return DFM2G_OK;
}

// ---------------------------------------------------------------------------
// SetFixedBC: for each fixed DOF zero its row and column, diagonal entry 1.
__global__ void k_bsr_fixed_bc(unsigned nblk, const unsigned *__restrict__ row_start,
                               const unsigned *__restrict__ col, double *__restrict__ vcrs,
                               double *__restrict__ vdia, const int *__restrict__ bc) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned nwarp = (gridDim.x * blockDim.x) >> 5;
  for (unsigned row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nblk; row += nwarp) {
    const bool f0 = bc[row * 3 + 0] != 0, f1 = bc[row * 3 + 1] != 0, f2 = bc[row * 3 + 2] != 0;
    const unsigned s0 = row_start[row], s1 = row_start[row + 1];
    for (unsigned s = s0 + lane; s < s1; s += 32) {
      const unsigned j = col[s];
      const bool g[3] = {bc[j * 3 + 0] != 0, bc[j * 3 + 1] != 0, bc[j * 3 + 2] != 0};
      const bool f[3] = {f0, f1, f2};
      double *a = vcrs + (size_t)s * 9;
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          if (f[r] || g[c]) a[r * 3 + c] = 0.0;
    }
    if (lane < 9) {
      const unsigned r = lane / 3, c = lane % 3;
      const bool f[3] = {f0, f1, f2};
      double *d = vdia + (size_t)row * 9;
      if (f[r] || f[c]) d[lane] = (r == c) ? 1.0 : 0.0;
    }
  }
}

// The same for B x B blocks with B = ndim in {1, 2}.
__global__ void k_nd_fixed_bc(unsigned nblk, unsigned B, const unsigned *__restrict__ row_start,
                              const unsigned *__restrict__ col, double *__restrict__ vcrs, double *__restrict__ vdia,
                              const int *__restrict__ bc) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned nwarp = (gridDim.x * blockDim.x) >> 5;
  const unsigned bb = B * B;
  for (unsigned row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nblk; row += nwarp) {
    const unsigned s0 = row_start[row], s1 = row_start[row + 1];
    for (unsigned s = s0 + lane; s < s1; s += 32) {
      const unsigned j = col[s];
      double *a = vcrs + (size_t)s * bb;
      for (unsigned r = 0; r < B; ++r)
        for (unsigned c = 0; c < B; ++c)
          if (bc[(size_t)row * B + r] != 0 || bc[(size_t)j * B + c] != 0) a[r * B + c] = 0.0;
    }
    if (lane < bb) {
      const unsigned r = lane / B, c = lane % B;
      if (bc[(size_t)row * B + r] != 0 || bc[(size_t)row * B + c] != 0)
        vdia[(size_t)row * bb + lane] = (r == c) ? 1.0 : 0.0;
    }
  }
}

// vdia_i += eps I for B x B blocks.
__global__ void k_add_dia(unsigned nblk, unsigned B, double *vdia, double eps) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < nblk; i += gridDim.x * blockDim.x)
    for (unsigned r = 0; r < B; ++r) vdia[(size_t)i * B * B + r * (B + 1)] += eps;
}

__global__ void k_zero_bc(size_t n, double *__restrict__ b, const int *__restrict__ bc) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (bc[i] != 0) b[i] = 0.0;
}

// ---------------------------------------------------------------------------
// Colour-scheduled Merge. slot[(e*nno + a)*nno + b] is the val_crs_ slot of
// block (elem[e][a], elem[e][b]) or kDiag when both nodes coincide.
constexpr unsigned kDiag = 0xFFFFFFFFu;
constexpr unsigned kMissing = 0xFFFFFFFEu;

__global__ void k_slot_map(size_t nelem, unsigned nno, const unsigned *__restrict__ elem,
                           const unsigned *__restrict__ row_start, const unsigned *__restrict__ col,
                           unsigned *__restrict__ slot, int *__restrict__ missing) {
  const size_t total = nelem * nno * nno;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const size_t e = t / (nno * nno);
    const unsigned ab = (unsigned)(t - e * nno * nno), a = ab / nno, b = ab - a * nno;
    const unsigned i = elem[e * nno + a], j = elem[e * nno + b];
    unsigned s = kDiag;
    if (i != j) {
      s = kMissing;
      for (unsigned q = row_start[i]; q < row_start[i + 1]; ++q)
        if (col[q] == j) { s = q; break; }
      if (s == kMissing) atomicExch(missing, 1);
    }
    slot[t] = s;
  }
}

// One thread per (element of this colour, local node a) adds block row a of
// the element matrix. As in the reference's Merge
// (include/delfem2/ls_block_sparse.h:209-358), a pair (a, b) whose nodes are
// the same block adds the (a, a) block to the diagonal; this differs from
// (a, b) only for an element that repeats a node. The rows of a repeated node
// all go to one block row, so the thread of its first occurrence adds them,
// in the reference's (a, b) order, and the other occurrences' threads add
// nothing.
__global__ void k_merge_color(unsigned n, const unsigned *__restrict__ list, unsigned nno,
                              const unsigned *__restrict__ elem, const unsigned *__restrict__ slot,
                              const double *__restrict__ emat, unsigned bb, double *__restrict__ vcrs,
                              double *__restrict__ vdia) {
  const size_t total = (size_t)n * nno;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const size_t e = list[t / nno];
    const unsigned a = (unsigned)(t % nno);
    const unsigned i = elem[e * nno + a];
    bool first = true;
    for (unsigned a0 = 0; a0 < a; ++a0) first = first && elem[e * nno + a0] != i;
    if (!first) continue;
    for (unsigned a2 = a; a2 < nno; ++a2) {
      if (elem[e * nno + a2] != i) continue;
      for (unsigned b = 0; b < nno; ++b) {
        const size_t k = (e * nno + a2) * nno + b;
        const unsigned s = slot[k];
        double *dst = (s == kDiag) ? vdia + (size_t)i * bb : vcrs + (size_t)s * bb;
        const double *src = emat + ((s == kDiag) ? (e * nno + a2) * nno + a2 : k) * bb;
        for (unsigned q = 0; q < bb; ++q) dst[q] += src[q];
      }
    }
  }
}

int build_slot_map(const unsigned *d_elem, size_t nelem, unsigned nno, const dfm2g_bsr_s *m, unsigned *d_slot) {
  DevBuf<int> d_missing;
  DFM2G_TRY(d_missing.resize(1));
  DFM2G_CUDA(cudaMemsetAsync(d_missing.p, 0, sizeof(int), stream()));
  const size_t nslot = nelem * nno * nno;
  if (nslot)
    k_slot_map<<<blocks_for(nslot, 256, ctx().num_sms * 16), 256, 0, stream()>>>(nelem, nno, d_elem, m->row_start.p,
                                                                                m->col.p, d_slot, d_missing.p);
  DFM2G_LAUNCH_CHECK();
  int missing = 0;
  DFM2G_CUDA(cudaMemcpyAsync(&missing, d_missing.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  if (missing) return fail(DFM2G_ERR_MISSING_SLOT, "an element block is not in the sparsity pattern");
  return DFM2G_OK;
}

// Greedy colouring: element e takes the lowest colour not yet used by any
// element sharing one of its nodes. Deterministic (elements in index order).
int color_elements(const unsigned *elem, size_t nelem, unsigned nno, size_t np,
                   std::vector<unsigned> &by_color, std::vector<unsigned> &color_start) {
  constexpr int kWords = 4;  // up to 256 colours
  std::vector<uint64_t> used(np * kWords, 0);
  std::vector<unsigned short> color(nelem);
  unsigned ncolor = 0;
  for (size_t e = 0; e < nelem; ++e) {
    uint64_t m[kWords] = {0, 0, 0, 0};
    for (unsigned a = 0; a < nno; ++a) {
      const unsigned n = elem[e * nno + a];
      if (n >= np) return fail(DFM2G_ERR_ARG, "element %zu names node %u >= %zu", e, n, np);
      for (int w = 0; w < kWords; ++w) m[w] |= used[(size_t)n * kWords + w];
    }
    int c = -1;
    for (int w = 0; w < kWords && c < 0; ++w)
      if (~m[w]) c = w * 64 + __builtin_ctzll(~m[w]);
    if (c < 0) return fail(DFM2G_ERR_UNSUPPORTED, "element colouring needs more than 256 colours");
    color[e] = (unsigned short)c;
    ncolor = std::max(ncolor, (unsigned)c + 1);
    for (unsigned a = 0; a < nno; ++a) used[(size_t)elem[e * nno + a] * kWords + c / 64] |= 1ull << (c % 64);
  }
  color_start.assign(ncolor + 1, 0);
  for (size_t e = 0; e < nelem; ++e) color_start[color[e] + 1]++;
  for (unsigned c = 0; c < ncolor; ++c) color_start[c + 1] += color_start[c];
  by_color.resize(nelem);
  std::vector<unsigned> cur(color_start.begin(), color_start.end() - 1);
  for (size_t e = 0; e < nelem; ++e) by_color[cur[color[e]]++] = (unsigned)e;
  return DFM2G_OK;
}

}  // namespace dfm2g

using namespace dfm2g;

static int check_bsr(dfm2g_bsr m, bool need_pattern = true) {
  if (!m) return fail(DFM2G_ERR_ARG, "null matrix handle");
  if (need_pattern && !m->has_pattern) return fail(DFM2G_ERR_STATE, "matrix has no pattern (call set_pattern)");
  return DFM2G_OK;
}

extern "C" {

int dfm2g_bsr_create(dfm2g_bsr *out, unsigned nblk, unsigned ndim) try {
  if (!out) return fail(DFM2G_ERR_ARG, "bsr_create: null out");
  if (ndim < 1 || ndim > 3) return fail(DFM2G_ERR_UNSUPPORTED, "block size ndim=%u (1, 2 or 3 supported)", ndim);
  DFM2G_TRY(ensure_context());
  auto *m = new dfm2g_bsr_s();
  m->nblk = nblk;
  m->ndim = ndim;
  *out = m;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_destroy(dfm2g_bsr m) try {
  if (m) {
    cudaStreamSynchronize(stream());
    delete m;
  }
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_set_pattern(dfm2g_bsr m, const unsigned *row_start, size_t n_row_start, const unsigned *col,
                          size_t ncol) try {
  DFM2G_TRY(check_bsr(m, false));
  if (!row_start || n_row_start != (size_t)m->nblk + 1)
    return fail(DFM2G_ERR_ARG, "set_pattern: row_start must have nblk+1 = %u entries", m->nblk + 1);
  if (row_start[0] != 0 || row_start[m->nblk] != ncol)
    return fail(DFM2G_ERR_PATTERN, "set_pattern: row_start[0] must be 0 and row_start[nblk] == ncol");
  if (ncol && !col) return fail(DFM2G_ERR_ARG, "set_pattern: null col");
  std::vector<unsigned> mark(m->nblk, 0xFFFFFFFFu);
  for (unsigned i = 0; i < m->nblk; ++i) {
    if (row_start[i + 1] < row_start[i]) return fail(DFM2G_ERR_PATTERN, "set_pattern: row_start decreases at %u", i);
    for (unsigned s = row_start[i]; s < row_start[i + 1]; ++s) {
      const unsigned j = col[s];
      if (j >= m->nblk) return fail(DFM2G_ERR_PATTERN, "set_pattern: column %u out of range in row %u", j, i);
      if (j == i) return fail(DFM2G_ERR_PATTERN, "set_pattern: row %u lists its own diagonal block", i);
      if (mark[j] == i) return fail(DFM2G_ERR_PATTERN, "set_pattern: duplicate column %u in row %u", j, i);
      mark[j] = i;
    }
  }
  DFM2G_TRY(ensure_context());
  m->nnz = ncol;
  m->h_row_start.assign(row_start, row_start + m->nblk + 1);
  m->h_col.assign(col, col + ncol);
  DFM2G_TRY(m->row_start.resize(m->nblk + 1));
  // slack past the last element: bulk copies round their byte range up to 16 B
  const size_t bb = (size_t)m->ndim * m->ndim;
  DFM2G_TRY(m->col.resize(ncol + 8));
  DFM2G_TRY(m->vcrs.resize(ncol * bb + 4));
  DFM2G_TRY(m->vdia.resize((size_t)m->nblk * bb + 4));
  DFM2G_CUDA(cudaMemcpyAsync(m->row_start.p, row_start, sizeof(unsigned) * (m->nblk + 1), cudaMemcpyHostToDevice,
                             stream()));
  if (ncol) DFM2G_CUDA(cudaMemcpyAsync(m->col.p, col, sizeof(unsigned) * ncol, cudaMemcpyHostToDevice, stream()));
  DFM2G_CUDA(cudaMemsetAsync(m->vcrs.p, 0, sizeof(double) * (ncol * bb + 1), stream()));
  DFM2G_CUDA(cudaMemsetAsync(m->vdia.p, 0, sizeof(double) * ((size_t)m->nblk * bb + 1), stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  m->has_pattern = true;
  m->f32_valid = false;
  m->pattern_version++;
  m->tiles_ok = false;
  if (m->ndim == 3) DFM2G_TRY(bsr_tiles_build(m));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_info(dfm2g_bsr m, unsigned *nblk, size_t *nnz) try {
  DFM2G_TRY(check_bsr(m, false));
  if (nblk) *nblk = m->nblk;
  if (nnz) *nnz = m->nnz;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_ndim(dfm2g_bsr m, unsigned *ndim) try {
  DFM2G_TRY(check_bsr(m, false));
  if (!ndim) return fail(DFM2G_ERR_ARG, "bsr_ndim: null out");
  *ndim = m->ndim;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_set_zero(dfm2g_bsr m) try {
  DFM2G_TRY(check_bsr(m));
  const size_t bb = (size_t)m->ndim * m->ndim;
  DFM2G_CUDA(cudaMemsetAsync(m->vcrs.p, 0, sizeof(double) * m->nnz * bb, stream()));
  DFM2G_CUDA(cudaMemsetAsync(m->vdia.p, 0, sizeof(double) * m->nblk * bb, stream()));
  m->f32_valid = false;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_set_values(dfm2g_bsr m, const double *vcrs, const double *vdia, int mem) try {
  DFM2G_TRY(check_bsr(m));
  const cudaMemcpyKind k = mem == DFM2G_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  const size_t bb = (size_t)m->ndim * m->ndim;
  if (vcrs && m->nnz) DFM2G_CUDA(cudaMemcpyAsync(m->vcrs.p, vcrs, sizeof(double) * bb * m->nnz, k, stream()));
  if (vdia && m->nblk) DFM2G_CUDA(cudaMemcpyAsync(m->vdia.p, vdia, sizeof(double) * bb * m->nblk, k, stream()));
  if (mem == DFM2G_MEM_HOST) DFM2G_CUDA(cudaStreamSynchronize(stream()));
  m->f32_valid = false;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_get_values(dfm2g_bsr m, double *vcrs, double *vdia, int mem) try {
  DFM2G_TRY(check_bsr(m));
  const cudaMemcpyKind k = mem == DFM2G_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  const size_t bb = (size_t)m->ndim * m->ndim;
  if (vcrs && m->nnz) DFM2G_CUDA(cudaMemcpyAsync(vcrs, m->vcrs.p, sizeof(double) * bb * m->nnz, k, stream()));
  if (vdia && m->nblk) DFM2G_CUDA(cudaMemcpyAsync(vdia, m->vdia.p, sizeof(double) * bb * m->nblk, k, stream()));
  if (mem == DFM2G_MEM_HOST) DFM2G_CUDA(cudaStreamSynchronize(stream()));
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_set_fixed_bc(dfm2g_bsr m, const int *bc, int mem) try {
  DFM2G_TRY(check_bsr(m));
  if (!bc) return fail(DFM2G_ERR_ARG, "set_fixed_bc: null bc");
  VecArg<int> a;
  DFM2G_TRY(a.in(bc, (size_t)m->nblk * m->ndim, mem, true));
  const unsigned blocks = blocks_for((size_t)m->nblk * 32, 256, ctx().num_sms * 16);
  if (m->ndim == 3)
    k_bsr_fixed_bc<<<blocks, 256, 0, stream()>>>(m->nblk, m->row_start.p, m->col.p, m->vcrs.p, m->vdia.p, a.dev());
  else
    k_nd_fixed_bc<<<blocks, 256, 0, stream()>>>(m->nblk, m->ndim, m->row_start.p, m->col.p, m->vcrs.p, m->vdia.p,
                                                a.dev());
  DFM2G_LAUNCH_CHECK();
  if (mem == DFM2G_MEM_HOST) DFM2G_CUDA(cudaStreamSynchronize(stream()));
  m->f32_valid = false;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_add_dia(dfm2g_bsr m, double eps) try {
  DFM2G_TRY(check_bsr(m));
  k_add_dia<<<blocks_for(m->nblk, 256, ctx().num_sms * 8), 256, 0, stream()>>>(m->nblk, m->ndim, m->vdia.p, eps);
  DFM2G_LAUNCH_CHECK();
  m->f32_valid = false;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_update_f32(dfm2g_bsr m) try {
  DFM2G_TRY(check_bsr(m));
  m->f32_valid = false;
  return bsr_ensure_f32(m);
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_matvec(dfm2g_bsr m, int prec, void *y, double alpha, const void *x, double beta, int mem) try {
  DFM2G_TRY(check_bsr(m));
  if (!y || !x) return fail(DFM2G_ERR_ARG, "matvec: null vector");
  const size_t n = (size_t)m->nblk * m->ndim;
  if (prec == DFM2G_F64) {
    VecArg<double> ay, ax;
    DFM2G_TRY(ay.in((double *)y, n, mem, true));
    DFM2G_TRY(ax.in((const double *)x, n, mem, true));
    DFM2G_TRY(bsr_spmv(m, prec, ay.dev(), alpha, ax.dev(), beta));
    DFM2G_TRY(bsr_check_err(m));
    return ay.copy_back();
  }
  if (prec == DFM2G_F32) {
    VecArg<float> ay, ax;
    DFM2G_TRY(ay.in((float *)y, n, mem, true));
    DFM2G_TRY(ax.in((const float *)x, n, mem, true));
    DFM2G_TRY(bsr_spmv(m, prec, ay.dev(), alpha, ax.dev(), beta));
    DFM2G_TRY(bsr_check_err(m));
    return ay.copy_back();
  }
  return fail(DFM2G_ERR_ARG, "matvec: prec must be DFM2G_F64 or DFM2G_F32");
} catch (...) {
  return host_failure();
}

int dfm2g_vec_zero_bc(double *b, const int *bc, size_t ndof, int mem) try {
  if (!b || !bc) return fail(DFM2G_ERR_ARG, "vec_zero_bc: null argument");
  DFM2G_TRY(ensure_context());
  VecArg<double> ab;
  VecArg<int> af;
  DFM2G_TRY(ab.in(b, ndof, mem, true));
  DFM2G_TRY(af.in(bc, ndof, mem, true));
  k_zero_bc<<<blocks_for(ndof, 256, ctx().num_sms * 8), 256, 0, stream()>>>(ndof, ab.dev(), af.dev());
  DFM2G_LAUNCH_CHECK();
  return ab.copy_back();
} catch (...) {
  return host_failure();
}

int dfm2g_bsr_merge(dfm2g_bsr m, unsigned nelem, unsigned nnoel, const unsigned *elem, const double *emat,
                    int mem) try {
  DFM2G_TRY(check_bsr(m));
  if (nelem == 0) return DFM2G_OK;
  if (!elem || !emat || nnoel == 0) return fail(DFM2G_ERR_ARG, "merge: null argument");
  // Colouring needs the connectivity on the host.
  std::vector<unsigned> h_elem((size_t)nelem * nnoel);
  if (mem == DFM2G_MEM_HOST) {
    std::memcpy(h_elem.data(), elem, h_elem.size() * sizeof(unsigned));
  } else {
    DFM2G_CUDA(cudaMemcpyAsync(h_elem.data(), elem, h_elem.size() * sizeof(unsigned), cudaMemcpyDeviceToHost,
                               stream()));
    DFM2G_CUDA(cudaStreamSynchronize(stream()));
  }
  std::vector<unsigned> by_color, color_start;
  DFM2G_TRY(color_elements(h_elem.data(), nelem, nnoel, m->nblk, by_color, color_start));
  DevBuf<unsigned> d_elem, d_list, d_slot;
  DevBuf<int> d_missing;
  DFM2G_TRY(d_elem.resize(h_elem.size()));
  DFM2G_TRY(d_list.resize(nelem));
  DFM2G_TRY(d_slot.resize((size_t)nelem * nnoel * nnoel));
  DFM2G_TRY(d_missing.resize(1));
  DFM2G_CUDA(cudaMemcpyAsync(d_elem.p, h_elem.data(), h_elem.size() * sizeof(unsigned), cudaMemcpyHostToDevice,
                             stream()));
  DFM2G_CUDA(cudaMemcpyAsync(d_list.p, by_color.data(), nelem * sizeof(unsigned), cudaMemcpyHostToDevice,
                             stream()));
  DFM2G_CUDA(cudaMemsetAsync(d_missing.p, 0, sizeof(int), stream()));
  const unsigned bb = m->ndim * m->ndim;
  VecArg<double> a_emat;
  DFM2G_TRY(a_emat.in(emat, (size_t)nelem * nnoel * nnoel * bb, mem, true));
  const size_t nslot = (size_t)nelem * nnoel * nnoel;
  k_slot_map<<<blocks_for(nslot, 256, ctx().num_sms * 16), 256, 0, stream()>>>(
      nelem, nnoel, d_elem.p, m->row_start.p, m->col.p, d_slot.p, d_missing.p);
  DFM2G_LAUNCH_CHECK();
  int missing = 0;
  DFM2G_CUDA(cudaMemcpyAsync(&missing, d_missing.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  if (missing) return fail(DFM2G_ERR_MISSING_SLOT, "merge: an element block is not in the sparsity pattern");
  for (size_t c = 0; c + 1 < color_start.size(); ++c) {
    const unsigned n = color_start[c + 1] - color_start[c];
    k_merge_color<<<blocks_for((size_t)n * nnoel, 128, ctx().num_sms * 16), 128, 0, stream()>>>(
        n, d_list.p + color_start[c], nnoel, d_elem.p, d_slot.p, a_emat.dev(), bb, m->vcrs.p, m->vdia.p);
    DFM2G_LAUNCH_CHECK();
  }
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  m->f32_valid = false;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

}  // extern "C"

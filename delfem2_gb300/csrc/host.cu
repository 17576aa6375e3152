// Library context, error reporting, and the host-side mesh / pattern helpers.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <new>
#include <numeric>
#include <stdexcept>

#include "common.cuh"

namespace dfm2g {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int fail(int status, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

int host_failure() noexcept {
  char buf[256];
  try {
    throw;
  } catch (const std::bad_alloc &) {
    snprintf(buf, sizeof buf, "host-side failure: out of host memory");
  } catch (const std::exception &e) {
    snprintf(buf, sizeof buf, "host-side failure: %s", e.what());
  } catch (...) {
    snprintf(buf, sizeof buf, "host-side failure: unknown exception");
  }
  try {
    g_last_error = buf;
  } catch (...) {  // no memory left for the message either
  }
  return DFM2G_ERR_HOST;
}

static Context g_ctx;
static std::mutex g_ctx_mutex;

Context &ctx() { return g_ctx; }

int ensure_context() {
  if (g_ctx.device >= 0) return DFM2G_OK;
  std::lock_guard<std::mutex> lock(g_ctx_mutex);
  if (g_ctx.device >= 0) return DFM2G_OK;
  int dev = 0;
  DFM2G_CUDA(cudaGetDevice(&dev));
  int sms = 0;
  DFM2G_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (!g_ctx.stream) {
    DFM2G_CUDA(cudaStreamCreateWithFlags(&g_ctx.own, cudaStreamNonBlocking));
    g_ctx.stream = g_ctx.own;
  }
  g_ctx.num_sms = sms;
  g_ctx.device = dev;
  return DFM2G_OK;
}

// ---- instrumentation --------------------------------------------------------
static std::atomic<unsigned long long> g_launches{0};
static bool g_prof_on = false;
struct ProfSample {
  int kind;
  cudaEvent_t a, b;
};
static std::vector<ProfSample> g_prof_pending;
static std::vector<cudaEvent_t> g_event_pool;
static unsigned g_prof_count[DFM2G_PROF_NKIND];
static double g_prof_ms[DFM2G_PROF_NKIND];

static std::atomic<unsigned long long> g_allocs{0};

void note_launches(unsigned n) { g_launches += n; }
void note_alloc() { g_allocs += 1; }

static cudaEvent_t take_event() {
  if (!g_event_pool.empty()) {
    cudaEvent_t e = g_event_pool.back();
    g_event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

static void drain_prof() {
  if (g_prof_pending.empty()) return;
  cudaStreamSynchronize(stream());
  for (auto &s : g_prof_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, s.a, s.b) == cudaSuccess) {
      g_prof_count[s.kind]++;
      g_prof_ms[s.kind] += ms;
    }
    g_event_pool.push_back(s.a);
    g_event_pool.push_back(s.b);
  }
  g_prof_pending.clear();
}

ProfScope::ProfScope(int k, unsigned launches) : kind(k), n(launches), on(g_prof_on) {
  if (on) {
    a = take_event();
    b = take_event();
    cudaEventRecord(a, stream());
  }
}

ProfScope::~ProfScope() {
  note_launches(n);
  if (on) {
    cudaEventRecord(b, stream());
    g_prof_pending.push_back({kind, a, b});
    if (g_prof_pending.size() > 4096) drain_prof();
  }
}

}  // namespace dfm2g

using namespace dfm2g;

extern "C" {

int dfm2g_version(void) { return 100; }

int dfm2g_profile_enable(int on) try {
  DFM2G_TRY(ensure_context());
  drain_prof();
  g_prof_on = on != 0;
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_profile_reset(void) try {
  drain_prof();
  for (int k = 0; k < DFM2G_PROF_NKIND; ++k) {
    g_prof_count[k] = 0;
    g_prof_ms[k] = 0.0;
  }
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_profile_read(int kind, unsigned *launches, double *total_ms) try {
  if (kind < 0 || kind >= DFM2G_PROF_NKIND) return fail(DFM2G_ERR_ARG, "unknown profile kind %d", kind);
  drain_prof();
  if (launches) *launches = g_prof_count[kind];
  if (total_ms) *total_ms = g_prof_ms[kind];
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_launch_count(unsigned long long *count) try {
  if (!count) return fail(DFM2G_ERR_ARG, "null count");
  *count = g_launches.load();
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_alloc_count(unsigned long long *count) try {
  if (!count) return fail(DFM2G_ERR_ARG, "null count");
  *count = g_allocs.load();
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

const char *dfm2g_status_string(int s) {
  switch (s) {
    case DFM2G_OK: return "ok";
    case DFM2G_ERR_ARG: return "invalid argument";
    case DFM2G_ERR_CUDA: return "CUDA error";
    case DFM2G_ERR_MISSING_SLOT: return "merge target block not in the sparsity pattern";
    case DFM2G_ERR_SINGULAR_PIVOT: return "ILU: more than 10 singular pivots";
    case DFM2G_ERR_NOT_CONVERGED: return "iteration limit reached before the tolerance";
    case DFM2G_ERR_WAIT_TIMEOUT: return "bounded device-side wait timed out";
    case DFM2G_ERR_PATTERN: return "invalid sparsity pattern";
    case DFM2G_ERR_UNSUPPORTED: return "unsupported block size or mode";
    case DFM2G_ERR_STATE: return "call order violated";
    case DFM2G_ERR_NONFINITE: return "non-finite value in a solve";
    case DFM2G_ERR_HOST: return "host-side failure (host memory or thread)";
    default: return "unknown status";
  }
}

const char *dfm2g_last_error(void) { return g_last_error.c_str(); }

int dfm2g_set_stream(void *s) try {
  DFM2G_TRY(ensure_context());
  // NULL is CUDA's legacy default stream (torch's default stream), not the
  // library's own non-blocking stream: work must order with the caller's.
  g_ctx.stream = static_cast<cudaStream_t>(s);
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_synchronize(void) try {
  DFM2G_TRY(ensure_context());
  DFM2G_CUDA(cudaStreamSynchronize(g_ctx.stream));
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

// Lattice node (ix,iy,iz) -> ix*(ny+1)*(nz+1) + iy*(nz+1) + iz; six tets per
// voxel around the corner-0 / corner-6 diagonal (gridvoxel.cpp:194-271).
int dfm2g_mesh_tet_voxel_grid(unsigned nx, unsigned ny, unsigned nz, double scale, double *xyz,
                              unsigned *tet) try {
  if (!xyz || !tet) return fail(DFM2G_ERR_ARG, "mesh: null output");
  const size_t my = ny + 1, mz = nz + 1;
  size_t p = 0;
  for (unsigned ix = 0; ix <= nx; ++ix)
    for (unsigned iy = 0; iy <= ny; ++iy)
      for (unsigned iz = 0; iz <= nz; ++iz, ++p) {
        xyz[p * 3 + 0] = ix * scale;
        xyz[p * 3 + 1] = iy * scale;
        xyz[p * 3 + 2] = iz * scale;
      }
  static const unsigned dxyz[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                      {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  static const int six[6][4] = {{0, 1, 2, 6}, {0, 1, 6, 5}, {0, 4, 5, 6},
                                {0, 2, 3, 6}, {0, 3, 7, 6}, {0, 4, 6, 7}};
  size_t t = 0;
  for (unsigned vx = 0; vx < nx; ++vx)
    for (unsigned vy = 0; vy < ny; ++vy)
      for (unsigned vz = 0; vz < nz; ++vz) {
        unsigned c[8];
        for (int k = 0; k < 8; ++k)
          c[k] = (unsigned)((vx + dxyz[k][0]) * my * mz + (vy + dxyz[k][1]) * mz + (vz + dxyz[k][2]));
        for (int s = 0; s < 6; ++s, ++t)
          for (int k = 0; k < 4; ++k) tet[t * 4 + k] = c[six[s][k]];
      }
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

// Elements-around-point then a marker sweep (self marked first, so excluded).
static int psup_impl(const unsigned *elem, size_t nelem, unsigned nnoel, size_t np,
                     unsigned *psup_ind, unsigned *psup) {
  std::vector<unsigned> eind(np + 1, 0);
  for (size_t e = 0; e < nelem; ++e)
    for (unsigned k = 0; k < nnoel; ++k) {
      const unsigned n = elem[e * nnoel + k];
      if (n >= np) return fail(DFM2G_ERR_ARG, "psup: element %zu names node %u >= np", e, n);
      eind[n + 1]++;
    }
  for (size_t p = 0; p < np; ++p) eind[p + 1] += eind[p];
  std::vector<unsigned> elsup(eind[np]);
  {
    std::vector<unsigned> cur(eind.begin(), eind.end() - 1);
    for (size_t e = 0; e < nelem; ++e)
      for (unsigned k = 0; k < nnoel; ++k) elsup[cur[elem[e * nnoel + k]]++] = (unsigned)e;
  }
  std::vector<unsigned> mark(np, 0xFFFFFFFFu);
  size_t total = 0;
  if (!psup) psup_ind[0] = 0;
  for (size_t p = 0; p < np; ++p) {
    mark[p] = (unsigned)p;
    size_t w = psup ? psup_ind[p] : 0;
    unsigned cnt = 0;
    for (unsigned q = eind[p]; q < eind[p + 1]; ++q) {
      const unsigned e = elsup[q];
      for (unsigned k = 0; k < nnoel; ++k) {
        const unsigned n = elem[(size_t)e * nnoel + k];
        if (mark[n] == p) continue;
        mark[n] = (unsigned)p;
        if (psup) psup[w++] = n;
        ++cnt;
      }
    }
    if (psup) {
      std::sort(psup + psup_ind[p], psup + psup_ind[p + 1]);
    } else {
      total += cnt;
      if (total > 0xFFFFFFFFull) return fail(DFM2G_ERR_ARG, "psup: more than 2^32 entries");
      psup_ind[p + 1] = (unsigned)total;
    }
  }
  return DFM2G_OK;
}

int dfm2g_psup_count(const unsigned *elem, size_t nelem, unsigned nnoel, size_t np,
                     unsigned *psup_ind, size_t *npsup) try {
  if (!elem || !psup_ind || !npsup || nnoel == 0) return fail(DFM2G_ERR_ARG, "psup_count: null argument");
  DFM2G_TRY(psup_impl(elem, nelem, nnoel, np, psup_ind, nullptr));
  *npsup = psup_ind[np];
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_psup_fill(const unsigned *elem, size_t nelem, unsigned nnoel, size_t np,
                    const unsigned *psup_ind, unsigned *psup) try {
  if (!elem || !psup_ind || nnoel == 0) return fail(DFM2G_ERR_ARG, "psup_fill: null argument");
  if (psup_ind[np] > 0 && !psup) return fail(DFM2G_ERR_ARG, "psup_fill: null psup");
  return psup_impl(elem, nelem, nnoel, np, const_cast<unsigned *>(psup_ind), psup);
} catch (...) {
  return host_failure();
}

// A kernel that waits for a value nobody writes: the wait must give up after
// `timeout_ns`, record the timeout and return.
__global__ void k_wait_never(const double *never, int *status, unsigned long long timeout_ns) {
  const unsigned long long t0 = globaltimer_ns();
  while (is_pending(ld_relaxed(never))) {
    if (globaltimer_ns() - t0 > timeout_ns) {
      atomicExch(status, DFM2G_ERR_WAIT_TIMEOUT);
      return;
    }
  }
  atomicExch(status, DFM2G_OK);
}

// Two grid_barrier rounds over the same words (cooperative launch); with
// `absent` the last CTA returns without arriving, so the others must give up
// after `timeout_ns` and record the timeout.
__global__ void k_grid_barrier_probe(unsigned *bar, int *err, int *status, unsigned long long timeout_ns,
                                     int absent) {
  if (absent && blockIdx.x == gridDim.x - 1) return;
  bool ok = grid_barrier(bar, err, timeout_ns);
  if (ok) ok = grid_barrier(bar, err, timeout_ns);
  if (threadIdx.x == 0 && !ok) atomicExch(status, DFM2G_ERR_WAIT_TIMEOUT);
}

int dfm2g_debug_wait_timeout(unsigned timeout_ms) try {
  DFM2G_TRY(ensure_context());
  if (timeout_ms == 0 || timeout_ms > 5000) return fail(DFM2G_ERR_ARG, "timeout_ms must be in [1, 5000]");
  DevBuf<double> never;
  DevBuf<int> st;
  DFM2G_TRY(never.resize(1));
  DFM2G_TRY(st.resize(1));
  DFM2G_CUDA(cudaMemsetAsync(never.p, 0xFF, sizeof(double), stream()));
  DFM2G_CUDA(cudaMemsetAsync(st.p, 0xFF, sizeof(int), stream()));
  k_wait_never<<<1, 1, 0, stream()>>>(never.p, st.p, 1000000ull * timeout_ms);
  DFM2G_LAUNCH_CHECK();
  int h = -1;
  DFM2G_CUDA(cudaMemcpyAsync(&h, st.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  if (h == DFM2G_ERR_WAIT_TIMEOUT) return fail(DFM2G_ERR_WAIT_TIMEOUT, "debug wait timed out after %u ms", timeout_ms);
  return h;
} catch (...) {
  return host_failure();
}

int dfm2g_debug_grid_barrier(unsigned timeout_ms, int one_block_absent) try {
  DFM2G_TRY(ensure_context());
  if (timeout_ms == 0 || timeout_ms > 5000) return fail(DFM2G_ERR_ARG, "timeout_ms must be in [1, 5000]");
  DevBuf<unsigned> bar;
  DevBuf<int> err, st;
  DFM2G_TRY(bar.resize(2));
  DFM2G_TRY(err.resize(1));
  DFM2G_TRY(st.resize(1));
  DFM2G_CUDA(cudaMemsetAsync(bar.p, 0, 2 * sizeof(unsigned), stream()));
  DFM2G_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), stream()));
  DFM2G_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), stream()));
  unsigned long long timeout_ns = 1000000ull * timeout_ms;
  int absent = one_block_absent ? 1 : 0;
  unsigned *pb = bar.p;
  int *pe = err.p, *ps = st.p;
  void *args[] = {(void *)&pb, (void *)&pe, (void *)&ps, (void *)&timeout_ns, (void *)&absent};
  DFM2G_CUDA(cudaLaunchCooperativeKernel((void *)k_grid_barrier_probe, dim3(4), dim3(64), args, 0, stream()));
  note_launches(1);
  int h = -1, e = -1;
  DFM2G_CUDA(cudaMemcpyAsync(&h, st.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream()));
  DFM2G_CUDA(cudaStreamSynchronize(stream()));
  if (h == DFM2G_ERR_WAIT_TIMEOUT && e == DFM2G_ERR_WAIT_TIMEOUT)
    return fail(DFM2G_ERR_WAIT_TIMEOUT, "debug grid barrier timed out after %u ms", timeout_ms);
  if (h != DFM2G_OK || e != DFM2G_OK) return fail(DFM2G_ERR_STATE, "debug grid barrier: status %d, error word %d", h, e);
  return DFM2G_OK;
} catch (...) {
  return host_failure();
}

int dfm2g_debug_host_failure(int kind) try {
  if (kind == 0) throw std::bad_alloc();
  if (kind == 1) throw std::runtime_error("debug exception");
  throw kind;
} catch (...) {
  return host_failure();
}

}  // extern "C"

// PageRank (reference semantics) over a caller-owned device CSC, without a
// single device allocation.
//
// Some callers cannot call cudaMalloc: a plugin running inside a host
// application whose allocator owns all device memory, a serving path that
// forbids allocation per request, or code that runs while the caller has
// reserved the whole device for its own pool.  For them this file keeps the
// superstep loop's scratch (control block, step records, work cursors, the
// second rank buffer, contribution buffers, frontier bitmap, warp work units)
// in one file-scope __device__ array of fixed size.  Every GPU that loads the
// library holds that array until the process exits.
//
// The kernels are the engine's own pull/finalize kernels (gx_kernels.cuh);
// only where their scratch lives differs.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "gx_internal.h"
#include "gx_kernels.cuh"

using namespace gx;

namespace {

constexpr int32_t kNoAllocMaxVertices = 1 << 20;
constexpr int32_t kNoAllocMaxSteps = 1024;
constexpr int32_t kNoAllocUnits = (kNoAllocMaxVertices + 31) / 32;
constexpr int32_t kNoAllocWords = kNoAllocMaxVertices / 32 + 2;
constexpr int32_t kNoAllocWork = kQueues + 64;

struct NoAllocScratch {
  Ctl ctl;
  StepStats stats[kNoAllocMaxSteps];
  unsigned int work[kNoAllocWork];
  unsigned int hticket[4];
  float partial[4];
  int4 heavy[1];
  int2 units[kNoAllocUnits];
  int32_t unit_shard[kNoAllocUnits];
  uint32_t bm[kNoAllocWords];
  float val1[kNoAllocMaxVertices];
  float con[2][kNoAllocMaxVertices];
};

// The scratch.  In host code this name is only a host-side handle: its
// device address comes from cudaGetSymbolAddress, per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

std::mutex g_setup_mu;
NoAllocScratch* g_scratch_addr[64] = {};

// Device address of the scratch on the current device; looked up once per
// device (with that device current) and cached for the life of the process.
// cudaDeviceReset destroys the module instance the cached address points
// into, so the entry point must not be called after a reset.
gx_status scratch_on_current_device(NoAllocScratch** out) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return fail(GX_ERR_NODEVICE, "gx_pagerank_noalloc: no current device: %s",
                                      cudaGetErrorString(err));
  if (dev < 0 || dev >= 64) return fail(GX_ERR_INVALID, "gx_pagerank_noalloc: device ordinal %d >= 64", dev);
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess || !p)
      return fail(GX_ERR_CUDA, "gx_pagerank_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(err));
    g_scratch_addr[dev] = static_cast<NoAllocScratch*>(p);
  }
  *out = g_scratch_addr[dev];
  return GX_OK;
}

__global__ void noalloc_setup_kernel(NoAllocScratch* s, int32_t V, int32_t max_iter, double damping) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = gridDim.x * blockDim.x;
  if (tid == 0) {
    Ctl c{};
    c.max_iter = max_iter;
    c.n_vertices = V;
    c.n_shards = 1;
    c.shard_words = 1;
    c.push_ok = 0;
    c.damping = damping;
    c.inv_n = 1.0 / V;
    c.fx_scale = static_cast<double>(V) * 1073741824.0;
    c.tolerance = 0;
    c.sel_threshold = 0.001;
    c.mode = MODE_DENSE;
    s->ctl = c;
  }
  const int32_t U = (V + 31) / 32;
  for (int i = tid; i < U; i += nt) {
    s->units[i] = make_int2(32 * i, 32 * i + 32 < V ? 32 * i + 32 : V);
    s->unit_shard[i] = 0;
  }
  for (int i = tid; i < kNoAllocWords; i += nt) s->bm[i] = 0;
  for (int i = tid; i < kNoAllocWork; i += nt) s->work[i] = 0;
  for (int i = tid; i < 4; i += nt) s->hticket[i] = 0;
}

// The caller's CSC, checked before any kernel indexes with it: off[0] == 0,
// off non-decreasing, off[V] == num_edges and every source id in [0, V).
// A failure marks the run done with error 3, so the pull and finalize
// launches queued behind this one return at once.
__global__ void noalloc_validate_kernel(NoAllocScratch* s, const int64_t* off, const int32_t* col, int32_t V,
                                        int64_t E) {
  const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t nt = static_cast<int64_t>(gridDim.x) * blockDim.x;
  bool bad = tid == 0 && (off[0] != 0 || off[V] != E);
  for (int64_t v = tid; v < V && !bad; v += nt) bad = off[v] > off[v + 1];
  for (int64_t k = tid; k < E && !bad; k += nt) bad = col[k] < 0 || col[k] >= V;
  if (bad) {
    atomicOr(&s->ctl.error, 3);
    s->ctl.done = 1;
  }
}

// The final ranks sit in whichever buffer the last swap left current.
__global__ void noalloc_result_kernel(NoAllocScratch* s, float* rank, int32_t V) {
  if (s->ctl.cur == 0) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x) rank[i] = s->val1[i];
}

}  // namespace

extern "C" gx_status gx_pagerank_noalloc(const int64_t* d_off, const int32_t* d_col, int64_t num_edges,
                                         int64_t col_capacity, const int32_t* d_outdeg, int32_t V, int32_t max_iter,
                                         double damping, float* d_rank, void* stream, int32_t* iterations_out) {
  if (!d_off || !d_outdeg || !d_rank || (num_edges > 0 && !d_col))
    return fail(GX_ERR_INVALID, "gx_pagerank_noalloc: NULL device pointer");
  if (V < 1 || V > kNoAllocMaxVertices)
    return fail(GX_ERR_INVALID, "gx_pagerank_noalloc: V=%d outside [1, %d], the size of the built-in scratch", V,
                kNoAllocMaxVertices);
  if (max_iter < 1 || max_iter > kNoAllocMaxSteps)
    return fail(GX_ERR_INVALID, "gx_pagerank_noalloc: max_iter=%d outside [1, %d]", max_iter, kNoAllocMaxSteps);
  if (num_edges < 0 || col_capacity < num_edges + 4)
    return fail(GX_ERR_INVALID,
                "gx_pagerank_noalloc: col must hold num_edges + 4 entries (128-bit index loads read up to 3 past "
                "the last edge); got capacity %lld for %lld edges",
                static_cast<long long>(col_capacity), static_cast<long long>(num_edges));
  if ((reinterpret_cast<uintptr_t>(d_col) & 15) || (reinterpret_cast<uintptr_t>(d_off) & 7))
    return fail(GX_ERR_INVALID, "gx_pagerank_noalloc: col must be 16-byte aligned and off 8-byte aligned");
  NoAllocScratch* s = nullptr;
  gx_status st = scratch_on_current_device(&s);
  if (st != GX_OK) return st;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  int dev = 0, n_sm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  void (*pull)(PullArgs) = pull_kernel<K_PR_REF, false>;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(pull), kThreads, 0);
  const int grid_pull = (per_sm > 0 ? per_sm : 1) * n_sm;
  const int32_t U = (V + 31) / 32;
  const int n_words = V / 32 + 2;
  const int grid_fin = std::max(1, std::min(n_sm * 4, (n_words + kThreads - 1) / kThreads));

  noalloc_setup_kernel<<<std::max(1, std::min(n_sm * 4, (U + 255) / 256)), 256, 0, cs>>>(s, V, max_iter, damping);
  noalloc_validate_kernel<<<n_sm * 4, 256, 0, cs>>>(s, d_off, d_col, V, num_edges);
  init_kernel<K_PR_REF><<<n_sm * 4, 256, 0, cs>>>(&s->ctl, d_rank, s->con[0], d_outdeg, V, 0, 0);

  PullArgs pa{};
  pa.ctl = &s->ctl;
  pa.off = d_off;
  pa.col = d_col;
  pa.w = nullptr;
  pa.outdeg = d_outdeg;
  pa.val[0] = d_rank;
  pa.val[1] = s->val1;
  pa.con[0] = s->con[0];
  pa.con[1] = s->con[1];
  pa.units = s->units;
  pa.unit_shard = s->unit_shard;
  pa.u_begin = 0;
  pa.u_end = U;
  pa.heavy = s->heavy;
  pa.partial = s->partial;
  pa.hticket = s->hticket;
  pa.ctr = s->work;
  pa.heavy_deg = INT32_MAX;  // no chunked vertices: long lists are swept by the tile's warp
  pa.bm = s->bm;
  FinArgs fa{};
  fa.ctl = &s->ctl;
  fa.stats = s->stats;
  fa.bm = s->bm;
  fa.n_words = n_words;
  fa.val[0] = d_rank;
  fa.val[1] = s->val1;
  fa.outdeg = nullptr;
  fa.frontier = nullptr;  // never written: push steps are off
  fa.frontier_cap = 0;
  fa.work_ctr = s->work;
  fa.n_work_ctr = kNoAllocWork;
  // Steps after termination return at once; no host round trip per step.
  for (int i = 0; i < max_iter; ++i) {
    pull<<<grid_pull, kThreads, 0, cs>>>(pa);
    finalize_kernel<K_PR_REF><<<grid_fin, kThreads, 0, cs>>>(fa);
  }
  noalloc_result_kernel<<<n_sm * 4, 256, 0, cs>>>(s, d_rank, V);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(GX_ERR_CUDA, "gx_pagerank_noalloc: launch failed: %s", cudaGetErrorString(err));
  if (iterations_out) {
    Ctl c{};
    err = cudaMemcpyAsync(&c, &s->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, cs);
    if (err == cudaSuccess) err = cudaStreamSynchronize(cs);
    if (err != cudaSuccess) return fail(GX_ERR_CUDA, "gx_pagerank_noalloc: %s", cudaGetErrorString(err));
    *iterations_out = c.step;
    if (c.error == 3)
      return fail(GX_ERR_INVALID,
                  "gx_pagerank_noalloc: the CSC failed its device-side checks (off[0] == 0, off non-decreasing, "
                  "off[V] == num_edges, source ids in [0, V)); no superstep ran");
    if (c.error != 0) return fail(GX_ERR_CUDA, "gx_pagerank_noalloc: device error %d", c.error);
  }
  return GX_OK;
}

// The engine object behind the C ABI and helpers shared by its translation
// units (superstep loop, triangle counting, batched runs, PPR, warm start).
#pragma once
#include <cuda_runtime.h>

#include <cstring>
#include <memory>
#include <utility>
#include <vector>

#include "gx_internal.h"
#include "gx_kernels.cuh"

#define GX_CUDA(call)                                                                                   \
  do {                                                                                                  \
    cudaError_t err_ = (call);                                                                          \
    if (err_ != cudaSuccess)                                                                            \
      return fail(err_ == cudaErrorMemoryAllocation ? GX_ERR_OOM : GX_ERR_CUDA, "%s:%d %s: %s", __FILE__, \
                  __LINE__, #call, cudaGetErrorString(err_));                                          \
  } while (0)

#define GX_TRY(call)                 \
  do {                               \
    gx_status st_ = (call);          \
    if (st_ != GX_OK) return st_;    \
  } while (0)

namespace gx {

// Device memory of the engines comes from one stream-ordered pool per device
// that keeps freed blocks (release threshold: unlimited), so loading a graph
// after another engine was destroyed maps no new memory and destroying an
// engine unmaps none.  gx_release_cached_memory() trims the pool.  Blocks are
// handed out and returned on a private stream that is synchronised after each
// call.
struct DevicePool {
  cudaMemPool_t pool = nullptr;
  cudaStream_t stream = nullptr;
};
DevicePool* device_pool(int dev);  // nullptr if the device has no pool support
int current_device();

inline cudaError_t pool_malloc(void** p, size_t bytes) {
  DevicePool* dp = device_pool(current_device());
  if (!dp) return cudaMalloc(p, bytes);
  cudaError_t err = cudaMallocFromPoolAsync(p, bytes, dp->pool, dp->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(dp->stream);
  return err;
}

// Frees a block of the pool once no work on the device can still use it
// (a pool block is never freed with cudaFree, which neither waits for that
// work nor goes through the pool's bookkeeping).
inline void pool_free(void* p) {
  if (!p) return;
  DevicePool* dp = device_pool(current_device());
  if (!dp) {
    cudaFree(p);
    return;
  }
  cudaDeviceSynchronize();
  cudaFreeAsync(p, dp->stream);
  cudaStreamSynchronize(dp->stream);
}

template <class T>
gx_status dev_alloc(T** p, size_t n) {
  if (*p) {
    pool_free(*p);
    *p = nullptr;
  }
  if (n == 0) n = 1;
  cudaError_t err = pool_malloc(reinterpret_cast<void**>(p), n * sizeof(T));
  if (err != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(GX_ERR_OOM, "device allocation of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(err));
  }
  return GX_OK;
}

template <class T>
void dev_free(T** p) {
  if (*p) pool_free(*p);
  *p = nullptr;
}

// std::vector storage without value-initialisation: large host arrays are
// filled by parallel loops, which also place their pages.
template <class T>
struct UninitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = UninitAlloc<U>;
  };
  UninitAlloc() = default;
  template <class U>
  UninitAlloc(const UninitAlloc<U>&) noexcept {}
  template <class U>
  void construct(U* ptr) noexcept {
    ::new (static_cast<void*>(ptr)) U;
  }
  template <class U, class... A>
  void construct(U* ptr, A&&... args) {
    ::new (static_cast<void*>(ptr)) U(std::forward<A>(args)...);
  }
};
template <class T>
using hvec = std::vector<T, UninitAlloc<T>>;

// Device sort and scan of the graph build (gx_build.cu), for the engine's
// load-time relabelling.  radix_scratch_sizes gives the element counts of
// the scratch for n keys: `hist` and `offs` hold hist_elems each, `part`
// part_elems.  radix_sort_bits sorts n 64-bit keys stably by bits
// [lo_bit, hi_bit) (8 a pass; keys and tmp alternate, *sorted is the one
// holding the result); scan_u32 writes the exclusive prefix sums of m
// 32-bit counts as 64-bit offsets.  Both only enqueue work on s.
void radix_scratch_sizes(int64_t n, int64_t* hist_elems, int64_t* part_elems);
gx_status radix_sort_bits(unsigned long long* keys, unsigned long long* tmp, int64_t n, int lo_bit, int hi_bit,
                          uint32_t* hist, unsigned long long* offs, unsigned long long* part, cudaStream_t s,
                          unsigned long long** sorted);
gx_status scan_u32(const uint32_t* in, int64_t m, unsigned long long* out, unsigned long long* part, cudaStream_t s);

// What a captured superstep graph depends on: the kernels, their launch
// shapes and their argument bytes (zero-filled before use, padding included).
struct GraphKey {
  int app, k, push;
  const void* pull;
  int grid_pull, threads_pull;
  size_t smem_pull;
  int grid_push, grid_fin;
  PullArgs pa;
  PushArgs qa;
  FinArgs fa;
};

inline int app_kind(const gx_run_params& p) {
  switch (p.app) {
    case GX_APP_PAGERANK_REF: return K_PR_REF;
    case GX_APP_PAGERANK_STD: return K_PR_STD;
    case GX_APP_SSSP: return p.weighted ? K_SSSP_W : K_SSSP_UNIT;
    case GX_APP_CC: return K_CC;
    case GX_APP_INDEGREE: return K_INDEG;
  }
  return -1;
}

}  // namespace gx

struct gx_engine {
  gx_config cfg{};
  int dev = 0;
  int n_sm = 0;
  cudaStream_t s_comp = nullptr, s_copy = nullptr;
  int pageable_access = 0;           // the device reads pageable host memory (cudaDevAttrPageableMemoryAccess)
  std::vector<cudaStream_t> s_copies;  // s_copy first
  bool loaded = false;

  // graph (host side)
  int32_t V = 0, P = 0;
  int64_t E = 0;
  std::vector<int32_t> bounds;
  gx::hvec<int64_t> off;
  gx::hvec<int32_t> outdeg;
  int64_t n_dangling = 0;            // vertices of out-degree 0
  gx::hvec<int2> units;
  gx::hvec<int32_t> unit_shard;
  std::vector<int32_t> unit_begin;  // P+1
  std::vector<int4> heavy;
  int64_t n_partials = 0;

  // shard cache
  std::vector<char> resident;
  std::vector<int64_t> dev_base;    // element offset of a resident shard's slice in d_col
  int32_t n_resident = 0;
  bool all_resident = true;
  int32_t* h_col = nullptr;         // pinned full copy when some shards stream
  uint32_t* h_w = nullptr;
  int64_t slot_elems = 0;
  std::vector<int32_t*> slot_col;
  std::vector<uint32_t*> slot_w;
  std::vector<cudaEvent_t> slot_free, slot_ready;
  int32_t n_slots = 0;

  // Compressed streaming (compress_cache on): each streamed shard is a blob
  // of chunk headers, byte offsets and byte weights (gx_kernels.cuh:
  // comp_idx4) in the pinned h_cblob, copied through slot_blob.
  bool comp = false;                // some streamed shard travels compressed
  bool comp_all = false;            // every streamed shard does
  bool w_narrow = false;            // every weight fits a byte
  uint8_t* h_cblob = nullptr;
  std::vector<int64_t> cb_off, cb_bytes, cb_c0, cb_pay, cb_w8;  // per shard
  std::vector<uint8_t*> slot_blob;
  int64_t comp_bytes = 0;           // all streamed blobs

  // device
  int64_t* d_off = nullptr;
  int32_t* d_col = nullptr;
  uint32_t* d_w = nullptr;
  bool has_weights = false;
  std::vector<uint32_t> w_host;     // kept until the shard plan is fixed
  int32_t* d_outdeg = nullptr;
  void* d_val[2] = {nullptr, nullptr};
  float* d_con[2] = {nullptr, nullptr};
  int2* d_units = nullptr;
  int32_t* d_unit_shard = nullptr;
  int4* d_heavy = nullptr;
  void* d_partial = nullptr;
  unsigned int* d_hticket = nullptr;
  uint32_t* d_bm = nullptr;
  int32_t n_words = 0;
  // Selective steps: shard bounds (P+1), two shard bitmaps marked by the
  // device (resident graphs), the changed-vertex list a streamed step hands
  // to the host and the host's per-vertex shard sets (P bits per vertex,
  // built when a streamed graph is loaded).
  int32_t* d_bounds = nullptr;
  uint32_t* d_shard_bm = nullptr;
  int32_t* d_changed_list = nullptr;
  int64_t changed_cap = 0;
  std::vector<unsigned long long> h_shard_sets;
  int shard_set_words = 0;
  bool out_unbuildable = false;      // vertexout.npy disagrees with the shards: no out-edge CSR
  int4* d_frontier = nullptr;
  unsigned long long frontier_cap = 0;
  int64_t* d_ooff = nullptr;
  int32_t* d_ocol = nullptr;
  uint32_t* d_ow = nullptr;
  bool out_built = false, out_weighted = false;
  gx::Ctl* d_ctl = nullptr;
  gx::Ctl* h_ctl = nullptr;
  gx::StepStats* d_stats = nullptr;
  int32_t stats_cap = 0;
  unsigned int* d_work = nullptr;
  int32_t n_work = 0;

  // Relabelled engine (config.relabel): the caller's vertex v is the
  // engine's vertex perm[v] (h_perm on the host, d_perm on the device), and
  // the engine's vertex i is the caller's d_inv[i].  d_off_old keeps the
  // caller's offsets for gx_set_weights; d_stage carries values between the
  // two numberings.  e->off and e->outdeg are in the engine's numbering.
  bool relabeled = false;
  gx::hvec<int32_t> h_perm;
  int32_t* d_perm = nullptr;
  int32_t* d_inv = nullptr;
  int64_t* d_off_old = nullptr;
  uint32_t* d_stage = nullptr;

  std::vector<uint32_t> init_vals;
  bool has_init = false;
  bool device_init = false;          // next gx_run starts from d_val[0] as it is
  double device_init_dangling = 0;   // PageRank STD: its dangling mass
  double last_uniform_resid = 0;     // warm start: uniform start's first-step L1 residual

  // last run
  gx_app last_app = GX_APP_PAGERANK_REF;
  bool last_weighted = false;
  int32_t last_steps = 0;
  std::vector<gx::StepStats> last_stats;
  gx_run_stats last_run{};

  // Executable superstep graphs of earlier runs, keyed by GraphKey bytes.
  std::vector<std::pair<gx::GraphKey, cudaGraphExec_t>> graphs;

  cudaGraphExec_t cached_graph(const gx::GraphKey& k) const {
    for (const auto& g : graphs)
      if (memcmp(&g.first, &k, sizeof(k)) == 0) return g.second;
    return nullptr;
  }
  void keep_graph(const gx::GraphKey& k, cudaGraphExec_t x) {
    if (graphs.size() >= 16) drop_graphs();
    graphs.emplace_back(k, x);
  }
  void drop_graphs() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    graphs.clear();
  }

  ~gx_engine() { release(); }

  void release_graph() {
    // Pool frees do not wait for the device: let this engine's work finish.
    if (s_comp) cudaStreamSynchronize(s_comp);
    for (cudaStream_t cs : s_copies) cudaStreamSynchronize(cs);
    gx::dev_free(&d_off);
    gx::dev_free(&d_col);
    gx::dev_free(&d_w);
    gx::dev_free(&d_outdeg);
    for (int i = 0; i < 2; ++i) {
      gx::dev_free(&d_val[i]);
      gx::dev_free(&d_con[i]);
    }
    gx::dev_free(&d_units);
    gx::dev_free(&d_unit_shard);
    gx::dev_free(&d_heavy);
    gx::dev_free(&d_partial);
    gx::dev_free(&d_hticket);
    gx::dev_free(&d_bm);
    gx::dev_free(&d_perm);
    gx::dev_free(&d_inv);
    gx::dev_free(&d_off_old);
    gx::dev_free(&d_stage);
    relabeled = false;
    h_perm.clear();
    gx::dev_free(&d_bounds);
    gx::dev_free(&d_shard_bm);
    gx::dev_free(&d_changed_list);
    changed_cap = 0;
    h_shard_sets.clear();
    h_shard_sets.shrink_to_fit();
    shard_set_words = 0;
    out_unbuildable = false;
    gx::dev_free(&d_frontier);
    gx::dev_free(&d_ooff);
    gx::dev_free(&d_ocol);
    gx::dev_free(&d_ow);
    gx::dev_free(&d_stats);
    gx::dev_free(&d_work);
    for (auto p : slot_col) gx::pool_free(p);
    for (auto p : slot_w) gx::pool_free(p);
    for (auto p : slot_blob) gx::pool_free(p);
    slot_col.clear();
    slot_w.clear();
    slot_blob.clear();
    if (h_cblob) cudaFreeHost(h_cblob);
    h_cblob = nullptr;
    comp = false;
    for (auto ev : slot_free) cudaEventDestroy(ev);
    for (auto ev : slot_ready) cudaEventDestroy(ev);
    slot_free.clear();
    slot_ready.clear();
    if (h_col) cudaFreeHost(h_col);
    if (h_w) cudaFreeHost(h_w);
    h_col = nullptr;
    h_w = nullptr;
    out_built = false;
    has_weights = false;
    loaded = false;
    stats_cap = 0;
  }

  void release() {
    cudaSetDevice(dev);
    release_graph();
    drop_graphs();
    gx::dev_free(&d_ctl);
    if (h_ctl) cudaFreeHost(h_ctl);
    h_ctl = nullptr;
    if (s_comp) cudaStreamDestroy(s_comp);
    for (cudaStream_t cs : s_copies) cudaStreamDestroy(cs);
    s_copies.clear();
    s_comp = s_copy = nullptr;
  }
};


// The engine behind the C ABI: GraphPS<T> (GraphMP/system/GraphPS.h:22-387)
// re-designed for one GB300.
//
// HBM layout (all-resident case):
//   off     int64[V+1]   global CSC offsets (the shards' indptr, rebased)
//   col     int32[E+8]   source ids, shards laid end to end (the shards' indices)
//   w       uint32[E+8]  SSSP weights aligned with col (optional)
//   outdeg  int32[V]     vertexout.npy
//   val     T[2][V]      Msg / MsgNew as a double buffer (swap instead of copy)
//   con     f32[2][V]    PageRank contributions Msg[u]/outdeg[u]
//   units   int2[U]      warp work units, unit_shard int32[U]
//   bm      u32[V/32+2]  next-frontier bitmap; frontier int4[V+E/256+1] (push only)
//   sig     u64[V]       per-vertex shard-group mask (selective scheduling),
//                        built at the first selective step
//   ooff/ocol/ow         out-edge CSR for sparse push steps (SSSP/CC)
// With a shard-cache budget, only the shards that fit stay in HBM; the others
// are kept in pinned host memory and streamed per step through a ring of
// device slots on a copy stream (the GPU form of load_edge, Global.h:129-255),
// compressed when that saves 30% of their bytes (encode_streamed).
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <cstddef>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "gx_engine.h"
#include "gx_nvtx.h"

#include <mutex>

using namespace gx;

namespace gx {

int current_device() {
  int d = 0;
  cudaGetDevice(&d);
  return d;
}

static std::mutex g_pool_mu;
static DevicePool g_pools[64];
static bool g_pool_tried[64];

DevicePool* device_pool(int dev) {
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (!g_pool_tried[dev]) {
    g_pool_tried[dev] = true;
    int supported = 0;
    cudaDeviceGetAttribute(&supported, cudaDevAttrMemoryPoolsSupported, dev);
    if (supported) {
      cudaMemPoolProps props{};
      props.allocType = cudaMemAllocationTypePinned;
      props.handleTypes = cudaMemHandleTypeNone;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      cudaMemPool_t pool = nullptr;
      cudaStream_t st = nullptr;
      if (cudaMemPoolCreate(&pool, &props) == cudaSuccess &&
          cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess) {
        unsigned long long keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        g_pools[dev].pool = pool;
        g_pools[dev].stream = st;
      } else {
        if (pool) cudaMemPoolDestroy(pool);
        cudaGetLastError();
      }
    }
  }
  return g_pools[dev].pool ? &g_pools[dev] : nullptr;
}

}  // namespace gx

namespace {

// Work units of one shard: heavy-vertex chunks first, then tiles of up to 32
// consecutive light vertices with at most tile_edges edges.
void build_units(gx_engine* e) {
  const int32_t P = e->P;
  const int64_t* off = e->off.data();
  // Exact-order mode never chunks a vertex: each list is folded in order.
  const int32_t heavy_deg = e->cfg.exact_order ? INT32_MAX : std::max(e->cfg.heavy_degree, 32);
  const int64_t cap = std::max<int64_t>(e->cfg.tile_edges, 32);
  std::vector<std::vector<int2>> su(P);
  std::vector<std::vector<int32_t>> sh(P);
#pragma omp parallel for schedule(dynamic, 1)
  for (int32_t p = 0; p < P; ++p) {
    std::vector<int2>& U = su[p];
    const int32_t s = e->bounds[p], t = e->bounds[p + 1];
    int32_t vb = s, cnt = 0;
    int64_t edges = 0;
    auto close = [&](int32_t ve) {
      if (cnt > 0) U.push_back(make_int2(vb, ve));
      cnt = 0;
      edges = 0;
    };
    // Tiles are runs of up to 32 consecutive vertices; a vertex above the
    // heavy threshold keeps its lane (masked in the kernel) and also gets
    // its own chunk units.
    for (int32_t v = s; v < t; ++v) {
      const int64_t d = off[v + 1] - off[v];
      const int64_t light = d > heavy_deg ? 0 : d;
      if (d > heavy_deg) sh[p].push_back(v);
      if (cnt == 32 || (cnt > 0 && edges + light > cap)) {
        close(v);
        vb = v;
      }
      if (cnt == 0) vb = v;
      ++cnt;
      edges += light;
    }
    close(t);
  }
  // Per shard: heavy vertices longest first, then counts; the shards' unit
  // ranges are laid end to end and filled in parallel.
  std::vector<int64_t> n_units(static_cast<size_t>(P) + 1, 0), n_heavy(static_cast<size_t>(P) + 1, 0),
      n_part(static_cast<size_t>(P) + 1, 0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int32_t p = 0; p < P; ++p) {
    std::vector<int32_t>& hv = sh[p];
    std::sort(hv.begin(), hv.end(), [&](int32_t a, int32_t b) {
      const int64_t da = off[a + 1] - off[a], db = off[b + 1] - off[b];
      return da > db || (da == db && a < b);
    });
    int64_t chunks = 0;
    for (int32_t v : hv) chunks += (off[v + 1] - off[v] + kHeavyChunk - 1) / kHeavyChunk;
    n_units[p + 1] = chunks + static_cast<int64_t>(su[p].size());
    n_heavy[p + 1] = static_cast<int64_t>(hv.size());
    n_part[p + 1] = chunks;
  }
  for (int32_t p = 0; p < P; ++p) {
    n_units[p + 1] += n_units[p];
    n_heavy[p + 1] += n_heavy[p];
    n_part[p + 1] += n_part[p];
  }
  e->units.resize(static_cast<size_t>(n_units[P]));
  e->unit_shard.resize(static_cast<size_t>(n_units[P]));
  e->heavy.resize(static_cast<size_t>(n_heavy[P]));
  e->unit_begin.assign(P + 1, 0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int32_t p = 0; p < P; ++p) {
    int64_t u = n_units[p];
    int64_t h = n_heavy[p];
    int64_t part = n_part[p];
    e->unit_begin[p] = static_cast<int32_t>(u);
    for (int32_t v : sh[p]) {
      const int64_t d = off[v + 1] - off[v];
      const int32_t nch = static_cast<int32_t>((d + kHeavyChunk - 1) / kHeavyChunk);
      e->heavy[h] = make_int4(v, nch, static_cast<int32_t>(part), p);
      for (int32_t c = 0; c < nch; ++c) {
        e->units[u] = make_int2(-(static_cast<int32_t>(h) + 1), c);
        e->unit_shard[u] = p;
        ++u;
      }
      part += nch;
      ++h;
    }
    for (const int2& t : su[p]) {
      e->units[u] = t;
      e->unit_shard[u] = p;
      ++u;
    }
  }
  e->unit_begin[P] = static_cast<int32_t>(n_units[P]);
  e->n_partials = n_part[P];
}

// Longest in-list that the warps of relabel_scatter_kernel move when the
// engine relabels; longer ones go to the CTAs of relabel_scatter_long_kernel.
constexpr int64_t kRelabelWarpMax = 512;

// Values in the caller's numbering from the engine's buffer (d_stage).
gx_status values_to_caller(gx_engine* e, const void* d_vals, cudaStream_t s) {
  gather_values_kernel<<<e->n_sm * 4, 256, 0, s>>>(static_cast<const uint32_t*>(d_vals), e->d_perm, e->V, e->d_stage);
  GX_CUDA(cudaGetLastError());
  GX_CUDA(cudaStreamSynchronize(s));
  return GX_OK;
}

gx_status alloc_ctl(gx_engine* e) {
  if (!e->d_ctl) GX_TRY(dev_alloc(&e->d_ctl, 1));
  if (!e->h_ctl) GX_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&e->h_ctl), sizeof(Ctl), cudaHostAllocDefault));
  return GX_OK;
}

// Copies `bytes` (a multiple of 4) from host memory the device reads in place
// (pageable memory on a system with cudaDevAttrPageableMemoryAccess) to the
// device, 16 bytes per thread step when both ends are 16-byte aligned.
__global__ void host_copy_kernel(const void* __restrict__ src, void* __restrict__ dst, size_t bytes) {
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  const size_t tid = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  size_t done = 0;
  if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0) {
    const size_t n16 = bytes / 16;
    const int4* s16 = static_cast<const int4*>(src);
    int4* d16 = static_cast<int4*>(dst);
    for (size_t i = tid; i < n16; i += stride) d16[i] = s16[i];
    done = n16 * 16;
  }
  const uint32_t* s4 = reinterpret_cast<const uint32_t*>(static_cast<const char*>(src) + done);
  uint32_t* d4 = reinterpret_cast<uint32_t*>(static_cast<char*>(dst) + done);
  const size_t n4 = (bytes - done) / 4;
  for (size_t i = tid; i < n4; i += stride) d4[i] = s4[i];
}

// Host-to-device copy of a caller's array on `s`: read in place by a kernel
// when the device can (no staging through pinned buffers, and the host thread
// is free at once), else cudaMemcpyAsync.
gx_status upload_async(gx_engine* e, void* dst, const void* src, size_t bytes, cudaStream_t s,
                       int blocks_per_sm = 8) {
  if (bytes == 0) return GX_OK;
  if (e->pageable_access && (reinterpret_cast<uintptr_t>(src) & 3u) == 0 && bytes % 4 == 0) {
    host_copy_kernel<<<e->n_sm * blocks_per_sm, 256, 0, s>>>(src, dst, bytes);
    GX_CUDA(cudaGetLastError());
  } else {
    GX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
  }
  return GX_OK;
}

// Device-to-host copy into a host array on `s`: written in place by a kernel
// when the device can reach pageable memory.
gx_status download_async(gx_engine* e, void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return GX_OK;
  if (e->pageable_access && (reinterpret_cast<uintptr_t>(dst) & 3u) == 0 && bytes % 4 == 0) {
    host_copy_kernel<<<e->n_sm * 8, 256, 0, s>>>(src, dst, bytes);
    GX_CUDA(cudaGetLastError());
  } else {
    GX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
  }
  return GX_OK;
}

// Host pages of a large array that the device is about to write in place are
// placed by the host threads first (a device write to an unmapped host page
// would fault it in from the device side, one page at a time).
template <class T>
void host_resize_placed(hvec<T>& v, size_t n) {
  const bool fresh = v.capacity() < n;
  v.resize(n);
  if (!fresh) return;
  T* p = v.data();
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < static_cast<int64_t>(n); ++i) p[i] = T();
}

// Lists longer than kRelabelWarpMax in a valid CSC of E edges.
unsigned int relabel_longs_cap(int64_t E) { return static_cast<unsigned int>(E / kRelabelWarpMax + 1); }

// Enqueues the move of per-edge data (source ids, renamed, or weights) from
// the caller's layout to the relabelled one (relabel_scatter_kernel).
gx_status relabel_scatter(gx_engine* e, const int32_t* src, int32_t* dst, bool rename, int32_t* longs,
                          unsigned int* n_longs, unsigned int* flag, cudaStream_t s) {
  const unsigned int cap = relabel_longs_cap(e->E);
  GX_CUDA(cudaMemsetAsync(n_longs, 0, sizeof(unsigned int), s));
  relabel_scatter_kernel<<<e->n_sm * 8, 256, 0, s>>>(e->d_off_old, src, e->d_off, e->d_inv,
                                                     rename ? e->d_perm : nullptr, e->V, e->E, kRelabelWarpMax, dst,
                                                     longs, cap, n_longs, flag);
  relabel_scatter_long_kernel<<<e->n_sm * 4, 256, 0, s>>>(e->d_off_old, src, e->d_off, e->d_inv,
                                                           rename ? e->d_perm : nullptr, e->V, dst, longs, cap,
                                                           n_longs, flag);
  GX_CUDA(cudaGetLastError());
  return GX_OK;
}

// Buffers of one load, freed once the copy stream is idle.
struct LoadScratch {
  cudaStream_t s;
  unsigned int* flag = nullptr;
  int32_t* col_old = nullptr;
  int32_t* od_old = nullptr;
  uint32_t* len = nullptr;
  unsigned long long* keys[2] = {nullptr, nullptr};
  uint32_t* hist = nullptr;
  unsigned long long* offs = nullptr;
  unsigned long long* part = nullptr;
  int32_t* longs = nullptr;
  unsigned int* n_longs = nullptr;
  hvec<int32_t> od_host;  // out-degrees computed on the host, read by the device in place
  explicit LoadScratch(cudaStream_t st) : s(st) {}
  ~LoadScratch() {
    if (flag || col_old || keys[0]) cudaStreamSynchronize(s);
    dev_free(&flag);
    dev_free(&col_old);
    dev_free(&od_old);
    dev_free(&len);
    dev_free(&keys[0]);
    dev_free(&keys[1]);
    dev_free(&hist);
    dev_free(&offs);
    dev_free(&part);
    dev_free(&longs);
    dev_free(&n_longs);
  }
};

int bits_for(int64_t n) {  // bits of the largest value below n
  int b = 1;
  while (b < 62 && (int64_t(1) << b) < n) ++b;
  return b;
}

__global__ void store_i64_kernel(int64_t* p, int64_t x) { *p = x; }

// A relabelling load up to the move of the source ids: the caller's offsets
// go to the device, which sorts the vertices into the new order and derives
// the new offsets and out-degrees; the new offsets come back to the host for
// its own planning (e->off, waited for here) while the source ids go up; the
// ids are then renamed into place in one pass, and the out-degrees and the
// permutation come back (e->outdeg, h_perm) — both still running on the copy
// stream when this returns (flag bits as validate_csc_kernel's).  Also
// counts the dangling vertices.
// Device-side phases of a load, for the verbose log: events recorded on a
// stream, their times printed relative to the first once the stream is done.
struct StreamMarks {
  bool on = false;
  std::vector<std::pair<const char*, cudaEvent_t>> ev;
  void mark(const char* what, cudaStream_t s) {
    if (!on) return;
    cudaEvent_t x = nullptr;
    if (cudaEventCreate(&x) != cudaSuccess) return;
    cudaEventRecord(x, s);
    ev.emplace_back(what, x);
  }
  ~StreamMarks() {
    for (auto& m : ev) {
      float ms = 0;
      if (cudaEventSynchronize(m.second) == cudaSuccess) cudaEventElapsedTime(&ms, ev[0].second, m.second);
      fprintf(stderr, "gx_load_csc device %-14s %8.2f ms\n", m.first, ms);
    }
    for (auto& m : ev) cudaEventDestroy(m.second);
  }
};

gx_status relabel_load(gx_engine* e, const int32_t* bounds, const int64_t* off, const int32_t* col,
                       const int32_t* outdeg, LoadScratch& sc) {
  const int32_t V = e->V, P = e->P;
  const int64_t E = e->E;
  cudaStream_t s = e->s_copy;
  StreamMarks marks;
  marks.on = e->cfg.verbose != 0;
  marks.mark("start", s);
  const int vb = bits_for(V), pb = bits_for(P);
  GX_TRY(dev_alloc(&e->d_off, static_cast<size_t>(V) + 1));
  GX_TRY(dev_alloc(&e->d_col, static_cast<size_t>(E) + 8));
  GX_TRY(dev_alloc(&e->d_off_old, static_cast<size_t>(V) + 1));
  GX_TRY(dev_alloc(&e->d_bounds, static_cast<size_t>(P) + 1));
  GX_TRY(dev_alloc(&e->d_perm, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&e->d_inv, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&e->d_outdeg, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&e->d_stage, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&sc.keys[0], static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&sc.keys[1], static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&sc.len, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&sc.od_old, static_cast<size_t>(V)));
  int64_t hist_n = 0, part_n = 0;
  radix_scratch_sizes(V, &hist_n, &part_n);
  GX_TRY(dev_alloc(&sc.hist, static_cast<size_t>(hist_n)));
  GX_TRY(dev_alloc(&sc.offs, static_cast<size_t>(hist_n)));
  GX_TRY(dev_alloc(&sc.part, static_cast<size_t>(part_n)));
  GX_TRY(dev_alloc(&sc.longs, relabel_longs_cap(E)));
  GX_TRY(dev_alloc(&sc.n_longs, 1));
  GX_TRY(dev_alloc(&sc.flag, 1));
  GX_CUDA(cudaMemsetAsync(sc.flag, 0, sizeof(unsigned int), s));
  GX_CUDA(cudaMemsetAsync(e->d_col + E, 0, 8 * sizeof(int32_t), s));
  // The offsets go up first and the device works out the order; then the
  // caller's source ids go up on the compute stream (idle during a load)
  // while the new offsets come back to the host.  (Renaming the ids read in
  // place from host memory took as long as this upload plus the renaming;
  // an upload beside the sort slows the sort several times over.)
  cudaEvent_t ev_order = nullptr, ev_col = nullptr;
  GX_CUDA(cudaEventCreateWithFlags(&ev_order, cudaEventDisableTiming));
  std::unique_ptr<CUevent_st, cudaError_t (*)(cudaEvent_t)> ev_order_g(ev_order, cudaEventDestroy);
  GX_CUDA(cudaEventCreateWithFlags(&ev_col, cudaEventDisableTiming));
  std::unique_ptr<CUevent_st, cudaError_t (*)(cudaEvent_t)> ev_col_g(ev_col, cudaEventDestroy);
  GX_TRY(dev_alloc(&sc.col_old, static_cast<size_t>(std::max<int64_t>(E, 1))));
  GX_TRY(upload_async(e, e->d_off_old, off, sizeof(int64_t) * (static_cast<size_t>(V) + 1), s));
  GX_TRY(upload_async(e, e->d_bounds, bounds, sizeof(int32_t) * (static_cast<size_t>(P) + 1), s));
  marks.mark("offsets", s);
  validate_csc_kernel<<<e->n_sm * 8, 256, 0, s>>>(e->d_off_old, V, nullptr, E, sc.flag);
  relabel_keys_kernel<<<e->n_sm * 8, 256, 0, s>>>(e->d_off_old, e->d_bounds, P, V, vb, sc.keys[0]);
  GX_CUDA(cudaGetLastError());
  marks.mark("keys", s);
  unsigned long long* sorted = nullptr;
  GX_TRY(radix_sort_bits(sc.keys[0], sc.keys[1], V, vb, vb + 12 + pb, sc.hist, sc.offs, sc.part, s, &sorted));
  marks.mark("sorted", s);
  // Out-degrees in the caller's numbering (while the device sorts).
  const int32_t* od = outdeg;
  if (!od) {
    sc.od_host.resize(static_cast<size_t>(V));
    GX_TRY(gx_out_degree(V, off, col, sc.od_host.data()));
    od = sc.od_host.data();
  }
  int64_t n_dang = 0;
#pragma omp parallel for reduction(+ : n_dang)
  for (int32_t v = 0; v < V; ++v) n_dang += od[v] == 0;
  e->n_dangling = n_dang;
  GX_TRY(upload_async(e, sc.od_old, od, sizeof(int32_t) * static_cast<size_t>(V), s));
  relabel_order_kernel<<<e->n_sm * 8, 256, 0, s>>>(sorted, (1ull << vb) - 1, V, e->d_off_old, sc.od_old, e->d_inv,
                                                   e->d_perm, e->d_outdeg, sc.len);
  GX_CUDA(cudaGetLastError());
  GX_TRY(scan_u32(sc.len, V, reinterpret_cast<unsigned long long*>(e->d_off), sc.part, s));
  store_i64_kernel<<<1, 1, 0, s>>>(e->d_off + V, E);
  GX_CUDA(cudaEventRecord(ev_order, s));
  marks.mark("new offsets", s);
  GX_CUDA(cudaStreamWaitEvent(e->s_comp, ev_order, 0));
  GX_TRY(upload_async(e, sc.col_old, col, sizeof(int32_t) * static_cast<size_t>(E), e->s_comp));
  GX_CUDA(cudaEventRecord(ev_col, e->s_comp));
  marks.mark("ids uploaded", e->s_comp);
  // The host's copies in the new numbering.
  host_resize_placed(e->off, static_cast<size_t>(V) + 1);
  host_resize_placed(e->outdeg, static_cast<size_t>(V));
  host_resize_placed(e->h_perm, static_cast<size_t>(V));
  // The new offsets first (the host plans the work units from them while
  // the ids go up); the out-degrees and the permutation, which the host
  // needs only once the load is done, after the renaming.
  GX_TRY(download_async(e, e->off.data(), e->d_off, sizeof(int64_t) * (static_cast<size_t>(V) + 1), s));
  cudaEvent_t ev = nullptr;
  GX_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  std::unique_ptr<CUevent_st, cudaError_t (*)(cudaEvent_t)> evg(ev, cudaEventDestroy);
  GX_CUDA(cudaEventRecord(ev, s));
  marks.mark("host offsets", s);
  GX_CUDA(cudaStreamWaitEvent(s, ev_col, 0));
  marks.mark("ids ready", s);
  GX_TRY(relabel_scatter(e, sc.col_old, e->d_col, true, sc.longs, sc.n_longs, sc.flag, s));
  marks.mark("ids renamed", s);
  GX_TRY(download_async(e, e->outdeg.data(), e->d_outdeg, sizeof(int32_t) * static_cast<size_t>(V), s));
  GX_TRY(download_async(e, e->h_perm.data(), e->d_perm, sizeof(int32_t) * static_cast<size_t>(V), s));
  marks.mark("host copies", s);
  GX_CUDA(cudaEventSynchronize(ev));
  return GX_OK;
}

gx_status setup_slot_events(gx_engine* e, int slots) {
  if (static_cast<int>(e->slot_free.size()) >= slots) return GX_OK;
  for (auto ev : e->slot_free) cudaEventDestroy(ev);
  for (auto ev : e->slot_ready) cudaEventDestroy(ev);
  e->slot_free.assign(slots, nullptr);
  e->slot_ready.assign(slots, nullptr);
  for (int i = 0; i < slots; ++i) {
    GX_CUDA(cudaEventCreateWithFlags(&e->slot_free[i], cudaEventDisableTiming));
    GX_CUDA(cudaEventCreateWithFlags(&e->slot_ready[i], cudaEventDisableTiming));
  }
  return GX_OK;
}

inline int64_t align16(int64_t x) { return (x + 15) & ~int64_t(15); }

// The compressed streaming format.  Chunk c holds the source ids of global
// edges [32c, 32c+32) as offsets from their minimum, nb bytes each, nb = 0..4
// the fewest that hold the largest (comp_idx4 in gx_kernels.cuh reads them).
// A streamed shard's blob: chunk headers (8 bytes each) | payload (32*nb bytes
// per chunk, every chunk 16-byte aligned) | one byte per weight.  Chunks
// straddling two shards are stored in both blobs.  Resident shards stay plain:
// their compute is not slowed by decoding, and the copy engine, the bound of
// a streamed superstep, moves fewer bytes.
gx_status encode_streamed(gx_engine* e, const int32_t* col) {
  const int32_t P = e->P;
  const int64_t E = e->E;
  const bool wt = e->has_weights;
  e->cb_off.assign(P + 1, 0);
  e->cb_bytes.assign(P, 0);
  e->cb_c0.assign(P, 0);
  e->cb_pay.assign(P, 0);
  e->cb_w8.assign(P, 0);
  std::vector<int64_t> nch(P, 0), c1s(P, 0);
  for (int32_t p = 0; p < P; ++p) {
    if (e->resident[p]) continue;
    const int64_t e0 = e->off[e->bounds[p]], e1 = e->off[e->bounds[p + 1]];
    e->cb_c0[p] = e0 >> 5;
    c1s[p] = e1 > e0 ? (e1 + 31) >> 5 : e->cb_c0[p];
    nch[p] = c1s[p] - e->cb_c0[p];
  }
  // Bytes per offset of every chunk of the streamed shards.
  std::vector<std::vector<uint8_t>> width(P);
#pragma omp parallel for schedule(dynamic, 1)
  for (int32_t p = 0; p < P; ++p) {
    if (e->resident[p]) continue;
    width[p].resize(static_cast<size_t>(nch[p]));
    for (int64_t i = 0; i < nch[p]; ++i) {
      const int64_t lo = 32 * (e->cb_c0[p] + i), hi = std::min(E, lo + 32);
      uint32_t mn = static_cast<uint32_t>(col[lo]), mx = mn;
      for (int64_t k = lo + 1; k < hi; ++k) {
        const uint32_t x = static_cast<uint32_t>(col[k]);
        mn = std::min(mn, x);
        mx = std::max(mx, x);
      }
      uint32_t bits = 0;
      for (uint32_t r = mx - mn; r; r >>= 1) ++bits;
      width[p][i] = static_cast<uint8_t>((bits + 7) / 8);
    }
  }
  // A shard travels compressed only when its blob is at most 70% of the
  // plain bytes: below that the decoding costs more compute than the copy
  // saves (measured on streamed PageRank at scale 28).
  int64_t max_blob = 16, n_blobs = 0, n_streamed = 0;
  for (int32_t p = 0; p < P; ++p) {
    int64_t pay = 0;  // 32*nb bytes per chunk, a multiple of 16
    for (int64_t i = 0; i < nch[p]; ++i) pay += 32 * width[p][i];
    e->cb_pay[p] = align16(8 * nch[p]);
    e->cb_w8[p] = align16(e->cb_pay[p] + pay);
    const int64_t blob = align16(e->cb_w8[p] + (wt ? 32 * nch[p] : 0));
    const int64_t plain = (e->off[e->bounds[p + 1]] - e->off[e->bounds[p]]) * (wt ? 8 : 4);
    const bool use = !e->resident[p] && nch[p] > 0 && blob * 100 <= plain * 70;
    n_streamed += !e->resident[p];
    n_blobs += use;
    e->cb_bytes[p] = use ? blob : 0;
    e->cb_off[p + 1] = e->cb_off[p] + e->cb_bytes[p];
    max_blob = std::max(max_blob, e->cb_bytes[p]);
  }
  e->comp_all = n_blobs == n_streamed;
  if (e->h_cblob) cudaFreeHost(e->h_cblob);
  e->h_cblob = nullptr;
  GX_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&e->h_cblob), std::max<int64_t>(e->cb_off[P], 16),
                        cudaHostAllocDefault));
#pragma omp parallel for schedule(dynamic, 1)
  for (int32_t p = 0; p < P; ++p) {
    if (e->cb_bytes[p] == 0) continue;
    uint8_t* blob = e->h_cblob + e->cb_off[p];
    uint2* hdr = reinterpret_cast<uint2*>(blob);
    uint8_t* pay = blob + e->cb_pay[p];
    uint8_t* w8 = blob + e->cb_w8[p];
    memset(blob, 0, static_cast<size_t>(e->cb_bytes[p]));
    uint32_t w16 = 0;  // payload position in 16-byte units
    for (int64_t i = 0; i < nch[p]; ++i) {
      const int64_t lo = 32 * (e->cb_c0[p] + i), hi = std::min(E, lo + 32);
      const uint32_t nb = width[p][i];
      uint32_t mn = static_cast<uint32_t>(col[lo]);
      for (int64_t k = lo + 1; k < hi; ++k) mn = std::min(mn, static_cast<uint32_t>(col[k]));
      hdr[i] = make_uint2(mn, (w16 << 3) | nb);
      uint8_t* q = pay + static_cast<size_t>(w16) * 16;
      for (int64_t k = lo; k < hi; ++k) {
        const uint32_t v = static_cast<uint32_t>(col[k]) - mn;  // little-endian bytes
        for (uint32_t t = 0; t < nb; ++t) q[(k - lo) * nb + t] = static_cast<uint8_t>(v >> (8 * t));
      }
      if (wt)
        for (int64_t k = lo; k < hi; ++k) w8[i * 32 + (k - lo)] = static_cast<uint8_t>(e->h_w[k]);
      w16 += 2 * nb;  // 32 * nb bytes
    }
  }
  for (auto ptr : e->slot_blob) gx::pool_free(ptr);
  e->slot_blob.assign(e->n_slots, nullptr);
  for (int i = 0; i < e->n_slots; ++i) GX_TRY(dev_alloc(&e->slot_blob[i], static_cast<size_t>(max_blob)));
  e->comp = n_blobs > 0;
  e->comp_bytes = e->cb_off[P];
  return GX_OK;
}

// Decides which shards stay in HBM under the budget (in shard order, like the
// reference's insert-until-full edge cache, Global.h:170-244), uploads them,
// and sets up the streaming ring for the rest.  When the plain shards exceed
// the budget and compression is on, the compressed shard cache is used.
gx_status plan_shards(gx_engine* e, const int32_t* src_col, bool col_on_device) {
  const int32_t P = e->P;
  const int64_t per_edge = e->has_weights ? 8 : 4;
  const int64_t budget = e->cfg.cache_budget_bytes;
  e->comp = false;
  e->resident.assign(P, 0);
  e->dev_base.assign(P, 0);
  int64_t used = 0, max_stream = 0;
  e->n_resident = 0;
  std::vector<int64_t> lo(P), hi(P);
  for (int32_t p = 0; p < P; ++p) {
    lo[p] = e->off[e->bounds[p]] & ~3ll;
    hi[p] = (e->off[e->bounds[p + 1]] + 3) & ~3ll;
    const int64_t bytes = (hi[p] - lo[p] + 4) * per_edge;
    if (budget < 0 || (used + hi[p] - lo[p] + 4) * per_edge <= budget) {
      e->resident[p] = 1;
      used += hi[p] - lo[p] + 4;  // elements
      ++e->n_resident;
    } else {
      max_stream = std::max(max_stream, bytes / per_edge);
    }
  }
  e->all_resident = e->n_resident == P;
  if (!(col_on_device && e->all_resident)) dev_free(&e->d_col);
  dev_free(&e->d_w);
  if (e->all_resident) {
    if (!col_on_device) {
      GX_TRY(dev_alloc(&e->d_col, static_cast<size_t>(e->E) + 8));
      GX_CUDA(cudaMemset(e->d_col, 0, (e->E + 8) * sizeof(int32_t)));
      GX_CUDA(cudaMemcpy(e->d_col, src_col, e->E * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    if (e->has_weights) {
      GX_TRY(dev_alloc(&e->d_w, static_cast<size_t>(e->E) + 8));
      GX_CUDA(cudaMemset(e->d_w, 0, (e->E + 8) * sizeof(uint32_t)));
      GX_CUDA(cudaMemcpy(e->d_w, e->h_w, e->E * sizeof(uint32_t), cudaMemcpyHostToDevice));
    }
    for (int32_t p = 0; p < P; ++p) e->dev_base[p] = 0;
  } else {
    GX_TRY(dev_alloc(&e->d_col, static_cast<size_t>(used) + 8));
    if (e->has_weights) GX_TRY(dev_alloc(&e->d_w, static_cast<size_t>(used) + 8));
    int64_t pos = 0;
    for (int32_t p = 0; p < P; ++p) {
      if (!e->resident[p]) continue;
      const int64_t n = std::min(hi[p], e->E + 4) - lo[p];
      GX_CUDA(cudaMemcpy(e->d_col + pos, src_col + lo[p], n * sizeof(int32_t), cudaMemcpyHostToDevice));
      if (e->has_weights)
        GX_CUDA(cudaMemcpy(e->d_w + pos, e->h_w + lo[p], n * sizeof(uint32_t), cudaMemcpyHostToDevice));
      e->dev_base[p] = pos - lo[p];  // d_col + dev_base[p] is indexed by global edge id
      pos += hi[p] - lo[p] + 4;
    }
    const int slots = std::max({2, e->cfg.stream_slots, static_cast<int>(e->s_copies.size())});
    e->slot_elems = max_stream + 8;
    for (auto ptr : e->slot_col) gx::pool_free(ptr);
    for (auto ptr : e->slot_w) gx::pool_free(ptr);
    for (auto ptr : e->slot_blob) gx::pool_free(ptr);
    e->slot_blob.clear();
    e->slot_col.assign(slots, nullptr);
    e->slot_w.assign(slots, nullptr);
    for (int i = 0; i < slots; ++i) {
      GX_TRY(dev_alloc(&e->slot_col[i], e->slot_elems));
      if (e->has_weights) GX_TRY(dev_alloc(&e->slot_w[i], e->slot_elems));
    }
    e->n_slots = slots;
    GX_TRY(setup_slot_events(e, slots));
    // Streamed shards travel compressed when the weights (if any) fit bytes.
    if (e->cfg.compress_cache && (!e->has_weights || e->w_narrow)) {
      // A chunk header addresses the payload in 16-byte units with 29 bits,
      // far beyond any shard of fewer than 2^31 edges.
      GX_TRY(encode_streamed(e, src_col));
      // With every streamed shard compressed, the plain ring is only needed
      // for the shard signatures.
      if (e->comp && e->comp_all) {
        for (int i = 1; i < slots; ++i) {
          gx::pool_free(e->slot_col[i]);
          if (!e->slot_w.empty() && e->slot_w[i]) gx::pool_free(e->slot_w[i]);
        }
        e->slot_col.resize(1);
        if (!e->slot_w.empty()) e->slot_w.resize(1);
      }
    }
  }
  e->out_built = false;
  return GX_OK;
}

// Streamed graphs: for every vertex, the set of shards it is a source in
// (a bitset of P bits), kept in host memory, where the host-driven step loop
// turns the changed vertices a finalize lists into the shards the next
// selective step streams and sweeps.  Built at load, on the GPU, shard by
// shard (streamed shards go through slot 0), then copied to the host.
__global__ void shard_sets_kernel(unsigned long long* sets, int words, const int32_t* col, int64_t e0, int64_t e1,
                                  int32_t p) {
  const int w = p >> 6;
  const unsigned long long bit = 1ull << (p & 63);
  for (int64_t k = e0 + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < e1;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    unsigned long long* x = sets + static_cast<int64_t>(col[k]) * words + w;
    if (!(*x & bit)) atomicOr(x, bit);
  }
}

gx_status build_shard_sets(gx_engine* e) {
  const int32_t P = e->P;
  const int words = (P + 63) / 64;
  unsigned long long* d_sets = nullptr;
  GX_TRY(dev_alloc(&d_sets, static_cast<size_t>(e->V) * words));
  struct Free {
    unsigned long long* p;
    ~Free() { gx::pool_free(p); }
  } guard{d_sets};
  GX_CUDA(cudaMemsetAsync(d_sets, 0, sizeof(unsigned long long) * e->V * words, e->s_comp));
  for (int32_t p = 0; p < P; ++p) {
    const int64_t e0 = e->off[e->bounds[p]], e1 = e->off[e->bounds[p + 1]];
    if (e1 == e0) continue;
    const int32_t* col = nullptr;
    if (e->resident[p]) {
      col = e->d_col + e->dev_base[p];
    } else {
      const int64_t lo = e0 & ~3ll;
      GX_CUDA(cudaMemcpyAsync(e->slot_col[0], e->h_col + lo, (e1 - lo) * sizeof(int32_t), cudaMemcpyHostToDevice,
                              e->s_comp));
      col = e->slot_col[0] - lo;
    }
    const int64_t n = e1 - e0;
    const int grid = static_cast<int>(std::min<int64_t>((n + 255) / 256, static_cast<int64_t>(e->n_sm) * 8));
    shard_sets_kernel<<<grid, 256, 0, e->s_comp>>>(d_sets, words, col, e0, e1, p);
    GX_CUDA(cudaGetLastError());
  }
  e->h_shard_sets.resize(static_cast<size_t>(e->V) * words);
  GX_CUDA(cudaMemcpyAsync(e->h_shard_sets.data(), d_sets, sizeof(unsigned long long) * e->h_shard_sets.size(),
                          cudaMemcpyDeviceToHost, e->s_comp));
  GX_CUDA(cudaStreamSynchronize(e->s_comp));
  e->shard_set_words = words;
  return GX_OK;
}

// Out-edge CSR for push steps (all-resident graphs only).
gx_status build_out_edges(gx_engine* e, bool weighted) {
  if (e->out_built && (!weighted || e->out_weighted)) return GX_OK;
  const int32_t V = e->V;
  std::vector<int64_t> ooff(static_cast<size_t>(V) + 1, 0);
  for (int32_t v = 0; v < V; ++v) ooff[v + 1] = ooff[v] + e->outdeg[v];
  if (ooff[V] != e->E)
    return fail(GX_ERR_FORMAT, "vertexout.npy sums to %lld out-edges but the shards hold %lld edges",
                static_cast<long long>(ooff[V]), static_cast<long long>(e->E));
  // Push frontier: one entry per kPushChunk out-edges of each vertex, so
  // V + E / kPushChunk + 1 entries hold any frontier.
  e->frontier_cap = static_cast<unsigned long long>(V) + static_cast<unsigned long long>(e->E) / kPushChunk + 1;
  if (!e->d_frontier) GX_TRY(dev_alloc(&e->d_frontier, static_cast<size_t>(e->frontier_cap)));
  GX_TRY(dev_alloc(&e->d_ooff, static_cast<size_t>(V) + 1));
  GX_TRY(dev_alloc(&e->d_ocol, static_cast<size_t>(e->E) + 8));
  if (weighted) GX_TRY(dev_alloc(&e->d_ow, static_cast<size_t>(e->E) + 8));
  unsigned long long* cursor = nullptr;
  GX_TRY(dev_alloc(&cursor, static_cast<size_t>(V) + 1));
  GX_CUDA(cudaMemcpy(e->d_ooff, ooff.data(), ooff.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  GX_CUDA(cudaMemcpy(cursor, ooff.data(), ooff.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  transpose_kernel<<<e->n_sm * 8, 256, 0, e->s_comp>>>(e->d_off, e->d_col, weighted ? e->d_w : nullptr, V, cursor,
                                                        e->d_ocol, weighted ? e->d_ow : nullptr);
  cudaError_t err = cudaGetLastError();
  if (err == cudaSuccess) err = cudaStreamSynchronize(e->s_comp);
  gx::pool_free(cursor);
  if (err != cudaSuccess) return fail(GX_ERR_CUDA, "transpose: %s", cudaGetErrorString(err));
  e->out_built = true;
  e->out_weighted = weighted;
  return GX_OK;
}

template <int APP>
int occupancy_grid(gx_engine* e, const void* fn) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0);
  return std::max(1, per_sm) * e->n_sm;
}

template <int APP>
gx_status run_app(gx_engine* e, const gx_run_params& prm, gx_run_stats* out) {
  typedef typename AppTraits<APP>::T T;
  const int32_t V = e->V;
  const bool weighted = APP == K_SSSP_W;
  const bool min_app = APP == K_SSSP_UNIT || APP == K_SSSP_W || APP == K_CC;
  const bool push_ok = min_app && e->cfg.push_sparse && e->all_resident &&
                       static_cast<int64_t>(V) + e->E / kPushChunk + 1 < INT32_MAX;
  if (push_ok) GX_TRY(build_out_edges(e, weighted));
  if (e->stats_cap < prm.max_iter) {
    GX_TRY(dev_alloc(&e->d_stats, static_cast<size_t>(std::max(prm.max_iter, 1))));
    e->stats_cap = prm.max_iter;
  }
  // A resumed run has no statistics for the steps before first_step.
  if (prm.first_step > 0)
    GX_CUDA(cudaMemsetAsync(e->d_stats, 0, sizeof(StepStats) * prm.first_step, e->s_comp));

  // Control block.
  Ctl c{};
  c.max_iter = prm.max_iter;
  c.n_vertices = V;
  c.n_shards = e->P;
  c.shard_words = (e->P + 31) / 32;
  c.push_ok = push_ok;
  c.push_edge_limit =
      push_ok ? static_cast<unsigned long long>(e->cfg.push_edge_fraction * static_cast<double>(e->E)) : 0ull;
  // Selective pull steps: resident graphs mark their shards on the device
  // from the out-edge CSR (built for push, or at the first selective step);
  // streamed graphs list their changed vertices for the host.
  c.shard_bm = e->d_shard_bm;
  c.bounds = e->d_bounds;
  if (e->all_resident) {
    c.mark_mode = e->out_built ? MARK_OUT : MARK_NONE;
    c.ooff = e->d_ooff;
    c.ocol = e->d_ocol;
  } else {
    c.mark_mode = MARK_LIST;
    c.changed_list = e->d_changed_list;
    c.changed_cap = static_cast<unsigned int>(e->changed_cap);
  }
  GX_CUDA(cudaMemsetAsync(e->d_shard_bm, 0, sizeof(uint32_t) * 2 * c.shard_words, e->s_comp));
  c.damping = prm.damping;
  c.inv_n = 1.0 / V;
  c.fx_scale = static_cast<double>(V) * 1073741824.0;  // 2^30 per 1/N of rank
  c.tolerance = prm.tolerance;
  c.sel_threshold = e->cfg.selective_threshold;
  c.step = prm.first_step;
  c.async_mode = (min_app && prm.async_mode) ? 1 : 0;
  c.cur = 0;
  c.mode = MODE_DENSE;
  c.done = prm.max_iter <= 0;
  // Initial values: init_vertex of the app, or the caller's values.
  int use_init = 0;
  if (e->device_init) {
    use_init = 1;  // values already placed in d_val[0] on the device (warm start)
  } else if (prm.use_init) {
    if (!e->has_init) return fail(GX_ERR_STATE, "gx_run: use_init set but gx_set_init was not called");
    if (e->relabeled) {
      // The caller's values, moved into the engine's numbering.
      GX_CUDA(cudaMemcpy(e->d_stage, e->init_vals.data(), sizeof(T) * V, cudaMemcpyHostToDevice));
      scatter_values_kernel<<<e->n_sm * 4, 256, 0, e->s_comp>>>(e->d_stage, e->d_perm, V,
                                                                static_cast<uint32_t*>(e->d_val[0]));
      GX_CUDA(cudaGetLastError());
    } else {
      GX_CUDA(cudaMemcpy(e->d_val[0], e->init_vals.data(), sizeof(T) * V, cudaMemcpyHostToDevice));
    }
    use_init = 1;
  }
  // The source in the engine's numbering.
  const int32_t source = (e->relabeled && prm.source >= 0 && prm.source < V) ? e->h_perm[prm.source] : prm.source;
  if (APP == K_PR_STD) {
    // D of the initial vector, in the same fixed point the device uses (summed
    // in the caller's vertex order).
    double D = 0;
    if (use_init && !e->device_init) {
      for (int32_t v = 0; v < V; ++v) {
        if (e->outdeg[e->relabeled ? e->h_perm[v] : v] != 0) continue;
        float x;
        memcpy(&x, &e->init_vals[v], sizeof(float));
        D += x;
      }
    }
    if (!use_init) D = static_cast<double>(e->n_dangling) * static_cast<double>(static_cast<float>(1.0 / V));
    if (e->device_init) D = e->device_init_dangling;
    c.base = (1.0 - prm.damping) * c.inv_n + prm.damping * D * c.inv_n;
  }
  // SSSP from init_vertex: only the source holds a finite distance, so step 0
  // is a push from it (the same values as the reference's full first pull).
  std::vector<int4> src_entries;
  if (push_ok && (APP == K_SSSP_UNIT || APP == K_SSSP_W) && !use_init && c.push_edge_limit > 0 &&
      prm.max_iter > 0) {
    const int32_t od = e->outdeg[source];
    for (int32_t k = 0; k < od; k += kPushChunk) src_entries.push_back(make_int4(source, 0, k, 0));
    c.step0_push = 1;
    c.mode = MODE_PUSH;
    c.n_frontier = static_cast<int>(src_entries.size());
    if (!src_entries.empty())
      GX_CUDA(cudaMemcpyAsync(e->d_frontier, src_entries.data(), sizeof(int4) * src_entries.size(),
                              cudaMemcpyHostToDevice, e->s_comp));
  }
  GX_CUDA(cudaMemcpyAsync(e->d_ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, e->s_comp));
  init_kernel<APP><<<e->n_sm * 4, 256, 0, e->s_comp>>>(e->d_ctl, e->d_val[0], e->d_con[0], e->d_outdeg, V, source,
                                                       use_init, e->relabeled ? e->d_inv : nullptr);
  GX_CUDA(cudaGetLastError());
  GX_CUDA(cudaMemsetAsync(e->d_bm, 0, sizeof(uint32_t) * e->n_words, e->s_comp));
  GX_CUDA(cudaMemsetAsync(e->d_work, 0, sizeof(unsigned int) * e->n_work, e->s_comp));
  GX_CUDA(cudaMemsetAsync(e->d_hticket, 0, sizeof(unsigned int) * std::max<size_t>(e->heavy.size(), 1), e->s_comp));

  PullArgs pa;
  memset(&pa, 0, sizeof(pa));  // every byte defined: the args are part of the graph cache key
  pa.ctl = e->d_ctl;
  pa.off = e->d_off;
  pa.col = e->d_col;
  pa.w = e->d_w;
  pa.outdeg = e->d_outdeg;
  pa.val[0] = e->d_val[0];
  pa.val[1] = e->d_val[1];
  pa.con[0] = e->d_con[0];
  pa.con[1] = e->d_con[1];
  pa.units = e->d_units;
  pa.unit_shard = e->d_unit_shard;
  pa.u_begin = 0;
  pa.u_end = static_cast<int32_t>(e->units.size());
  pa.heavy = e->d_heavy;
  pa.partial = e->d_partial;
  pa.hticket = e->d_hticket;
  pa.ctr = e->d_work;
  pa.heavy_deg = e->cfg.exact_order ? INT32_MAX : std::max(e->cfg.heavy_degree, 32);
  pa.bm = e->d_bm;
  PushArgs qa;
  memset(&qa, 0, sizeof(qa));
  qa.ctl = e->d_ctl;
  qa.ooff = e->d_ooff;
  qa.ocol = e->d_ocol;
  qa.ow = e->d_ow;
  qa.val[0] = e->d_val[0];
  qa.val[1] = e->d_val[1];
  qa.outdeg = e->d_outdeg;
  qa.frontier = e->d_frontier;
  qa.ctr = e->d_work + kQueues;
  qa.bm = e->d_bm;
  FinArgs fa;
  memset(&fa, 0, sizeof(fa));
  fa.ctl = e->d_ctl;
  fa.stats = e->d_stats;
  fa.bm = e->d_bm;
  fa.n_words = e->n_words;
  fa.val[0] = e->d_val[0];
  fa.val[1] = e->d_val[1];
  fa.outdeg = e->d_outdeg;
  fa.frontier = e->d_frontier;
  fa.frontier_cap = e->frontier_cap;
  fa.work_ctr = e->d_work;
  fa.n_work_ctr = e->n_work;

  void (*pull)(PullArgs) = e->cfg.exact_order ? pull_kernel<APP, true> : pull_kernel<APP, false>;
  if constexpr (APP == K_SSSP_UNIT || APP == K_SSSP_W || APP == K_CC) {
    if (c.async_mode) pull = pull_kernel<APP, false, true>;
  }
  int grid_pull = occupancy_grid<APP>(e, reinterpret_cast<const void*>(pull));
  // Hot-source table (resident graphs): one CTA of kHotThreads per SM whose
  // dynamic shared memory holds the values of sources [0, hot_n).
  int threads_pull = kThreads;
  size_t hot_smem = 0;
  pa.hot_n = 0;
  if constexpr (APP != K_INDEG) {
    if (e->cfg.hot_vertices > 0 && !c.async_mode && e->all_resident) {
      void (*hk)(PullArgs) = e->cfg.exact_order ? pull_kernel<APP, true, false, false, true>
                                                : pull_kernel<APP, false, false, false, true>;
      cudaFuncAttributes attr{};
      GX_CUDA(cudaFuncGetAttributes(&attr, reinterpret_cast<const void*>(hk)));
      int optin = 0;
      GX_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, e->dev));
      const int64_t cap = std::max<int64_t>(0, (static_cast<int64_t>(optin) - static_cast<int64_t>(attr.sharedSizeBytes) -
                                                1024) / static_cast<int64_t>(sizeof(T)));
      const int64_t n = std::min<int64_t>({static_cast<int64_t>(e->cfg.hot_vertices), V, cap}) & ~int64_t(3);
      if (n > 0) {
        hot_smem = static_cast<size_t>(n) * sizeof(T);
        GX_CUDA(cudaFuncSetAttribute(reinterpret_cast<const void*>(hk), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(hot_smem)));
        int per_sm = 0;
        GX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(hk), kHotThreads,
                                                              hot_smem));
        grid_pull = std::max(1, per_sm) * e->n_sm;
        pull = hk;
        threads_pull = kHotThreads;
        pa.hot_n = static_cast<int32_t>(n);
      }
    }
  }
  const int grid_push = occupancy_grid<APP>(e, reinterpret_cast<const void*>(push_kernel<APP>));
  const int grid_fin = std::max(1, std::min(e->n_sm * 4, (e->n_words + kThreads - 1) / kThreads));

  cudaEvent_t ev0, ev1;
  GX_CUDA(cudaEventCreate(&ev0));
  GX_CUDA(cudaEventCreate(&ev1));
  std::unique_ptr<cudaEvent_t, void (*)(cudaEvent_t*)> g0(&ev0, [](cudaEvent_t* x) { cudaEventDestroy(*x); });
  std::unique_ptr<cudaEvent_t, void (*)(cudaEvent_t*)> g1(&ev1, [](cudaEvent_t* x) { cudaEventDestroy(*x); });
  // Checkpoints: the values after every checkpoint_every supersteps, written
  // at the host's sync points ({prefix}{step}.npy).
  const int every = prm.checkpoint_every > 0 ? prm.checkpoint_every : 0;
  int32_t last_ckpt = prm.first_step;
  std::vector<uint32_t> ckpt_buf;
  auto checkpoint = [&](const Ctl& hc) -> gx_status {
    if (!every || hc.step == last_ckpt || hc.step % every != 0) return GX_OK;
    ckpt_buf.resize(static_cast<size_t>(V));
    const void* cur_vals = hc.cur ? e->d_val[1] : e->d_val[0];
    if (e->relabeled) {
      GX_TRY(values_to_caller(e, cur_vals, e->s_comp));
      cur_vals = e->d_stage;
    }
    GX_CUDA(cudaMemcpy(ckpt_buf.data(), cur_vals, sizeof(uint32_t) * V, cudaMemcpyDeviceToHost));
    const std::string path = std::string(prm.checkpoint_prefix) + std::to_string(hc.step) + ".npy";
    const char* descr = is_pr<APP>() ? "<f4" : (APP == K_SSSP_W ? "<u4" : "<i4");
    if (!write_npy_4(path, ckpt_buf.data(), V, descr)) return fail(GX_ERR_IO, "cannot write checkpoint %s", path.c_str());
    last_ckpt = hc.step;
    return GX_OK;
  };
  int64_t h2d_bytes = 0;
  int32_t streamed = 0;
  std::vector<int32_t> host_shards_active;  // streamed runs: shards each selective step swept
  int32_t launches = 1;  // init_kernel
  int32_t pull_launches = 0;
  double ms_pull = 0;
  double copy_ms = 0, comp_ms = 0;

  GX_CUDA(cudaEventRecord(ev0, e->s_comp));
  if (e->all_resident) {
    // Replay K supersteps per CUDA graph launch; the control block makes
    // steps after termination no-ops.
    // Checkpointing syncs after every superstep, so it launches directly.
    const int K = every ? 1 : std::max(1, std::min(prm.max_iter - prm.first_step, 8));
    const bool prof = e->cfg.profile != 0;
    std::vector<cudaEvent_t> pev(prof ? 2 * K : 0);
    for (auto& ev : pev) GX_CUDA(cudaEventCreate(&ev));
    std::unique_ptr<std::vector<cudaEvent_t>, void (*)(std::vector<cudaEvent_t>*)> pev_guard(
        &pev, [](std::vector<cudaEvent_t>* v) {
          for (auto ev : *v) cudaEventDestroy(ev);
        });
    auto enqueue = [&](int i) -> gx_status {
      if (prof) GX_CUDA(cudaEventRecord(pev[2 * i], e->s_comp));
      pull<<<grid_pull, threads_pull, hot_smem, e->s_comp>>>(pa);
      if (prof) GX_CUDA(cudaEventRecord(pev[2 * i + 1], e->s_comp));
      if (push_ok) push_kernel<APP><<<grid_push, kThreads, 0, e->s_comp>>>(qa);
      finalize_kernel<APP><<<grid_fin, kThreads, 0, e->s_comp>>>(fa);
      GX_CUDA(cudaGetLastError());
      launches += push_ok ? 3 : 2;
      return GX_OK;
    };
    cudaGraphExec_t exec = nullptr;
    // Profiling times each pull launch with its own events, so it launches
    // directly instead of replaying a graph.
    if (e->cfg.use_graph && !prof && !every) {
      // A replay bakes in kernels, launch shapes and arguments only, so an
      // executable graph captured by an earlier run with the same bytes of
      // all three is replayed again instead of captured anew.
      GraphKey key;
      memset(&key, 0, sizeof(key));
      key.app = APP;
      key.k = K;
      key.push = push_ok;
      key.pull = reinterpret_cast<const void*>(pull);
      key.grid_pull = grid_pull;
      key.threads_pull = threads_pull;
      key.smem_pull = hot_smem;
      key.grid_push = grid_push;
      key.grid_fin = grid_fin;
      key.pa = pa;
      key.qa = qa;
      key.fa = fa;
      exec = e->cached_graph(key);
      if (!exec) {
        cudaGraph_t graph;
        GX_CUDA(cudaStreamBeginCapture(e->s_comp, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < K; ++i) {
          gx_status st = enqueue(i);
          if (st != GX_OK) {
            cudaStreamEndCapture(e->s_comp, &graph);
            return st;
          }
        }
        GX_CUDA(cudaStreamEndCapture(e->s_comp, &graph));
        cudaError_t err = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (err != cudaSuccess) return fail(GX_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(err));
        e->keep_graph(key, exec);
      }
      launches = 0;
    }
    const int per_step = push_ok ? 3 : 2;
    int steps_before = prm.first_step;
    for (int launched = prm.first_step; launched < prm.max_iter; launched += K) {
      if (exec) {
        GX_CUDA(cudaGraphLaunch(exec, e->s_comp));
        launches += K * per_step;
      } else {
        for (int i = 0; i < K; ++i) GX_TRY(enqueue(i));
      }
      GX_CUDA(cudaMemcpyAsync(e->h_ctl, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, e->s_comp));
      cudaError_t err = cudaStreamSynchronize(e->s_comp);
      if (err != cudaSuccess) return fail(GX_ERR_CUDA, "superstep loop: %s", cudaGetErrorString(err));
      const int ran = std::min(K, e->h_ctl->step - steps_before);
      for (int i = 0; i < ran && prof; ++i) {
        float t = 0;
        GX_CUDA(cudaEventElapsedTime(&t, pev[2 * i], pev[2 * i + 1]));
        ms_pull += t;
      }
      pull_launches += ran;
      steps_before = e->h_ctl->step;
      GX_TRY(checkpoint(*e->h_ctl));
      if (e->h_ctl->done) break;
      // Apps without push steps get the out-edge CSR that marks their
      // selective steps' shards the first time a step turns selective; until
      // then (and where vertexout.npy disagrees with the shards) a selective
      // step sweeps every shard.
      if (e->h_ctl->mark_mode == MARK_NONE && e->h_ctl->mode == MODE_SELECTIVE && !e->out_unbuildable) {
        if (build_out_edges(e, false) == GX_OK) {
          const int mm = MARK_OUT;
          const void* ptrs[2] = {e->d_ooff, e->d_ocol};
          GX_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(e->d_ctl) + offsetof(Ctl, mark_mode), &mm, sizeof(int),
                                  cudaMemcpyHostToDevice, e->s_comp));
          GX_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(e->d_ctl) + offsetof(Ctl, ooff), ptrs, sizeof(ptrs),
                                  cudaMemcpyHostToDevice, e->s_comp));
          GX_CUDA(cudaStreamSynchronize(e->s_comp));
        } else {
          e->out_unbuildable = true;
        }
      }
    }
  } else {
    // Host-driven steps: one launch per shard, streamed shards through the
    // slot ring on the copy stream, overlapped with compute.  A Jacobi step
    // may sweep its shards in any order, so streamed shards are spread evenly
    // among the resident ones: the copy engine then works through the whole
    // step instead of waiting for the resident shards' compute.
    const int slots = e->n_slots;
    // Compressed shards are read by the COMP variant of the pull kernel.
    void (*pull_comp)(PullArgs) = e->cfg.exact_order ? pull_kernel<APP, true, false, true>
                                                     : pull_kernel<APP, false, false, true>;
    if constexpr (APP == K_SSSP_UNIT || APP == K_SSSP_W || APP == K_CC) {
      if (c.async_mode) pull_comp = pull_kernel<APP, false, true, true>;
    }
    std::vector<int32_t> order;
    {
      std::vector<int32_t> res, str;
      for (int32_t p = 0; p < e->P; ++p) (e->resident[p] ? res : str).push_back(p);
      const int64_t S = static_cast<int64_t>(str.size()), Pn = e->P;
      size_t i_r = 0, i_s = 0;
      for (int64_t pos = 0; pos < Pn; ++pos) {
        const bool take_s = i_s < str.size() && (i_r >= res.size() || (2 * static_cast<int64_t>(i_s) + 1) * Pn <= 2 * pos * S);
        order.push_back(take_s ? str[i_s++] : res[i_r++]);
      }
    }
    cudaEvent_t c0, c1, k0, k1;
    GX_CUDA(cudaEventCreate(&c0));
    GX_CUDA(cudaEventCreate(&c1));
    GX_CUDA(cudaEventCreate(&k0));
    GX_CUDA(cudaEventCreate(&k1));
    int slot = 0;
    host_shards_active.assign(static_cast<size_t>(std::max(prm.max_iter, 1)), -1);
    std::vector<char> shard_on(static_cast<size_t>(e->P), 1);
    std::vector<int32_t> changed;
    for (int step = prm.first_step; step < prm.max_iter; ++step) {
      GX_CUDA(cudaMemcpyAsync(e->h_ctl, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, e->s_comp));
      GX_CUDA(cudaStreamSynchronize(e->s_comp));
      const Ctl& hc = *e->h_ctl;
      GX_TRY(checkpoint(hc));
      if (hc.done) break;
      const bool sel = hc.mode == MODE_SELECTIVE;
      // A selective step streams and sweeps only the shards in which the
      // last step's changed vertices are sources.
      std::fill(shard_on.begin(), shard_on.end(), 1);
      if (sel && !hc.list_overflow) {
        if (e->shard_set_words == 0) GX_TRY(build_shard_sets(e));
        const unsigned n = std::min<unsigned>(hc.n_changed_list, static_cast<unsigned>(e->changed_cap));
        changed.resize(n);
        if (n)
          GX_CUDA(cudaMemcpyAsync(changed.data(), e->d_changed_list, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                                  e->s_comp));
        GX_CUDA(cudaStreamSynchronize(e->s_comp));
        const int words = e->shard_set_words;
        std::vector<unsigned long long> m(words, 0ull);
        for (int32_t u : changed)
          for (int w = 0; w < words; ++w) m[w] |= e->h_shard_sets[static_cast<size_t>(u) * words + w];
        int n_on = 0;
        for (int32_t p = 0; p < e->P; ++p) n_on += shard_on[p] = (m[p >> 6] >> (p & 63)) & 1ull;
        host_shards_active[hc.step] = n_on;
      }
      {
        const unsigned int zero[2] = {0u, 0u};  // n_changed_list, list_overflow
        GX_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(e->d_ctl) + offsetof(Ctl, n_changed_list), zero,
                                sizeof(zero), cudaMemcpyHostToDevice, e->s_comp));
      }
      GX_CUDA(cudaEventRecord(k0, e->s_comp));
      GX_CUDA(cudaEventRecord(c0, e->s_comp));
      for (const int32_t p : order) {
        PullArgs sp = pa;
        sp.u_begin = e->unit_begin[p];
        sp.u_end = e->unit_begin[p + 1];
        sp.ctr = e->d_work + 2 * kQueues + kQueues * p;
        if (sp.u_end == sp.u_begin) continue;
        const bool active = shard_on[p] != 0;
        const bool use_comp = e->comp && !e->resident[p] && active && e->cb_bytes[p] > 0;
        if (use_comp) {
          cudaStream_t cs = e->s_copies[slot % e->s_copies.size()];
          GX_CUDA(cudaStreamWaitEvent(cs, e->slot_free[slot], 0));
          GX_CUDA(cudaMemcpyAsync(e->slot_blob[slot], e->h_cblob + e->cb_off[p], e->cb_bytes[p],
                                  cudaMemcpyHostToDevice, cs));
          h2d_bytes += e->cb_bytes[p];
          GX_CUDA(cudaEventRecord(e->slot_ready[slot], cs));
          GX_CUDA(cudaStreamWaitEvent(e->s_comp, e->slot_ready[slot], 0));
          const uint8_t* base = e->slot_blob[slot];
          sp.col = nullptr;
          sp.w = nullptr;
          sp.chdr = reinterpret_cast<const uint2*>(base) - e->cb_c0[p];
          sp.cpay = reinterpret_cast<const uint32_t*>(base + e->cb_pay[p]);
          sp.w8 = base + e->cb_w8[p] - 32 * e->cb_c0[p];
          ++streamed;
        } else if (e->resident[p]) {
          sp.col = e->d_col + e->dev_base[p];
          if (e->d_w) sp.w = e->d_w + e->dev_base[p];
          sp.skip = !active;
        } else if (!active) {
          // Not streamed: the launch only carries the shard's values over.
          sp.col = nullptr;
          sp.w = nullptr;
          sp.skip = 1;
        } else {
          const int64_t lo = e->off[e->bounds[p]] & ~3ll;
          const int64_t n = std::min<int64_t>((e->off[e->bounds[p + 1]] + 3) & ~3ll, e->E + 4) - lo;
          // Slots alternate over the copy streams, so several copy engines
          // move shards at once.
          cudaStream_t cs = e->s_copies[slot % e->s_copies.size()];
          GX_CUDA(cudaStreamWaitEvent(cs, e->slot_free[slot], 0));
          GX_CUDA(cudaMemcpyAsync(e->slot_col[slot], e->h_col + lo, n * sizeof(int32_t), cudaMemcpyHostToDevice, cs));
          h2d_bytes += n * sizeof(int32_t);
          if (weighted) {
            GX_CUDA(cudaMemcpyAsync(e->slot_w[slot], e->h_w + lo, n * sizeof(uint32_t), cudaMemcpyHostToDevice, cs));
            h2d_bytes += n * sizeof(uint32_t);
          }
          GX_CUDA(cudaEventRecord(e->slot_ready[slot], cs));
          GX_CUDA(cudaStreamWaitEvent(e->s_comp, e->slot_ready[slot], 0));
          sp.col = e->slot_col[slot] - lo;
          if (weighted) sp.w = e->slot_w[slot] - lo;
          ++streamed;
        }
        const int units = sp.u_end - sp.u_begin;
        const int grid = std::max(1, std::min(grid_pull, (units + kWarps - 1) / kWarps));
        if (use_comp) pull_comp<<<grid, kThreads, 0, e->s_comp>>>(sp);
        else pull<<<grid, kThreads, 0, e->s_comp>>>(sp);
        GX_CUDA(cudaGetLastError());
        ++launches;
        ++pull_launches;
        if (!e->resident[p] && active) {
          GX_CUDA(cudaEventRecord(e->slot_free[slot], e->s_comp));
          slot = (slot + 1) % slots;
        }
      }
      GX_CUDA(cudaEventRecord(k1, e->s_comp));
      finalize_kernel<APP><<<grid_fin, kThreads, 0, e->s_comp>>>(fa);
      GX_CUDA(cudaGetLastError());
      ++launches;
      // Copy time: from the step's start to the last copy stream's end.
      float ms_c = 0, ms_k = 0;
      for (cudaStream_t cs : e->s_copies) {
        GX_CUDA(cudaEventRecord(c1, cs));
        GX_CUDA(cudaEventSynchronize(c1));
        float t = 0;
        cudaEventElapsedTime(&t, c0, c1);
        ms_c = std::max(ms_c, t);
      }
      GX_CUDA(cudaStreamSynchronize(e->s_comp));
      cudaEventElapsedTime(&ms_k, k0, k1);
      copy_ms += ms_c;
      comp_ms += ms_k;
    }
    cudaEventDestroy(c0);
    cudaEventDestroy(c1);
    cudaEventDestroy(k0);
    cudaEventDestroy(k1);
  }
  GX_CUDA(cudaEventRecord(ev1, e->s_comp));
  GX_CUDA(cudaEventSynchronize(ev1));
  GX_CUDA(cudaMemcpy(e->h_ctl, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  float ms = 0;
  GX_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));

  // The superstep kernels raise one error: a push frontier that outgrew its
  // buffer (impossible by construction, checked on every write).
  if (e->h_ctl->error != 0)
    return fail(GX_ERR_CUDA, "gx_run: device error %d (%s)", e->h_ctl->error,
                e->h_ctl->error == 2 ? "push frontier overflow" : "unknown");
  GX_TRY(checkpoint(*e->h_ctl));
  const int32_t steps = e->h_ctl->step;
  e->last_steps = steps;
  e->last_stats.assign(std::max(steps, 0), StepStats{});
  if (steps > 0)
    GX_CUDA(cudaMemcpy(e->last_stats.data(), e->d_stats, sizeof(StepStats) * steps, cudaMemcpyDeviceToHost));
  for (int32_t i = 0; i < steps && i < static_cast<int32_t>(host_shards_active.size()); ++i)
    if (host_shards_active[i] >= 0) e->last_stats[i].shards_active = host_shards_active[i];
  gx_run_stats rs{};
  rs.iterations = steps;
  for (const StepStats& s : e->last_stats) {
    rs.edges_scanned += static_cast<int64_t>(s.edges);
    rs.push_iterations += s.mode == MODE_PUSH;
  }
  if (steps > 0) {
    rs.changed_last = static_cast<int64_t>(e->last_stats[steps - 1].changed);
    rs.residual_l1_last = static_cast<double>(e->last_stats[steps - 1].resid_fx) / c.fx_scale;
  }
  rs.ms_total = ms;
  rs.ms_copy = copy_ms;
  rs.ms_compute = e->all_resident ? ms : comp_ms;
  rs.h2d_bytes = h2d_bytes;
  rs.shards_resident = e->n_resident;
  rs.shards_streamed = streamed;
  rs.kernel_launches = launches;
  rs.pull_launches = pull_launches;
  rs.ms_pull = ms_pull;
  if (!e->all_resident && copy_ms > 0 && comp_ms > 0) {
    const double lo_t = std::min(copy_ms, comp_ms), hi_t = std::max(copy_ms, comp_ms);
    rs.overlap = std::max(0.0, std::min(1.0, 1.0 - (ms - hi_t) / lo_t));
  }
  e->last_run = rs;
  e->last_app = prm.app;
  e->last_weighted = APP == K_SSSP_W;
  if (out) *out = rs;
  return GX_OK;
}

}  // namespace

extern "C" {

void gx_config_default(gx_config* cfg) {
  if (!cfg) return;
  cfg->device = 0;
  cfg->cache_budget_bytes = -1;
  cfg->stream_slots = 4;
  cfg->copy_streams = 1;
  cfg->selective_threshold = 0.001;
  cfg->heavy_degree = 4096;
  cfg->tile_edges = 2048;
  cfg->exact_order = 0;
  cfg->push_sparse = 1;
  cfg->use_graph = 1;
  cfg->wait_limit = 1u << 24;
  cfg->verbose = 0;
  cfg->profile = 0;
  cfg->push_edge_fraction = 0.5;
  cfg->compress_cache = 1;
  cfg->hot_vertices = 0;
  cfg->relabel = 0;
}

void gx_run_params_default(gx_run_params* p, gx_app app) {
  if (!p) return;
  p->app = app;
  p->max_iter = 10;
  p->damping = 0.85;
  p->source = app == GX_APP_SSSP ? 1 : 0;
  p->weighted = 0;
  p->tolerance = 0;
  p->use_init = 0;
  p->first_step = 0;
  p->async_mode = 0;
  p->checkpoint_every = 0;
  p->checkpoint_prefix = nullptr;
}

gx_status gx_create(const gx_config* cfg, gx_engine** out) {
  if (!out) return fail(GX_ERR_INVALID, "gx_create: out is NULL");
  *out = nullptr;
  gx_config c;
  gx_config_default(&c);
  if (cfg) c = *cfg;
  int n = 0;
  cudaError_t err = cudaGetDeviceCount(&n);
  if (err != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(GX_ERR_NODEVICE, "no CUDA device visible (%s)", cudaGetErrorString(err));
  }
  if (c.device < 0 || c.device >= n) return fail(GX_ERR_INVALID, "device %d out of range [0,%d)", c.device, n);
  if (!(c.push_edge_fraction >= 0.0 && c.push_edge_fraction <= 1.0))
    return fail(GX_ERR_INVALID, "push_edge_fraction %g outside [0,1]", c.push_edge_fraction);
  if (c.wait_limit == 0) return fail(GX_ERR_INVALID, "wait_limit must be at least 1");
  std::unique_ptr<gx_engine> e(new gx_engine());
  e->cfg = c;
  e->dev = c.device;
  GX_CUDA(cudaSetDevice(e->dev));
  GX_CUDA(cudaDeviceGetAttribute(&e->n_sm, cudaDevAttrMultiProcessorCount, e->dev));
  GX_CUDA(cudaDeviceGetAttribute(&e->pageable_access, cudaDevAttrPageableMemoryAccess, e->dev));
  GX_CUDA(cudaStreamCreateWithFlags(&e->s_comp, cudaStreamNonBlocking));
  GX_CUDA(cudaStreamCreateWithFlags(&e->s_copy, cudaStreamNonBlocking));
  e->s_copies.push_back(e->s_copy);
  for (int i = 1; i < std::max(1, c.copy_streams); ++i) {
    cudaStream_t cs;
    GX_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    e->s_copies.push_back(cs);
  }
  GX_TRY(alloc_ctl(e.get()));
  *out = e.release();
  return GX_OK;
}

gx_status gx_destroy(gx_engine* e) {
  if (!e) return GX_OK;
  delete e;
  return GX_OK;
}

gx_status gx_set_wait_limit(gx_engine* e, uint32_t polls) {
  if (!e || polls == 0) return fail(GX_ERR_INVALID, "gx_set_wait_limit: engine NULL or limit 0");
  e->cfg.wait_limit = polls;
  return GX_OK;
}

gx_status gx_release_cached_memory(int32_t device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(GX_ERR_NODEVICE, "no CUDA device visible");
  }
  if (device < 0 || device >= n) return fail(GX_ERR_INVALID, "device %d out of range [0,%d)", device, n);
  int prev = 0;
  GX_CUDA(cudaGetDevice(&prev));
  GX_CUDA(cudaSetDevice(device));
  DevicePool* dp = device_pool(device);
  cudaError_t err = dp ? cudaMemPoolTrimTo(dp->pool, 0) : cudaSuccess;
  cudaSetDevice(prev);
  if (err != cudaSuccess) return fail(GX_ERR_CUDA, "cudaMemPoolTrimTo: %s", cudaGetErrorString(err));
  return GX_OK;
}

gx_status gx_load_csc(gx_engine* e, int32_t V, int32_t P, const int32_t* bounds, const int64_t* off,
                      const int32_t* col, const int32_t* outdeg) {
  gx::NvtxRange nvtx_range("gx_load_csc");
  const auto t_start = std::chrono::steady_clock::now();
  auto phase = [&](const char* what) {
    if (e && e->cfg.verbose)
      fprintf(stderr, "gx_load_csc %-12s %8.2f ms\n", what,
              std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count());
  };
  if (!e) return fail(GX_ERR_INVALID, "gx_load_csc: engine is NULL");
  if (V <= 0 || P <= 0 || !bounds || !off || (off[V] > 0 && !col))
    return fail(GX_ERR_INVALID, "gx_load_csc: bad arguments (V=%d, P=%d)", V, P);
  if (bounds[0] != 0 || bounds[P] != V) return fail(GX_ERR_INVALID, "gx_load_csc: bounds must run from 0 to V");
  for (int32_t p = 0; p < P; ++p)
    if (bounds[p] > bounds[p + 1]) return fail(GX_ERR_INVALID, "gx_load_csc: bounds not monotone at %d", p);
  if (off[0] != 0) return fail(GX_ERR_INVALID, "gx_load_csc: off[0] must be 0");
  const int64_t E = off[V];
  if (E > (int64_t(1) << 40)) return fail(GX_ERR_INVALID, "gx_load_csc: too many edges");
  GX_CUDA(cudaSetDevice(e->dev));
  e->release_graph();
  e->V = V;
  e->P = P;
  e->E = E;
  // Without a shard-cache budget every shard is resident: the offsets, the
  // out-degrees and the source ids go to the device at once, on the copy
  // stream, while the host prepares the work units below.
  const bool direct = e->cfg.cache_budget_bytes < 0;
  // Relabelling (config.relabel) for resident loads whose sort keys (shard,
  // degree rank, vertex id) fit 64 bits and whose lists fit 32-bit lengths.
  const bool relabel = direct && e->cfg.relabel != 0 && bits_for(V) + 12 + bits_for(P) <= 64 &&
                       E <= static_cast<int64_t>(UINT32_MAX);
  LoadScratch scratch(e->s_copy);
  if (relabel) {
    GX_TRY(relabel_load(e, bounds, off, col, outdeg, scratch));
    phase("relabelled");
  } else if (direct) {
    GX_TRY(dev_alloc(&e->d_off, static_cast<size_t>(V) + 1));
    GX_TRY(dev_alloc(&e->d_col, static_cast<size_t>(E) + 8));
    GX_CUDA(cudaMemsetAsync(e->d_col + E, 0, 8 * sizeof(int32_t), e->s_copy));
    GX_TRY(upload_async(e, e->d_off, off, sizeof(int64_t) * (static_cast<size_t>(V) + 1), e->s_copy));
    GX_TRY(upload_async(e, e->d_col, col, sizeof(int32_t) * static_cast<size_t>(E), e->s_copy));
    if (outdeg) {
      GX_TRY(dev_alloc(&e->d_outdeg, static_cast<size_t>(V)));
      GX_TRY(upload_async(e, e->d_outdeg, outdeg, sizeof(int32_t) * static_cast<size_t>(V), e->s_copy));
    }
    // Behind the uploads: the load-time checks.
    GX_TRY(dev_alloc(&scratch.flag, 1));
    GX_CUDA(cudaMemsetAsync(scratch.flag, 0, sizeof(unsigned int), e->s_copy));
    validate_csc_kernel<<<e->n_sm * 8, 256, 0, e->s_copy>>>(e->d_off, V, e->d_col, E, scratch.flag);
    GX_CUDA(cudaGetLastError());
  }
  e->bounds.assign(bounds, bounds + P + 1);
  if (!relabel) {
    e->off.resize(static_cast<size_t>(V) + 1);
    e->outdeg.resize(static_cast<size_t>(V));
    int64_t* hoff = e->off.data();
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v <= V; ++v) hoff[v] = off[v];
    if (outdeg) {
      int32_t* hod = e->outdeg.data();
#pragma omp parallel for schedule(static)
      for (int64_t v = 0; v < V; ++v) hod[v] = outdeg[v];
    } else {
      gx_status st = gx_out_degree(V, off, col, e->outdeg.data());
      if (st != GX_OK) return st;
    }
    int64_t n_dang = 0;
#pragma omp parallel for reduction(+ : n_dang)
    for (int32_t v = 0; v < V; ++v) n_dang += e->outdeg[v] == 0;
    e->n_dangling = n_dang;
  }
  // With a shard-cache budget not every shard reaches the device: check the
  // source ids on the host.  Otherwise the device checks them after the
  // upload, before any kernel indexes with them.
  if (e->cfg.cache_budget_bytes >= 0) {
    int bad = 0;
#pragma omp parallel for reduction(| : bad)
    for (int32_t v = 0; v < V; ++v) bad |= off[v] > off[v + 1];
    if (bad) return fail(GX_ERR_INVALID, "gx_load_csc: off is not non-decreasing");
#pragma omp parallel for reduction(| : bad)
    for (int64_t k = 0; k < E; ++k) bad |= (col[k] < 0 || col[k] >= V);
    if (bad) return fail(GX_ERR_INVALID, "gx_load_csc: source id outside [0, %d)", V);
  }
  phase("validated");
  // Without a shard-cache budget every shard is resident: upload straight
  // from the caller's array.  With a budget, keep a pinned host copy, the
  // streaming source of the shards that do not fit.
  const int32_t* src_col = col;
  if (e->cfg.cache_budget_bytes >= 0) {
    GX_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&e->h_col), (E + 8) * sizeof(int32_t), cudaHostAllocDefault));
    memset(e->h_col + E, 0, 8 * sizeof(int32_t));
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < E; ++k) e->h_col[k] = col[k];
    src_col = e->h_col;
  }

  build_units(e);
  phase("units");
  if (!direct) {
    GX_TRY(dev_alloc(&e->d_off, static_cast<size_t>(V) + 1));
    GX_CUDA(cudaMemcpy(e->d_off, off, sizeof(int64_t) * (V + 1), cudaMemcpyHostToDevice));
  }
  if (!relabel && !(direct && outdeg)) {
    GX_TRY(dev_alloc(&e->d_outdeg, static_cast<size_t>(V)));
    GX_CUDA(cudaMemcpy(e->d_outdeg, e->outdeg.data(), sizeof(int32_t) * V, cudaMemcpyHostToDevice));
  }
  for (int i = 0; i < 2; ++i) {
    uint32_t* vp = nullptr;
    GX_TRY(dev_alloc(&vp, static_cast<size_t>(V)));
    e->d_val[i] = vp;
    GX_TRY(dev_alloc(&e->d_con[i], static_cast<size_t>(V)));
  }
  const size_t U = e->units.size();
  GX_TRY(dev_alloc(&e->d_units, U));
  GX_TRY(dev_alloc(&e->d_unit_shard, U));
  if (U) {
    GX_CUDA(cudaMemcpy(e->d_units, e->units.data(), sizeof(int2) * U, cudaMemcpyHostToDevice));
    GX_CUDA(cudaMemcpy(e->d_unit_shard, e->unit_shard.data(), sizeof(int32_t) * U, cudaMemcpyHostToDevice));
  }
  GX_TRY(dev_alloc(&e->d_heavy, e->heavy.size()));
  if (!e->heavy.empty())
    GX_CUDA(cudaMemcpy(e->d_heavy, e->heavy.data(), sizeof(int4) * e->heavy.size(), cudaMemcpyHostToDevice));
  {
    uint32_t* pp = nullptr;
    GX_TRY(dev_alloc(&pp, static_cast<size_t>(e->n_partials)));
    e->d_partial = pp;
  }
  GX_TRY(dev_alloc(&e->d_hticket, e->heavy.size()));
  e->n_words = (V + 31) / 32 + 2;
  GX_TRY(dev_alloc(&e->d_bm, static_cast<size_t>(e->n_words)));
  e->n_work = kQueues * (P + 2);
  GX_TRY(dev_alloc(&e->d_work, static_cast<size_t>(e->n_work)));
  phase("vertex arrays");
  if (direct) {
    unsigned int h = 0;
    cudaError_t err = cudaMemcpyAsync(&h, scratch.flag, sizeof(h), cudaMemcpyDeviceToHost, e->s_copy);
    if (err == cudaSuccess) err = cudaStreamSynchronize(e->s_copy);
    if (err != cudaSuccess) return fail(GX_ERR_CUDA, "gx_load_csc upload: %s", cudaGetErrorString(err));
    phase("uploaded");
    if (h & 1u) {
      e->release_graph();
      return fail(GX_ERR_INVALID, "gx_load_csc: off is not non-decreasing");
    }
    if (h & 2u) {
      e->release_graph();
      return fail(GX_ERR_INVALID, "gx_load_csc: source id outside [0, %d)", V);
    }
    e->relabeled = relabel;
  }
  GX_TRY(plan_shards(e, src_col, direct));
  if (!direct) {
    // Offsets non-decreasing, and (fully resident) every source id in range.
    unsigned int* flag = nullptr;
    GX_TRY(dev_alloc(&flag, 1));
    GX_CUDA(cudaMemsetAsync(flag, 0, sizeof(unsigned int), e->s_comp));
    validate_csc_kernel<<<e->n_sm * 8, 256, 0, e->s_comp>>>(e->d_off, V, e->all_resident ? e->d_col : nullptr, E,
                                                             flag);
    unsigned int h = 0;
    cudaError_t err = cudaMemcpyAsync(&h, flag, sizeof(h), cudaMemcpyDeviceToHost, e->s_comp);
    if (err == cudaSuccess) err = cudaStreamSynchronize(e->s_comp);
    gx::pool_free(flag);
    if (err != cudaSuccess) return fail(GX_ERR_CUDA, "gx_load_csc validation: %s", cudaGetErrorString(err));
    if (h & 1u) {
      e->release_graph();
      return fail(GX_ERR_INVALID, "gx_load_csc: off is not non-decreasing");
    }
    if (h & 2u) {
      e->release_graph();
      return fail(GX_ERR_INVALID, "gx_load_csc: source id outside [0, %d)", V);
    }
  }
  phase("edges");
  // Shard bounds and bitmaps of the selective steps; the changed-vertex list
  // that streamed graphs hand to the host (a selective step changes fewer
  // than BF_THRE * V vertices).
  if (!relabel) {
    GX_TRY(dev_alloc(&e->d_bounds, static_cast<size_t>(P) + 1));
    GX_CUDA(cudaMemcpy(e->d_bounds, bounds, sizeof(int32_t) * (P + 1), cudaMemcpyHostToDevice));
  }
  GX_TRY(dev_alloc(&e->d_shard_bm, 2 * static_cast<size_t>((P + 31) / 32)));
  if (!e->all_resident) {
    e->changed_cap = std::max<int64_t>(4096, V / 256);
    GX_TRY(dev_alloc(&e->d_changed_list, static_cast<size_t>(e->changed_cap)));
    GX_TRY(build_shard_sets(e));
  }
  phase("shard sets");
  if (e->all_resident) {
    if (e->h_col) cudaFreeHost(e->h_col);
    e->h_col = nullptr;
  }
  e->loaded = true;
  return GX_OK;
}

gx_status gx_load_shards(gx_engine* e, const char* dir, int32_t V, int32_t P) {
  gx::NvtxRange nvtx_range("gx_load_shards");
  if (!e || !dir) return fail(GX_ERR_INVALID, "gx_load_shards: bad arguments");
  int64_t E = 0;
  GX_TRY(gx_read_shards(dir, V, P, nullptr, nullptr, nullptr, nullptr, &E));
  std::vector<int32_t> bounds(P + 1), outdeg(V);
  std::vector<int64_t> off(static_cast<size_t>(V) + 1);
  std::vector<int32_t> col(static_cast<size_t>(E) + 1);
  GX_TRY(gx_read_shards(dir, V, P, bounds.data(), off.data(), col.data(), outdeg.data(), &E));
  return gx_load_csc(e, V, P, bounds.data(), off.data(), col.data(), outdeg.data());
}

gx_status gx_set_weights(gx_engine* e, const uint32_t* w) {
  gx::NvtxRange nvtx_range("gx_set_weights");
  if (!e || !w) return fail(GX_ERR_INVALID, "gx_set_weights: bad arguments");
  if (!e->loaded) return fail(GX_ERR_STATE, "gx_set_weights: no graph loaded");
  GX_CUDA(cudaSetDevice(e->dev));
  if (!e->all_resident && !e->h_col) return fail(GX_ERR_STATE, "gx_set_weights: streaming source missing");
  if (e->all_resident && e->cfg.cache_budget_bytes < 0) {
    // No budget: the weights go straight to the device (a relabelled engine
    // moves them into its own layout there).
    e->has_weights = true;
    GX_TRY(dev_alloc(&e->d_w, static_cast<size_t>(e->E) + 8));
    GX_CUDA(cudaMemsetAsync(e->d_w + e->E, 0, 8 * sizeof(uint32_t), e->s_copy));
    if (e->relabeled) {
      LoadScratch sc(e->s_copy);
      GX_TRY(dev_alloc(&sc.longs, relabel_longs_cap(e->E)));
      GX_TRY(dev_alloc(&sc.n_longs, 1));
      GX_TRY(dev_alloc(&sc.flag, 1));
      GX_CUDA(cudaMemsetAsync(sc.flag, 0, sizeof(unsigned int), e->s_copy));
      GX_TRY(dev_alloc(&sc.col_old, static_cast<size_t>(std::max<int64_t>(e->E, 1))));
      GX_TRY(upload_async(e, sc.col_old, w, sizeof(uint32_t) * static_cast<size_t>(e->E), e->s_copy));
      GX_TRY(relabel_scatter(e, sc.col_old, reinterpret_cast<int32_t*>(e->d_w), false, sc.longs, sc.n_longs, sc.flag,
                             e->s_copy));
    } else {
      GX_TRY(upload_async(e, e->d_w, w, sizeof(uint32_t) * static_cast<size_t>(e->E), e->s_copy));
    }
    GX_CUDA(cudaStreamSynchronize(e->s_copy));
    e->out_built = false;
    return GX_OK;
  }
  if (e->h_w) cudaFreeHost(e->h_w);
  e->h_w = nullptr;
  GX_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&e->h_w), (e->E + 8) * sizeof(uint32_t), cudaHostAllocDefault));
  memcpy(e->h_w, w, e->E * sizeof(uint32_t));
  memset(e->h_w + e->E, 0, 8 * sizeof(uint32_t));
  e->has_weights = true;
  {
    uint32_t mx = 0;
    const int64_t E = e->E;
#pragma omp parallel for reduction(max : mx)
    for (int64_t k = 0; k < E; ++k) mx = std::max(mx, w[k]);
    e->w_narrow = mx <= 255u;  // byte weights in the compressed shard cache
  }
  if (e->all_resident) {
    // Resident plan with the weights: re-plan against the budget, which now
    // counts 8 bytes per edge.
    if (e->cfg.cache_budget_bytes >= 0) {
      // Need the column data on the host again to re-plan.
      GX_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&e->h_col), (e->E + 8) * sizeof(int32_t), cudaHostAllocDefault));
      GX_CUDA(cudaMemcpy(e->h_col, e->d_col, (e->E + 8) * sizeof(int32_t), cudaMemcpyDeviceToHost));
      GX_TRY(plan_shards(e, e->h_col, false));
      if (!e->all_resident && !e->d_changed_list) {
        e->changed_cap = std::max<int64_t>(4096, e->V / 256);
        GX_TRY(dev_alloc(&e->d_changed_list, static_cast<size_t>(e->changed_cap)));
      }
      if (!e->all_resident && e->shard_set_words == 0) GX_TRY(build_shard_sets(e));
      if (e->all_resident) {
        cudaFreeHost(e->h_col);
        e->h_col = nullptr;
      }
    } else {
      GX_TRY(dev_alloc(&e->d_w, static_cast<size_t>(e->E) + 8));
      GX_CUDA(cudaMemset(e->d_w, 0, (e->E + 8) * sizeof(uint32_t)));
      GX_CUDA(cudaMemcpy(e->d_w, w, e->E * sizeof(uint32_t), cudaMemcpyHostToDevice));
    }
  } else {
    GX_TRY(plan_shards(e, e->h_col, false));
  }
  if (e->all_resident) {
    cudaFreeHost(e->h_w);
    e->h_w = nullptr;
  }
  e->out_built = false;
  return GX_OK;
}

gx_status gx_set_init(gx_engine* e, const void* host_vals) {
  if (!e || !host_vals) return fail(GX_ERR_INVALID, "gx_set_init: bad arguments");
  if (!e->loaded) return fail(GX_ERR_STATE, "gx_set_init: no graph loaded");
  e->init_vals.resize(e->V);
  memcpy(e->init_vals.data(), host_vals, sizeof(uint32_t) * e->V);
  e->has_init = true;
  return GX_OK;
}

gx_status gx_run(gx_engine* e, const gx_run_params* prm, gx_run_stats* stats) {
  gx::NvtxRange nvtx_range("gx_run");
  if (!e || !prm) return fail(GX_ERR_INVALID, "gx_run: bad arguments");
  if (!e->loaded) return fail(GX_ERR_STATE, "gx_run: no graph loaded");
  if (prm->max_iter < 0) return fail(GX_ERR_INVALID, "gx_run: max_iter < 0");
  const int kind = app_kind(*prm);
  if (kind < 0) return fail(GX_ERR_INVALID, "gx_run: unknown app %d", static_cast<int>(prm->app));
  if (prm->app == GX_APP_SSSP && (prm->source < 0 || prm->source >= e->V))
    return fail(GX_ERR_INVALID, "gx_run: SSSP source %d outside [0, %d)", prm->source, e->V);
  if (kind == K_SSSP_W && !e->has_weights) return fail(GX_ERR_STATE, "gx_run: weighted SSSP needs gx_set_weights");
  if (prm->first_step < 0 || (prm->max_iter > 0 && prm->first_step >= prm->max_iter))
    return fail(GX_ERR_INVALID, "gx_run: first_step %d outside [0, max_iter=%d)", prm->first_step, prm->max_iter);
  if (prm->first_step > 0 && !prm->use_init)
    return fail(GX_ERR_INVALID, "gx_run: first_step > 0 resumes from gx_set_init values; set use_init");
  if (prm->async_mode && !(kind == K_SSSP_UNIT || kind == K_SSSP_W || kind == K_CC))
    return fail(GX_ERR_INVALID, "gx_run: async_mode is for SSSP and CC");
  if (prm->checkpoint_every < 0 || (prm->checkpoint_every > 0 && !prm->checkpoint_prefix))
    return fail(GX_ERR_INVALID, "gx_run: checkpoint_every needs checkpoint_prefix");
  GX_CUDA(cudaSetDevice(e->dev));
  gx_run_params p = *prm;
  if (p.max_iter == 0) {
    e->last_steps = 0;
    e->last_stats.clear();
    if (stats) *stats = gx_run_stats{};
    return GX_OK;
  }
  gx_status st = GX_ERR_INVALID;
  switch (kind) {
    case K_PR_REF: st = run_app<K_PR_REF>(e, p, stats); break;
    case K_PR_STD: st = run_app<K_PR_STD>(e, p, stats); break;
    case K_SSSP_UNIT: st = run_app<K_SSSP_UNIT>(e, p, stats); break;
    case K_SSSP_W: st = run_app<K_SSSP_W>(e, p, stats); break;
    case K_CC: st = run_app<K_CC>(e, p, stats); break;
    case K_INDEG: st = run_app<K_INDEG>(e, p, stats); break;
  }
  e->device_init = false;
  return st;
}

gx_status gx_get_values(gx_engine* e, void* host_out) {
  gx::NvtxRange nvtx_range("gx_get_values");
  if (!e || !host_out) return fail(GX_ERR_INVALID, "gx_get_values: bad arguments");
  if (!e->loaded) return fail(GX_ERR_STATE, "gx_get_values: no graph loaded");
  GX_CUDA(cudaSetDevice(e->dev));
  GX_CUDA(cudaMemcpy(e->h_ctl, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  const int cur = e->h_ctl->cur & 1;
  const void* src = e->d_val[cur];
  if (e->relabeled) {
    GX_TRY(values_to_caller(e, src, e->s_comp));
    src = e->d_stage;
  }
  GX_CUDA(cudaMemcpy(host_out, src, sizeof(uint32_t) * e->V, cudaMemcpyDeviceToHost));
  return GX_OK;
}

gx_status gx_write_values_npy(gx_engine* e, const char* path) {
  if (!e || !path) return fail(GX_ERR_INVALID, "gx_write_values_npy: bad arguments");
  if (!e->loaded) return fail(GX_ERR_STATE, "gx_write_values_npy: no graph loaded");
  std::vector<uint32_t> buf(static_cast<size_t>(e->V));
  GX_TRY(gx_get_values(e, buf.data()));
  const bool pr = e->last_app == GX_APP_PAGERANK_REF || e->last_app == GX_APP_PAGERANK_STD;
  const bool wt = e->last_app == GX_APP_SSSP && e->last_weighted;
  if (!write_npy_4(path, buf.data(), e->V, pr ? "<f4" : (wt ? "<u4" : "<i4")))
    return fail(GX_ERR_IO, "cannot write %s", path);
  return GX_OK;
}

gx_status gx_get_device_graph(gx_engine* e, gx_device_graph* out) {
  if (!e || !out) return fail(GX_ERR_INVALID, "gx_get_device_graph: bad arguments");
  if (!e->loaded) return fail(GX_ERR_STATE, "gx_get_device_graph: no graph loaded");
  if (!e->all_resident) return fail(GX_ERR_STATE, "gx_get_device_graph: some shards are not resident");
  if (e->relabeled)
    return fail(GX_ERR_STATE, "gx_get_device_graph: the engine renumbered the vertices (config.relabel); load "
                              "without it");
  out->V = e->V;
  out->P = e->P;
  out->E = e->E;
  out->off = e->d_off;
  out->col = e->d_col;
  out->w = e->has_weights ? e->d_w : nullptr;
  out->outdeg = e->d_outdeg;
  out->bounds = e->d_bounds;
  out->stream = e->s_comp;
  return GX_OK;
}

gx_status gx_get_iter_stats(gx_engine* e, int32_t step, gx_iter_stats* out) {
  if (!e || !out) return fail(GX_ERR_INVALID, "gx_get_iter_stats: bad arguments");
  if (step < 0 || step >= e->last_steps)
    return fail(GX_ERR_INVALID, "gx_get_iter_stats: step %d outside [0, %d)", step, e->last_steps);
  const StepStats& s = e->last_stats[step];
  const double fx = static_cast<double>(e->V) * 1073741824.0;
  out->changed = static_cast<int64_t>(s.changed);
  out->active = static_cast<int64_t>(s.active);
  out->shards_active = s.shards_active < 0 ? e->P : s.shards_active * 1;
  out->mode = s.mode;
  out->residual_l1 = static_cast<double>(s.resid_fx) / fx;
  out->dangling = static_cast<double>(s.dangl_fx) / fx;
  out->edges_scanned = static_cast<int64_t>(s.edges);
  return GX_OK;
}

}  // extern "C"

// Graph construction on the GPU: edge list (or seeded R-MAT) -> CSC with
// sources ascending within each destination, self-loops dropped,
// duplicates removed and the graph symmetrised on request.  It produces
// exactly what gx_build_csc computes on the host, in place of the offline
// Spark job (GraphMP/tools/format_spark.py) and cal.cpp's degree pass.
//
// Pipeline (all on one stream, two key buffers of 8 bytes per edge):
//   1. keys: (dst << sb) | src for every kept edge (and its reverse when
//      symmetrising), compacted with one atomic per warp;
//   2. LSD radix sort of the keys, 8 bits per pass over 2*sb bits, each pass
//      a per-tile digit histogram, an exclusive scan of the (digit, tile)
//      counts and a stable scatter (warps own consecutive sub-tiles; lanes
//      rank within a warp with __match_any_sync);
//   3. one more scan over "first of its run" flags gives each kept key its
//      position: col = the key's source, off[v] = position of the first key
//      whose destination is >= v.
// The output does not depend on the order of the keys before the sort
// (equal keys are identical), so the atomic compaction in step 1 leaves it
// deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "gx_engine.h"
#include "gx_nvtx.h"

using namespace gx;

namespace {

constexpr int kBuildThreads = 256;
constexpr int kRadixItems = 32;                                 // keys per thread per tile
constexpr int kRadixTile = kBuildThreads * kRadixItems;         // 8192 keys per block
constexpr int kRadixWarps = kBuildThreads / 32;
constexpr int kWarpSpan = kRadixTile / kRadixWarps;             // consecutive keys per warp
constexpr int kScanItems = 16;
constexpr int kScanTile = kBuildThreads * kScanItems;           // 4096 elements per block
constexpr unsigned kBadId = 1u;

__device__ __forceinline__ void push_key(unsigned long long* keys, unsigned long long* count, bool keep,
                                         unsigned long long key, int lane) {
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  if (!m) return;
  unsigned long long base = 0;
  const int leader = __ffs(m) - 1;
  if (lane == leader) base = atomicAdd(count, static_cast<unsigned long long>(__popc(m)));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (keep) keys[base + __popc(m & ((1u << lane) - 1u))] = key;
}

// Keys of a device edge list.  Every thread of a warp runs the same number of
// loop trips, so the ballots see full warps.
__global__ void keys_from_edges_kernel(const int32_t* src, const int32_t* dst, int64_t n, int32_t V, int sb,
                                       int drop_self, int sym, unsigned long long* keys,
                                       unsigned long long* count, unsigned int* err) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x; b < n; b += stride) {
    const int64_t i = b + threadIdx.x;
    bool ok = false;
    int32_t s = 0, d = 0;
    if (i < n) {
      s = src[i];
      d = dst[i];
      ok = s >= 0 && s < V && d >= 0 && d < V;
      if (!ok) atomicOr(err, kBadId);
      if (ok && drop_self && s == d) ok = false;
    }
    const unsigned long long us = static_cast<uint32_t>(s), ud = static_cast<uint32_t>(d);
    push_key(keys, count, ok, (ud << sb) | us, lane);
    if (sym) push_key(keys, count, ok, (us << sb) | ud, lane);
  }
}

struct RmatParams {
  int scale;
  uint32_t ta, tb, tc;
  unsigned long long key0;
  int64_t first;
};

// The generator of gx_rmat_edges (gx_graph.cpp), edge by edge on the device.
__device__ __forceinline__ void rmat_edge(const RmatParams& r, int64_t k, uint32_t* s_out, uint32_t* d_out) {
  const uint64_t i = static_cast<uint64_t>(r.first + k);
  const uint64_t key = r.key0 ^ (i * 0xd1b54a32d192ed03ull);
  uint32_t s = 0, d = 0;
  for (int lv = 0; lv < r.scale; lv += 4) {
    const uint64_t h = mix64(key + static_cast<uint64_t>(lv / 4 + 1) * 0x9e3779b97f4a7c15ull);
    for (int j = 0; j < 4 && lv + j < r.scale; ++j) {
      const uint32_t u = static_cast<uint32_t>(h >> (16 * j)) & 0xffffu;
      const uint32_t bit = 1u << (r.scale - 1 - (lv + j));
      if (u < r.ta) {
      } else if (u < r.tb) {
        d |= bit;
      } else if (u < r.tc) {
        s |= bit;
      } else {
        s |= bit;
        d |= bit;
      }
    }
  }
  *s_out = s;
  *d_out = d;
}

__global__ void keys_from_rmat_kernel(RmatParams r, int64_t n, int sb, int drop_self, int sym,
                                      unsigned long long* keys, unsigned long long* count) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x; b < n; b += stride) {
    const int64_t i = b + threadIdx.x;
    bool ok = false;
    uint32_t s = 0, d = 0;
    if (i < n) {
      rmat_edge(r, i, &s, &d);
      ok = !(drop_self && s == d);
    }
    const unsigned long long us = s, ud = d;
    push_key(keys, count, ok, (ud << sb) | us, lane);
    if (sym) push_key(keys, count, ok, (us << sb) | ud, lane);
  }
}

// Digit histogram of one tile: hist[digit * n_tiles + tile].
__global__ void __launch_bounds__(kBuildThreads) radix_hist_kernel(const unsigned long long* keys, int64_t n,
                                                                   int shift, uint32_t* hist, int64_t n_tiles) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * kRadixTile;
  for (int j = 0; j < kRadixItems; ++j) {
    const int64_t i = t0 + static_cast<int64_t>(j) * kBuildThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[static_cast<int64_t>(threadIdx.x) * n_tiles + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter of one tile.  Warp w owns keys [t0 + w*kWarpSpan, +kWarpSpan)
// and places them after the tile's keys of the same digit in warps < w.
__global__ void __launch_bounds__(kBuildThreads) radix_scatter_kernel(const unsigned long long* in,
                                                                      unsigned long long* out, int64_t n, int shift,
                                                                      const unsigned long long* offs,
                                                                      int64_t n_tiles) {
  __shared__ uint32_t wcnt[kRadixWarps][256];
  __shared__ unsigned long long base[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kRadixWarps * 256; i += kBuildThreads) wcnt[i >> 8][i & 255] = 0;
  base[threadIdx.x] = offs[static_cast<int64_t>(threadIdx.x) * n_tiles + blockIdx.x];
  __syncthreads();
  const int64_t w0 = static_cast<int64_t>(blockIdx.x) * kRadixTile + static_cast<int64_t>(warp) * kWarpSpan;
  for (int it = 0; it < kWarpSpan / 32; ++it) {
    const int64_t i = w0 + it * 32 + lane;
    if (i < n) atomicAdd(&wcnt[warp][(in[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  {
    const int d = threadIdx.x;
    uint32_t run = 0;
    for (int w = 0; w < kRadixWarps; ++w) {
      const uint32_t c = wcnt[w][d];
      wcnt[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
  for (int it = 0; it < kWarpSpan / 32; ++it) {
    const int64_t i = w0 + it * 32 + lane;
    const bool valid = i < n;
    const unsigned long long key = valid ? in[i] : 0ull;
    const int d = valid ? static_cast<int>((key >> shift) & 255u) : 256;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    const uint32_t b = valid ? wcnt[warp][d] : 0u;
    if (valid) out[base[d] + b + rank] = key;
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = b + __popc(peers);
    __syncwarp();
  }
}

// ---- exclusive scan of m counts (uint32) into uint64 offsets ----

__device__ __forceinline__ unsigned long long block_excl_scan(unsigned long long x, unsigned long long* total) {
  __shared__ unsigned long long s_w[kBuildThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long incl = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) s_w[warp] = incl;
  __syncthreads();
  unsigned long long wbase = 0, tot = 0;
  for (int w = 0; w < kBuildThreads / 32; ++w) {
    if (w < warp) wbase += s_w[w];
    tot += s_w[w];
  }
  __syncthreads();
  *total = tot;
  return wbase + incl - x;
}

__global__ void __launch_bounds__(kBuildThreads) scan_partial_kernel(const uint32_t* in, int64_t m,
                                                                     unsigned long long* part) {
  unsigned long long s = 0;
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
  for (int j = 0; j < kScanItems; ++j)
    if (t0 + j < m) s += in[t0 + j];
  unsigned long long tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// In-place exclusive scan of the per-block partials by one block.
__global__ void __launch_bounds__(kBuildThreads) scan_partials_kernel(unsigned long long* part, int64_t np) {
  unsigned long long carry = 0;
  for (int64_t c0 = 0; c0 < np; c0 += kBuildThreads) {
    const int64_t i = c0 + threadIdx.x;
    const unsigned long long x = i < np ? part[i] : 0ull;
    unsigned long long tot;
    const unsigned long long ex = block_excl_scan(x, &tot);
    if (i < np) part[i] = carry + ex;
    carry += tot;
  }
}

__global__ void __launch_bounds__(kBuildThreads) scan_final_kernel(const uint32_t* in, int64_t m,
                                                                   const unsigned long long* part,
                                                                   unsigned long long* out) {
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
  unsigned long long s = 0;
  for (int j = 0; j < kScanItems; ++j)
    if (t0 + j < m) s += in[t0 + j];
  unsigned long long tot;
  unsigned long long run = part[blockIdx.x] + block_excl_scan(s, &tot);
  for (int j = 0; j < kScanItems; ++j)
    if (t0 + j < m) {
      out[t0 + j] = run;
      run += in[t0 + j];
    }
}

// ---- CSC from the sorted keys ----

__device__ __forceinline__ bool first_of_run(const unsigned long long* k, int64_t i, int dedup) {
  return !dedup || i == 0 || k[i] != k[i - 1];
}

__global__ void __launch_bounds__(kBuildThreads) unique_partial_kernel(const unsigned long long* k, int64_t n,
                                                                       int dedup, unsigned long long* part) {
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
  unsigned long long s = 0;
  for (int j = 0; j < kScanItems; ++j)
    if (t0 + j < n) s += first_of_run(k, t0 + j, dedup);
  unsigned long long tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// col[pos] = source of each kept key; off[v] for v in (dst of the previous
// key, dst of this key] = pos.  The vertices after the last key's
// destination are filled by tail_offsets_kernel.
__global__ void __launch_bounds__(kBuildThreads) unique_write_kernel(const unsigned long long* k, int64_t n,
                                                                     int dedup, int sb,
                                                                     const unsigned long long* part, int32_t* col,
                                                                     int64_t* off) {
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
  unsigned long long s = 0;
  for (int j = 0; j < kScanItems; ++j)
    if (t0 + j < n) s += first_of_run(k, t0 + j, dedup);
  unsigned long long tot;
  unsigned long long pos = part[blockIdx.x] + block_excl_scan(s, &tot);
  const unsigned long long smask = (1ull << sb) - 1ull;
  for (int j = 0; j < kScanItems; ++j) {
    const int64_t i = t0 + j;
    if (i >= n || !first_of_run(k, i, dedup)) continue;
    const unsigned long long key = k[i];
    col[pos] = static_cast<int32_t>(key & smask);
    const int64_t d = static_cast<int64_t>(key >> sb);
    const int64_t dprev = i == 0 ? -1 : static_cast<int64_t>(k[i - 1] >> sb);
    for (int64_t v = dprev + 1; v <= d; ++v) off[v] = static_cast<int64_t>(pos);
    ++pos;
  }
}

__global__ void tail_offsets_kernel(int64_t* off, int64_t v0, int32_t V, int64_t E) {
  for (int64_t v = v0 + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; v <= V;
       v += static_cast<int64_t>(gridDim.x) * blockDim.x)
    off[v] = E;
}

struct BuildBuffers {
  unsigned long long* keys[2] = {nullptr, nullptr};
  uint32_t* hist = nullptr;
  unsigned long long* offs = nullptr;
  unsigned long long* part = nullptr;
  unsigned long long* count = nullptr;
  unsigned int* err = nullptr;
  int32_t* src = nullptr;
  int32_t* dst = nullptr;
  int32_t* col = nullptr;
  int64_t* off = nullptr;
  cudaStream_t s = nullptr;
  ~BuildBuffers() {
    if (s) cudaStreamSynchronize(s);
    dev_free(&keys[0]);
    dev_free(&keys[1]);
    dev_free(&hist);
    dev_free(&offs);
    dev_free(&part);
    dev_free(&count);
    dev_free(&err);
    dev_free(&src);
    dev_free(&dst);
    dev_free(&col);
    dev_free(&off);
    if (s) cudaStreamDestroy(s);
  }
};

gx_status scan_counts(BuildBuffers& B, const uint32_t* in, int64_t m, unsigned long long* out, int n_sm) {
  (void)n_sm;
  const int64_t nb = (m + kScanTile - 1) / kScanTile;
  scan_partial_kernel<<<static_cast<unsigned>(nb), kBuildThreads, 0, B.s>>>(in, m, B.part);
  scan_partials_kernel<<<1, kBuildThreads, 0, B.s>>>(B.part, nb);
  scan_final_kernel<<<static_cast<unsigned>(nb), kBuildThreads, 0, B.s>>>(in, m, B.part, out);
  GX_CUDA(cudaGetLastError());
  return GX_OK;
}

// Sorts n keys of 2*sb significant bits (result in B.keys[*which]) and
// writes the CSC to host off[V+1] / col[...].
gx_status sort_and_emit(BuildBuffers& B, int64_t n, int sb, int32_t V, bool dedup, int n_sm, int64_t* h_off,
                        int32_t* h_col, int64_t* n_out) {
  int cur = 0;
  if (n > 0) {
    const int64_t n_tiles = (n + kRadixTile - 1) / kRadixTile;
    if (n_tiles > INT32_MAX / 2) return fail(GX_ERR_INVALID, "gx build: %lld keys are too many", (long long)n);
    GX_TRY(dev_alloc(&B.hist, static_cast<size_t>(256 * n_tiles)));
    GX_TRY(dev_alloc(&B.offs, static_cast<size_t>(256 * n_tiles)));
    const int64_t scan_blocks = std::max<int64_t>((256 * n_tiles + kScanTile - 1) / kScanTile,
                                                  (n + kScanTile - 1) / kScanTile);
    GX_TRY(dev_alloc(&B.part, static_cast<size_t>(scan_blocks)));
    for (int shift = 0; shift < 2 * sb; shift += 8) {
      radix_hist_kernel<<<static_cast<unsigned>(n_tiles), kBuildThreads, 0, B.s>>>(B.keys[cur], n, shift, B.hist,
                                                                                  n_tiles);
      GX_CUDA(cudaGetLastError());
      GX_TRY(scan_counts(B, B.hist, 256 * n_tiles, B.offs, n_sm));
      radix_scatter_kernel<<<static_cast<unsigned>(n_tiles), kBuildThreads, 0, B.s>>>(
          B.keys[cur], B.keys[cur ^ 1], n, shift, B.offs, n_tiles);
      GX_CUDA(cudaGetLastError());
      cur ^= 1;
    }
  }
  // Kept keys -> col / off on the device.
  GX_TRY(dev_alloc(&B.off, static_cast<size_t>(V) + 1));
  GX_TRY(dev_alloc(&B.col, static_cast<size_t>(std::max<int64_t>(n, 1))));
  int64_t E = 0;
  if (n > 0) {
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    unique_partial_kernel<<<static_cast<unsigned>(nb), kBuildThreads, 0, B.s>>>(B.keys[cur], n, dedup, B.part);
    // The partials' total (E) is read back from the last one after the scan.
    unsigned long long last_part = 0, last_pref = 0;
    GX_CUDA(cudaMemcpyAsync(&last_part, B.part + nb - 1, sizeof(last_part), cudaMemcpyDeviceToHost, B.s));
    scan_partials_kernel<<<1, kBuildThreads, 0, B.s>>>(B.part, nb);
    GX_CUDA(cudaMemcpyAsync(&last_pref, B.part + nb - 1, sizeof(last_pref), cudaMemcpyDeviceToHost, B.s));
    unique_write_kernel<<<static_cast<unsigned>(nb), kBuildThreads, 0, B.s>>>(B.keys[cur], n, dedup, sb, B.part,
                                                                            B.col, B.off);
    GX_CUDA(cudaGetLastError());
    unsigned long long last_key = 0;
    GX_CUDA(cudaMemcpyAsync(&last_key, B.keys[cur] + n - 1, sizeof(last_key), cudaMemcpyDeviceToHost, B.s));
    GX_CUDA(cudaStreamSynchronize(B.s));
    E = static_cast<int64_t>(last_pref + last_part);
    const int64_t v0 = static_cast<int64_t>(last_key >> sb) + 1;
    tail_offsets_kernel<<<n_sm * 4, 256, 0, B.s>>>(B.off, v0, V, E);
  } else {
    tail_offsets_kernel<<<n_sm * 4, 256, 0, B.s>>>(B.off, 0, V, 0);
  }
  GX_CUDA(cudaGetLastError());
  GX_CUDA(cudaMemcpyAsync(h_off, B.off, sizeof(int64_t) * (static_cast<size_t>(V) + 1), cudaMemcpyDeviceToHost, B.s));
  if (E > 0) GX_CUDA(cudaMemcpyAsync(h_col, B.col, sizeof(int32_t) * E, cudaMemcpyDeviceToHost, B.s));
  GX_CUDA(cudaStreamSynchronize(B.s));
  *n_out = E;
  return GX_OK;
}

int key_bits(int32_t V) {
  int sb = 1;
  while (sb < 31 && (int64_t(1) << sb) < V) ++sb;
  return sb;
}

gx_status begin_build(int32_t device, BuildBuffers& B, int* n_sm) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(GX_ERR_NODEVICE, "no CUDA device visible");
  }
  if (device < 0 || device >= n) return fail(GX_ERR_INVALID, "device %d out of range [0,%d)", device, n);
  GX_CUDA(cudaSetDevice(device));
  GX_CUDA(cudaDeviceGetAttribute(n_sm, cudaDevAttrMultiProcessorCount, device));
  GX_CUDA(cudaStreamCreateWithFlags(&B.s, cudaStreamNonBlocking));
  GX_TRY(dev_alloc(&B.count, 1));
  GX_TRY(dev_alloc(&B.err, 1));
  GX_CUDA(cudaMemsetAsync(B.count, 0, sizeof(unsigned long long), B.s));
  GX_CUDA(cudaMemsetAsync(B.err, 0, sizeof(unsigned int), B.s));
  return GX_OK;
}

}  // namespace

namespace gx {

void radix_scratch_sizes(int64_t n, int64_t* hist_elems, int64_t* part_elems) {
  const int64_t n_tiles = std::max<int64_t>((n + kRadixTile - 1) / kRadixTile, 1);
  *hist_elems = 256 * n_tiles;
  *part_elems = std::max<int64_t>((256 * n_tiles + kScanTile - 1) / kScanTile, (n + kScanTile - 1) / kScanTile) + 1;
}

gx_status radix_sort_bits(unsigned long long* keys, unsigned long long* tmp, int64_t n, int lo_bit, int hi_bit,
                          uint32_t* hist, unsigned long long* offs, unsigned long long* part, cudaStream_t s,
                          unsigned long long** sorted) {
  unsigned long long* buf[2] = {keys, tmp};
  int cur = 0;
  if (n > 0) {
    const int64_t n_tiles = (n + kRadixTile - 1) / kRadixTile;
    if (n_tiles > INT32_MAX / 2) return fail(GX_ERR_INVALID, "radix sort: %lld keys are too many", (long long)n);
    for (int shift = lo_bit; shift < hi_bit; shift += 8) {
      radix_hist_kernel<<<static_cast<unsigned>(n_tiles), kBuildThreads, 0, s>>>(buf[cur], n, shift, hist, n_tiles);
      GX_TRY(scan_u32(hist, 256 * n_tiles, offs, part, s));
      radix_scatter_kernel<<<static_cast<unsigned>(n_tiles), kBuildThreads, 0, s>>>(buf[cur], buf[cur ^ 1], n, shift,
                                                                                  offs, n_tiles);
      GX_CUDA(cudaGetLastError());
      cur ^= 1;
    }
  }
  *sorted = buf[cur];
  return GX_OK;
}

gx_status scan_u32(const uint32_t* in, int64_t m, unsigned long long* out, unsigned long long* part, cudaStream_t s) {
  if (m <= 0) return GX_OK;
  const int64_t nb = (m + kScanTile - 1) / kScanTile;
  scan_partial_kernel<<<static_cast<unsigned>(nb), kBuildThreads, 0, s>>>(in, m, part);
  scan_partials_kernel<<<1, kBuildThreads, 0, s>>>(part, nb);
  scan_final_kernel<<<static_cast<unsigned>(nb), kBuildThreads, 0, s>>>(in, m, part, out);
  GX_CUDA(cudaGetLastError());
  return GX_OK;
}

}  // namespace gx

extern "C" {

gx_status gx_build_csc_gpu(int32_t device, int32_t V, int64_t n, const int32_t* src, const int32_t* dst,
                           int32_t flags, int64_t* off, int32_t* col, int64_t* n_out) {
  gx::NvtxRange nvtx_range("gx_build_csc_gpu");
  if (V < 0 || n < 0 || !off || (n > 0 && (!src || !dst || !col)) || !n_out)
    return fail(GX_ERR_INVALID, "gx_build_csc_gpu: bad arguments");
  BuildBuffers B;
  int n_sm = 0;
  GX_TRY(begin_build(device, B, &n_sm));
  const bool sym = flags & GX_BUILD_SYMMETRIZE;
  const int64_t cap = sym ? 2 * n : n;
  const int sb = key_bits(V);
  GX_TRY(dev_alloc(&B.keys[0], static_cast<size_t>(std::max<int64_t>(cap, 1))));
  GX_TRY(dev_alloc(&B.keys[1], static_cast<size_t>(std::max<int64_t>(cap, 1))));
  unsigned long long kept = 0;
  if (n > 0) {
    GX_TRY(dev_alloc(&B.src, static_cast<size_t>(n)));
    GX_TRY(dev_alloc(&B.dst, static_cast<size_t>(n)));
    GX_CUDA(cudaMemcpyAsync(B.src, src, sizeof(int32_t) * n, cudaMemcpyHostToDevice, B.s));
    GX_CUDA(cudaMemcpyAsync(B.dst, dst, sizeof(int32_t) * n, cudaMemcpyHostToDevice, B.s));
    keys_from_edges_kernel<<<n_sm * 8, kBuildThreads, 0, B.s>>>(B.src, B.dst, n, V, sb,
                                                                (flags & GX_BUILD_DROP_SELF) ? 1 : 0, sym ? 1 : 0,
                                                                B.keys[0], B.count, B.err);
    GX_CUDA(cudaGetLastError());
    unsigned int err = 0;
    GX_CUDA(cudaMemcpyAsync(&kept, B.count, sizeof(kept), cudaMemcpyDeviceToHost, B.s));
    GX_CUDA(cudaMemcpyAsync(&err, B.err, sizeof(err), cudaMemcpyDeviceToHost, B.s));
    GX_CUDA(cudaStreamSynchronize(B.s));
    if (err & kBadId) return fail(GX_ERR_INVALID, "gx_build_csc_gpu: vertex id outside [0, %d)", V);
    dev_free(&B.src);
    dev_free(&B.dst);
  }
  return sort_and_emit(B, static_cast<int64_t>(kept), sb, V, (flags & GX_BUILD_DEDUP) != 0, n_sm, off, col, n_out);
}

gx_status gx_rmat_csc_gpu(int32_t device, int32_t scale, int64_t n, double a, double b, double c, uint64_t seed,
                          int32_t flags, int64_t* off, int32_t* col, int64_t* n_out) {
  gx::NvtxRange nvtx_range("gx_rmat_csc_gpu");
  if (scale < 1 || scale > 30 || n < 0 || !off || (n > 0 && !col) || !n_out)
    return fail(GX_ERR_INVALID, "gx_rmat_csc_gpu: bad arguments (scale %d, n %lld)", scale,
                static_cast<long long>(n));
  if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0 + 1e-12)
    return fail(GX_ERR_INVALID, "gx_rmat_csc_gpu: bad quadrant probabilities");
  BuildBuffers B;
  int n_sm = 0;
  GX_TRY(begin_build(device, B, &n_sm));
  const int32_t V = 1 << scale;
  const bool sym = flags & GX_BUILD_SYMMETRIZE;
  const int64_t cap = sym ? 2 * n : n;
  const int sb = key_bits(V);
  GX_TRY(dev_alloc(&B.keys[0], static_cast<size_t>(std::max<int64_t>(cap, 1))));
  GX_TRY(dev_alloc(&B.keys[1], static_cast<size_t>(std::max<int64_t>(cap, 1))));
  RmatParams r;
  r.scale = scale;
  r.ta = static_cast<uint32_t>(std::llround(a * 65536.0));
  r.tb = r.ta + static_cast<uint32_t>(std::llround(b * 65536.0));
  r.tc = r.tb + static_cast<uint32_t>(std::llround(c * 65536.0));
  r.key0 = mix64(seed ^ 0x5ca1ab1e0ddba11ull);
  r.first = 0;
  unsigned long long kept = 0;
  if (n > 0) {
    keys_from_rmat_kernel<<<n_sm * 8, kBuildThreads, 0, B.s>>>(r, n, sb, (flags & GX_BUILD_DROP_SELF) ? 1 : 0,
                                                               sym ? 1 : 0, B.keys[0], B.count);
    GX_CUDA(cudaGetLastError());
    GX_CUDA(cudaMemcpyAsync(&kept, B.count, sizeof(kept), cudaMemcpyDeviceToHost, B.s));
    GX_CUDA(cudaStreamSynchronize(B.s));
  }
  return sort_and_emit(B, static_cast<int64_t>(kept), sb, V, (flags & GX_BUILD_DEDUP) != 0, n_sm, off, col, n_out);
}

}  // extern "C"

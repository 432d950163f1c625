// Triangle counting on the loaded graph, taken as undirected: the CSC of a
// symmetrised, deduplicated edge list (each undirected edge stored in both
// directions, no self-loops).  No reference counterpart: the reference's
// only "tc" (GraphH/list/system/GraphPS.h:15-95) counts reciprocal edges.
//
//  1. orient u -> v iff (deg u, u) < (deg v, v) (a DAG; every triangle has
//     exactly one vertex whose two out-neighbours close it);
//  2. build the oriented adjacency N+(u) with warp-ballot compaction, which
//     keeps the ascending id order of the input lists;
//  3. count sum over u, v in N+(u) of |N+(u) ∩ N+(v)|: a warp stages N+(u)
//     in shared memory and its lanes binary-search every w of N+(v) in it.
//     Vertices are claimed in descending |N+(u)| order; lists too long for
//     a warp's slice get a whole CTA, and the rare list beyond the CTA's
//     shared memory is searched in place in global memory.
// Counts are exact (64-bit integer sums).
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <numeric>
#include <vector>

#include "gx_engine.h"

using namespace gx;

namespace {

constexpr int kTcThreads = 256;
constexpr int kTcWarps = kTcThreads / 32;
constexpr int kWarpList = 1024;             // N+(u) entries staged per warp
constexpr int kCtaList = 48 * 1024;         // entries staged per CTA (192 KB)
constexpr int kTcGrab = 4;                  // vertices a warp claims per atomic

__global__ void tc_degree_kernel(const int64_t* off, int32_t V, int32_t* deg) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    deg[v] = static_cast<int32_t>(off[v + 1] - off[v]);
}

__device__ __forceinline__ bool tc_before(int32_t du, int32_t u, int32_t dv, int32_t v) {
  return du < dv || (du == dv && u < v);
}

// |N+(u)| per vertex (self-loops never qualify: u is not before itself).
__global__ void tc_count_kernel(const int64_t* off, const int32_t* col, const int32_t* deg, int32_t V,
                                int32_t* cnt) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < V; u += warps) {
    const int32_t du = deg[u];
    int c = 0;
    for (int64_t k = off[u] + lane; k < off[u + 1]; k += 32) {
      const int32_t v = col[k];
      c += tc_before(du, u, deg[v], v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) cnt[u] = c;
  }
}

// N+(u), in the input's ascending order, via ballot + popc compaction.
__global__ void tc_fill_kernel(const int64_t* off, const int32_t* col, const int32_t* deg, int32_t V,
                               const int64_t* doff, int32_t* dcol) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < V; u += warps) {
    const int32_t du = deg[u];
    int64_t pos = doff[u];
    for (int64_t base = off[u]; base < off[u + 1]; base += 32) {
      const int64_t k = base + lane;
      int32_t v = 0;
      bool keep = false;
      if (k < off[u + 1]) {
        v = col[k];
        keep = tc_before(du, u, deg[v], v);
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep) dcol[pos + __popc(m & ((1u << lane) - 1u))] = v;
      pos += __popc(m);
    }
  }
}

__device__ __forceinline__ bool tc_search(const int32_t* list, int n, int32_t w) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (list[mid] < w) lo = mid + 1;
    else hi = mid;
  }
  return lo < n && list[lo] == w;
}

// Lanes of one warp intersect N+(v) (global) with the staged list.
__device__ __forceinline__ unsigned long long tc_probe(const int64_t* doff, const int32_t* dcol, const int32_t* list,
                                                       int n, int32_t v, int lane, int stride,
                                                       unsigned long long* work) {
  const int64_t vb = doff[v], ve = doff[v + 1];
  unsigned long long c = 0;
  for (int64_t j = vb + lane; j < ve; j += stride) c += tc_search(list, n, dcol[j]);
  if (lane == 0) *work += ve - vb;
  return c;
}

// Warp per vertex; vertices in `order` (descending |N+|) with |N+| <= kWarpList.
__global__ void __launch_bounds__(kTcThreads) tc_warp_kernel(const int64_t* doff, const int32_t* dcol,
                                                             const int32_t* order, int32_t n_order, unsigned int* ctr,
                                                             unsigned long long* out) {
  __shared__ int32_t s_list[kTcWarps][kWarpList];
  __shared__ unsigned long long s_red[2][kTcWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int32_t* list = s_list[wid];
  unsigned long long cnt = 0, work = 0;
  for (;;) {
    int i0 = 0;
    if (lane == 0) i0 = static_cast<int>(atomicAdd(ctr, static_cast<unsigned>(kTcGrab)));
    i0 = __shfl_sync(0xffffffffu, i0, 0);
    if (i0 >= n_order) break;
    const int i1 = i0 + kTcGrab < n_order ? i0 + kTcGrab : n_order;
    for (int i = i0; i < i1; ++i) {
      const int32_t u = order[i];
      const int64_t b = doff[u];
      const int n = static_cast<int>(doff[u + 1] - b);
      for (int k = lane; k < n; k += 32) list[k] = dcol[b + k];
      __syncwarp();
      for (int k = 0; k < n; ++k) cnt += tc_probe(doff, dcol, list, n, list[k], lane, 32, &work);
      __syncwarp();
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    work += __shfl_xor_sync(0xffffffffu, work, o);
  }
  if (lane == 0) {
    s_red[0][wid] = cnt;
    s_red[1][wid] = work;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    unsigned long long t = 0;
    for (int w = 0; w < kTcWarps; ++w) t += s_red[threadIdx.x][w];
    if (t) atomicAdd(out + threadIdx.x, t);
  }
}

// CTA per vertex for |N+(u)| > kWarpList: the list is staged in dynamic
// shared memory when it fits, else searched where it lies.
__global__ void __launch_bounds__(kTcThreads) tc_cta_kernel(const int64_t* doff, const int32_t* dcol,
                                                            const int32_t* order, int32_t n_order,
                                                            unsigned long long* out) {
  extern __shared__ int32_t s_big[];
  __shared__ unsigned long long s_red[2][kTcWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long cnt = 0, work = 0;
  for (int i = blockIdx.x; i < n_order; i += gridDim.x) {
    const int32_t u = order[i];
    const int64_t b = doff[u];
    const int n = static_cast<int>(doff[u + 1] - b);
    const bool staged = n <= kCtaList;
    const int32_t* list = staged ? s_big : dcol + b;
    if (staged)
      for (int k = threadIdx.x; k < n; k += kTcThreads) s_big[k] = dcol[b + k];
    __syncthreads();
    for (int k = wid; k < n; k += kTcWarps) cnt += tc_probe(doff, dcol, list, n, list[k], lane, 32, &work);
    __syncthreads();
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    work += __shfl_xor_sync(0xffffffffu, work, o);
  }
  if (lane == 0) {
    s_red[0][wid] = cnt;
    s_red[1][wid] = work;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    unsigned long long t = 0;
    for (int w = 0; w < kTcWarps; ++w) t += s_red[threadIdx.x][w];
    if (t) atomicAdd(out + threadIdx.x, t);
  }
}

struct TcBuffers {
  int32_t* deg = nullptr;
  int32_t* cnt = nullptr;
  int64_t* doff = nullptr;
  int32_t* dcol = nullptr;
  int32_t* order = nullptr;
  unsigned long long* out = nullptr;
  unsigned int* ctr = nullptr;
  ~TcBuffers() {
    dev_free(&deg);
    dev_free(&cnt);
    dev_free(&doff);
    dev_free(&dcol);
    dev_free(&order);
    dev_free(&out);
    dev_free(&ctr);
  }
};

}  // namespace

extern "C" gx_status gx_triangle_count(gx_engine* e, uint64_t* total, gx_run_stats* stats) {
  if (!e || !total) return fail(GX_ERR_INVALID, "gx_triangle_count: bad arguments");
  if (!e->loaded) return fail(GX_ERR_STATE, "gx_triangle_count: no graph loaded");
  if (!e->all_resident)
    return fail(GX_ERR_STATE, "gx_triangle_count: needs every shard resident (no shard-cache budget)");
  GX_CUDA(cudaSetDevice(e->dev));
  const int32_t V = e->V;
  cudaStream_t s = e->s_comp;
  TcBuffers b;
  cudaEvent_t ev0, ev1;
  GX_CUDA(cudaEventCreate(&ev0));
  GX_CUDA(cudaEventCreate(&ev1));
  GX_CUDA(cudaEventRecord(ev0, s));
  GX_TRY(dev_alloc(&b.deg, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&b.cnt, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&b.out, 2));
  GX_TRY(dev_alloc(&b.ctr, 1));
  const int grid = e->n_sm * 8;
  tc_degree_kernel<<<grid, 256, 0, s>>>(e->d_off, V, b.deg);
  tc_count_kernel<<<grid, 256, 0, s>>>(e->d_off, e->d_col, b.deg, V, b.cnt);
  GX_CUDA(cudaGetLastError());
  // Offsets of N+ and the claim order (descending |N+|, by power-of-two bins).
  std::vector<int32_t> cnt(V);
  GX_CUDA(cudaMemcpyAsync(cnt.data(), b.cnt, sizeof(int32_t) * V, cudaMemcpyDeviceToHost, s));
  GX_CUDA(cudaStreamSynchronize(s));
  // Prefix sums and the claim order on the host threads: each thread scans
  // and bins a contiguous block of vertices; blocks are joined in order.
  const int nt = std::max(1, omp_get_max_threads());
  std::vector<int64_t> doff(static_cast<size_t>(V) + 1, 0);
  std::vector<int64_t> part(static_cast<size_t>(nt) + 1, 0);
  std::vector<std::vector<std::vector<int32_t>>> tbins(nt, std::vector<std::vector<int32_t>>(34));
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    const int32_t lo = static_cast<int32_t>(static_cast<int64_t>(V) * t / nt);
    const int32_t hi = static_cast<int32_t>(static_cast<int64_t>(V) * (t + 1) / nt);
    int64_t run = 0;
    for (int32_t v = lo; v < hi; ++v) {
      run += cnt[v];
      if (cnt[v] < 2) continue;  // no pair of out-neighbours, no triangle
      tbins[t][cnt[v] > kWarpList ? 33 : 31 - __builtin_clz(static_cast<unsigned>(cnt[v]))].push_back(v);
    }
    part[t + 1] = run;
#pragma omp barrier
#pragma omp single
    for (int i = 0; i < nt; ++i) part[i + 1] += part[i];
    int64_t acc = part[t];
    for (int32_t v = lo; v < hi; ++v) {
      doff[v] = acc;
      acc += cnt[v];
    }
  }
  doff[V] = part[nt];
  const int64_t m = doff[V];
  std::vector<int32_t> big;
  for (int t = 0; t < nt; ++t) big.insert(big.end(), tbins[t][33].begin(), tbins[t][33].end());
  std::sort(big.begin(), big.end(), [&](int32_t a, int32_t c) { return cnt[a] > cnt[c] || (cnt[a] == cnt[c] && a < c); });
  std::vector<int32_t> order(big);
  for (int k = 32; k >= 0; --k)
    for (int t = 0; t < nt; ++t) order.insert(order.end(), tbins[t][k].begin(), tbins[t][k].end());
  const int32_t n_big = static_cast<int32_t>(big.size());
  const int32_t n_small = static_cast<int32_t>(order.size()) - n_big;
  GX_TRY(dev_alloc(&b.doff, static_cast<size_t>(V) + 1));
  GX_TRY(dev_alloc(&b.dcol, static_cast<size_t>(m) + 1));
  GX_TRY(dev_alloc(&b.order, order.size() + 1));
  GX_CUDA(cudaMemcpyAsync(b.doff, doff.data(), sizeof(int64_t) * (V + 1), cudaMemcpyHostToDevice, s));
  if (!order.empty())
    GX_CUDA(cudaMemcpyAsync(b.order, order.data(), sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice, s));
  tc_fill_kernel<<<grid, 256, 0, s>>>(e->d_off, e->d_col, b.deg, V, b.doff, b.dcol);
  GX_CUDA(cudaMemsetAsync(b.out, 0, 2 * sizeof(unsigned long long), s));
  GX_CUDA(cudaMemsetAsync(b.ctr, 0, sizeof(unsigned int), s));
  // The long lists run on the copy stream beside the warp kernel, so the
  // few CTAs they need do not hold the rest of the GPU idle.
  cudaEvent_t filled = nullptr, big_done = nullptr;
  if (n_big > 0) {
    GX_CUDA(cudaEventCreateWithFlags(&filled, cudaEventDisableTiming));
    GX_CUDA(cudaEventCreateWithFlags(&big_done, cudaEventDisableTiming));
    GX_CUDA(cudaEventRecord(filled, s));
    GX_CUDA(cudaStreamWaitEvent(e->s_copy, filled, 0));
    const size_t smem = sizeof(int32_t) * kCtaList;
    GX_CUDA(cudaFuncSetAttribute(tc_cta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    tc_cta_kernel<<<std::min(n_big, e->n_sm), kTcThreads, smem, e->s_copy>>>(b.doff, b.dcol, b.order, n_big, b.out);
    GX_CUDA(cudaEventRecord(big_done, e->s_copy));
  }
  if (n_small > 0) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc_warp_kernel, kTcThreads, 0);
    tc_warp_kernel<<<std::max(1, per_sm) * e->n_sm, kTcThreads, 0, s>>>(b.doff, b.dcol, b.order + n_big, n_small,
                                                                        b.ctr, b.out);
  }
  GX_CUDA(cudaGetLastError());
  if (big_done) {
    GX_CUDA(cudaStreamWaitEvent(s, big_done, 0));
    cudaEventDestroy(filled);
    cudaEventDestroy(big_done);
  }
  unsigned long long res[2] = {0, 0};
  GX_CUDA(cudaMemcpyAsync(res, b.out, sizeof(res), cudaMemcpyDeviceToHost, s));
  GX_CUDA(cudaEventRecord(ev1, s));
  GX_CUDA(cudaEventSynchronize(ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  *total = res[0];
  if (stats) {
    *stats = gx_run_stats{};
    stats->iterations = 1;
    stats->edges_scanned = static_cast<int64_t>(res[1]);
    stats->ms_total = ms;
    stats->ms_compute = ms;
    stats->kernel_launches = 4 + (n_big > 0) + (n_small > 0);
  }
  return GX_OK;
}

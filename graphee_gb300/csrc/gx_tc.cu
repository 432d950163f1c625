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
//     in shared memory with an 8192-bit filter of its ids; its lanes test
//     every w of N+(v) against the filter, and only the ids that pass are
//     queued and binary-searched in the staged list, 32 at a time.
//     Vertices are claimed in descending |N+(u)| order; lists too long for
//     a warp's slice get a whole CTA (a 2^16-bit filter, warps splitting
//     N+(u)), whose shared memory is sized to the longest such list so it
//     runs beside the warp kernel; the rare list beyond kCtaList entries is
//     searched in place in global memory.
// Counts are exact (64-bit integer sums).
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include "gx_engine.h"
#include "gx_nvtx.h"

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

// Warp per vertex u.  Its list is read 8 chunks of 32 at a time, all ids
// and their degrees loaded before any is used, so a hub's long list costs
// one dependent load chain per 256 entries, not per 32 (the hubs set the
// kernels' length).  Self-loops never qualify: u is not before itself.
constexpr int kOrientChunks = 8;

// The oriented graph is built in the caller's numbering: on an engine that
// renumbered its vertices (inv non-null: engine vertex u is the caller's
// inv[u]) the ids are mapped back while the lists are read, so N+ keeps the
// input's ascending id order and the counting kernels below index by the
// caller's ids.  deg stays in the engine's numbering.

// |N+(u)| per vertex.
__global__ void tc_count_kernel(const int64_t* __restrict__ off, const int32_t* __restrict__ col,
                                const int32_t* __restrict__ deg, const int32_t* __restrict__ inv, int32_t V,
                                int32_t* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < V; u += warps) {
    const int32_t du = deg[u];
    const int32_t uo = inv ? inv[u] : u;
    const int64_t e1 = off[u + 1];
    int c = 0;
    for (int64_t base = off[u]; base < e1; base += 32 * kOrientChunks) {
      int32_t v[kOrientChunks], dv[kOrientChunks];
#pragma unroll
      for (int j = 0; j < kOrientChunks; ++j) v[j] = base + 32 * j + lane < e1 ? col[base + 32 * j + lane] : 0;
#pragma unroll
      for (int j = 0; j < kOrientChunks; ++j) dv[j] = base + 32 * j + lane < e1 ? deg[v[j]] : 0;
      if (inv) {
#pragma unroll
        for (int j = 0; j < kOrientChunks; ++j) v[j] = inv[v[j]];
      }
#pragma unroll
      for (int j = 0; j < kOrientChunks; ++j) c += base + 32 * j + lane < e1 && tc_before(du, uo, dv[j], v[j]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) cnt[uo] = c;
  }
}

// N+(u), in the input's ascending order: chunk by chunk, ballot + popc
// compaction.
__global__ void tc_fill_kernel(const int64_t* __restrict__ off, const int32_t* __restrict__ col,
                               const int32_t* __restrict__ deg, const int32_t* __restrict__ inv, int32_t V,
                               const int64_t* __restrict__ doff, int32_t* __restrict__ dcol) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < V; u += warps) {
    const int32_t du = deg[u];
    const int32_t uo = inv ? inv[u] : u;
    int64_t pos = doff[uo];
    const int64_t e1 = off[u + 1];
    for (int64_t base = off[u]; base < e1; base += 32 * kOrientChunks) {
      int32_t v[kOrientChunks], dv[kOrientChunks];
#pragma unroll
      for (int j = 0; j < kOrientChunks; ++j) v[j] = base + 32 * j + lane < e1 ? col[base + 32 * j + lane] : 0;
#pragma unroll
      for (int j = 0; j < kOrientChunks; ++j) dv[j] = base + 32 * j + lane < e1 ? deg[v[j]] : 0;
      if (inv) {
#pragma unroll
        for (int j = 0; j < kOrientChunks; ++j) v[j] = inv[v[j]];
      }
#pragma unroll
      for (int j = 0; j < kOrientChunks; ++j) {
        const bool keep = base + 32 * j + lane < e1 && tc_before(du, uo, dv[j], v[j]);
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) dcol[pos + __popc(m & below)] = v[j];
        pos += __popc(m);
      }
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

// Bit filter of a staged list: bit h(w) is set for every w of the list, so a
// clear bit proves w absent.  Multiplicative hashing spreads R-MAT's
// structured ids over the 2^kFilterBits bits.
constexpr int kFilterBits = 13;                          // a warp's list (<= 1024 ids)
constexpr int kFilterWords = (1 << kFilterBits) / 32;
constexpr int kCtaFilterBits = 16;                       // a CTA's list (> 1024 ids)
constexpr int kCtaFilterWords = (1 << kCtaFilterBits) / 32;
template <int BITS>
__device__ __forceinline__ uint32_t tc_hash(int32_t w) {
  return (static_cast<uint32_t>(w) * 2654435761u) >> (32 - BITS);
}

// Lanes of one warp test every w of N+(v) against the staged list's bit
// filter.  Most probes miss (about 90% on R-MAT) and the filter rejects all
// but 1-2% of those with one shared-memory load; the ids that pass are
// appended to the warp's queue (ballot + prefix) and binary-searched 32 at a
// time, so the searches run with every lane busy.  Two rounds of 32 ids go
// through per loop step, each round's ids loaded a step ahead so the loads'
// latency overlaps the filter tests.  qn (warp-uniform) is the queue's fill:
// below 32 between steps, at most 95 after a step's appends (kQueue slots).
// N+(v) lies at dcol[vb, vb + len).
constexpr int kQueue = 96;
template <int BITS>
__device__ __forceinline__ void tc_probe_filtered(const int32_t* __restrict__ dcol, int64_t vb, int len,
                                                  const int32_t* list, int n, const uint32_t* bits, int32_t* q,
                                                  int& qn, int lane, unsigned long long& cnt,
                                                  unsigned long long& work) {
  const int32_t* nv = dcol + vb;
  if (lane == 0) work += static_cast<unsigned long long>(len);
  const unsigned below = (1u << lane) - 1u;
  int32_t n0 = lane < len ? nv[lane] : 0, n1 = lane + 32 < len ? nv[lane + 32] : 0;
  for (int base = 0; base < len; base += 64) {
    const int j0 = base + lane, j1 = j0 + 32;
    const int32_t w0 = n0, w1 = n1;
    if (j0 + 64 < len) n0 = nv[j0 + 64];
    if (j1 + 64 < len) n1 = nv[j1 + 64];
    bool p0 = false, p1 = false;
    if (j0 < len) {
      const uint32_t h = tc_hash<BITS>(w0);
      p0 = (bits[h >> 5] >> (h & 31)) & 1u;
    }
    if (j1 < len) {
      const uint32_t h = tc_hash<BITS>(w1);
      p1 = (bits[h >> 5] >> (h & 31)) & 1u;
    }
    const unsigned m0 = __ballot_sync(0xffffffffu, p0), m1 = __ballot_sync(0xffffffffu, p1);
    if (p0) q[qn + __popc(m0 & below)] = w0;
    qn += __popc(m0);
    if (p1) q[qn + __popc(m1 & below)] = w1;
    qn += __popc(m1);
    while (qn >= 32) {
      __syncwarp();
      cnt += tc_search(list, n, q[lane]);
      __syncwarp();
      for (int i = lane; i < qn - 32; i += 32) q[i] = q[32 + i];
      qn -= 32;
    }
  }
  __syncwarp();
}

// Warp per vertex; vertices in `order` (descending |N+|) with |N+| <= kWarpList.
__global__ void __launch_bounds__(kTcThreads) tc_warp_kernel(const int64_t* doff, const int32_t* dcol,
                                                             const int32_t* order, int32_t n_order, unsigned int* ctr,
                                                             unsigned long long* out) {
  __shared__ int32_t s_list[kTcWarps][kWarpList];
  __shared__ uint32_t s_bits[kTcWarps][kFilterWords];
  __shared__ int32_t s_q[kTcWarps][kQueue];
  __shared__ unsigned long long s_red[2][kTcWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int32_t* list = s_list[wid];
  uint32_t* bits = s_bits[wid];
  int32_t* q = s_q[wid];
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
      for (int k = lane; k < kFilterWords; k += 32) bits[k] = 0u;
      __syncwarp();
      for (int k = lane; k < n; k += 32) {
        const int32_t x = dcol[b + k];
        list[k] = x;
        const uint32_t h = tc_hash<kFilterBits>(x);
        atomicOr(&bits[h >> 5], 1u << (h & 31));
      }
      __syncwarp();
      int qn = 0;
      // Offsets of N+(v) for the next v are loaded while this one is probed.
      int64_t vb = doff[list[0]], ve = doff[list[0] + 1];
      for (int k = 0; k < n; ++k) {
        int64_t nb = 0, ne = 0;
        if (k + 1 < n) {
          nb = doff[list[k + 1]];
          ne = doff[list[k + 1] + 1];
        }
        tc_probe_filtered<kFilterBits>(dcol, vb, static_cast<int>(ve - vb), list, n, bits, q, qn, lane, cnt, work);
        vb = nb;
        ve = ne;
      }
      // The queue's rest belongs to this list: searched before the next is staged.
      if (lane < qn) cnt += tc_search(list, n, q[lane]);
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

// CTA per vertex for |N+(u)| > kWarpList, claimed one at a time from ctr;
// the CTA's warps split N+(u) and probe through the filter like the warp
// kernel.  Dynamic shared memory holds the 2^16-bit filter, the warps'
// queues, then room for `cap` list entries (the longest list of the launch,
// at most kCtaList); a longer list is searched where it lies in global
// memory, its filter still in shared memory.
__global__ void __launch_bounds__(kTcThreads) tc_cta_kernel(const int64_t* doff, const int32_t* dcol,
                                                            const int32_t* order, int32_t n_order, int cap,
                                                            unsigned int* ctr, unsigned long long* out) {
  extern __shared__ uint32_t s_dyn[];
  uint32_t* bits = s_dyn;
  int32_t* q = reinterpret_cast<int32_t*>(s_dyn + kCtaFilterWords) + kQueue * (threadIdx.x >> 5);
  int32_t* s_big = reinterpret_cast<int32_t*>(s_dyn + kCtaFilterWords) + kQueue * kTcWarps;
  __shared__ unsigned long long s_red[2][kTcWarps];
  __shared__ int s_i;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long cnt = 0, work = 0;
  for (;;) {
    if (threadIdx.x == 0) s_i = static_cast<int>(atomicAdd(ctr, 1u));
    __syncthreads();
    const int i = s_i;
    if (i >= n_order) break;
    const int32_t u = order[i];
    const int64_t b = doff[u];
    const int n = static_cast<int>(doff[u + 1] - b);
    const bool staged = n <= cap;
    const int32_t* list = staged ? s_big : dcol + b;
    for (int k = threadIdx.x; k < kCtaFilterWords; k += kTcThreads) bits[k] = 0u;
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += kTcThreads) {
      const int32_t x = dcol[b + k];
      if (staged) s_big[k] = x;
      const uint32_t h = tc_hash<kCtaFilterBits>(x);
      atomicOr(&bits[h >> 5], 1u << (h & 31));
    }
    __syncthreads();
    int qn = 0;
    for (int k = wid; k < n; k += kTcWarps) {
      const int32_t v = list[k];
      const int64_t vb = doff[v];
      tc_probe_filtered<kCtaFilterBits>(dcol, vb, static_cast<int>(doff[v + 1] - vb), list, n, bits, q, qn, lane,
                                        cnt, work);
    }
    if (lane < qn) cnt += tc_search(list, n, q[lane]);
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
  gx::NvtxRange nvtx_range("gx_triangle_count");
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
  GX_TRY(dev_alloc(&b.ctr, 2));  // claim counters of the warp and CTA kernels
  const int grid = e->n_sm * 8;
  tc_degree_kernel<<<grid, 256, 0, s>>>(e->d_off, V, b.deg);
  const int32_t* inv = e->relabeled ? e->d_inv : nullptr;
  tc_count_kernel<<<grid, 256, 0, s>>>(e->d_off, e->d_col, b.deg, inv, V, b.cnt);
  GX_CUDA(cudaGetLastError());
  // Offsets of N+ and the claim order (descending |N+|, by power-of-two bins).
  // Host buffers are not zero-filled (every element is written below) and are
  // first touched by the threads that fill them.
  std::unique_ptr<int32_t[]> cnt(new int32_t[V]);
  GX_CUDA(cudaMemcpyAsync(cnt.get(), b.cnt, sizeof(int32_t) * V, cudaMemcpyDeviceToHost, s));
  GX_CUDA(cudaStreamSynchronize(s));
  // Prefix sums and the claim order on the host threads: each thread scans
  // and bins a contiguous block of vertices; blocks are joined in order.
  const int nt = std::max(1, omp_get_max_threads());
  std::unique_ptr<int64_t[]> doff(new int64_t[static_cast<size_t>(V) + 1]);
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
  // Claim order: the long lists sorted by (|N+| descending, id), then bins 32
  // down to 0, each bin in thread order; copied in parallel to offsets
  // computed first.
  std::vector<int32_t> big;
  for (int t = 0; t < nt; ++t) big.insert(big.end(), tbins[t][33].begin(), tbins[t][33].end());
  std::sort(big.begin(), big.end(), [&](int32_t a, int32_t c) { return cnt[a] > cnt[c] || (cnt[a] == cnt[c] && a < c); });
  const int32_t n_big = static_cast<int32_t>(big.size());
  std::vector<int64_t> at(static_cast<size_t>(33) * nt);
  int64_t n_order = n_big;
  for (int k = 32; k >= 0; --k)
    for (int t = 0; t < nt; ++t) {
      at[static_cast<size_t>(k) * nt + t] = n_order;
      n_order += static_cast<int64_t>(tbins[t][k].size());
    }
  std::unique_ptr<int32_t[]> order(new int32_t[std::max<int64_t>(n_order, 1)]);
  if (n_big) memcpy(order.get(), big.data(), sizeof(int32_t) * n_big);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int i = 0; i < 33 * nt; ++i) {
    const int k = i / nt, t = i % nt;
    const std::vector<int32_t>& bin = tbins[t][k];
    if (!bin.empty()) memcpy(order.get() + at[i], bin.data(), sizeof(int32_t) * bin.size());
  }
  const int32_t n_small = static_cast<int32_t>(n_order) - n_big;
  GX_TRY(dev_alloc(&b.doff, static_cast<size_t>(V) + 1));
  GX_TRY(dev_alloc(&b.dcol, static_cast<size_t>(m) + 1));
  GX_TRY(dev_alloc(&b.order, static_cast<size_t>(n_order) + 1));
  GX_CUDA(cudaMemcpyAsync(b.doff, doff.get(), sizeof(int64_t) * (V + 1), cudaMemcpyHostToDevice, s));
  if (n_order > 0)
    GX_CUDA(cudaMemcpyAsync(b.order, order.get(), sizeof(int32_t) * n_order, cudaMemcpyHostToDevice, s));
  tc_fill_kernel<<<grid, 256, 0, s>>>(e->d_off, e->d_col, b.deg, inv, V, b.doff, b.dcol);
  GX_CUDA(cudaMemsetAsync(b.out, 0, 2 * sizeof(unsigned long long), s));
  GX_CUDA(cudaMemsetAsync(b.ctr, 0, 2 * sizeof(unsigned int), s));
  // The long lists run on the copy stream beside the warp kernel, so the
  // few CTAs they need do not hold the rest of the GPU idle.
  cudaEvent_t filled = nullptr, big_done = nullptr;
  if (n_big > 0) {
    GX_CUDA(cudaEventCreateWithFlags(&filled, cudaEventDisableTiming));
    GX_CUDA(cudaEventCreateWithFlags(&big_done, cudaEventDisableTiming));
    GX_CUDA(cudaEventRecord(filled, s));
    GX_CUDA(cudaStreamWaitEvent(e->s_copy, filled, 0));
    // Shared memory for the longest list only (big[0]), so the CTAs leave
    // room on their SMs for the warp kernel's.
    const int cap = std::min(cnt[big[0]], kCtaList);
    const size_t smem = sizeof(uint32_t) * (kCtaFilterWords + kQueue * kTcWarps + static_cast<size_t>(cap));
    GX_CUDA(cudaFuncSetAttribute(tc_cta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc_cta_kernel, kTcThreads, smem);
    const int grid_cta = std::min(n_big, std::max(1, per_sm) * e->n_sm);
    tc_cta_kernel<<<grid_cta, kTcThreads, smem, e->s_copy>>>(b.doff, b.dcol, b.order, n_big, cap, b.ctr + 1,
                                                             b.out);
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

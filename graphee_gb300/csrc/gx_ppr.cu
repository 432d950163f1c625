// Multi-source personalized PageRank as a sparse-times-dense product over
// the loaded CSC:  R <- restart*S + (1-restart) * A^T D^-1 R,  R0 = S,
// with R a V x k FP32 matrix (k <= 64 sources, rows padded to 64 columns =
// 256 bytes) and S the one-hot source matrix.  No reference counterpart;
// the per-edge arithmetic is PageRank's pull (GraphMP/app/pagerank.cpp:44-48)
// applied to k rank vectors at once.
//
// HBM layout: Rs[2][V][64] holds R[u,:]/outdeg[u] (double buffer, so an
// edge costs one 256-byte coalesced row gather); the final R is written on
// the last step only.  Work: a warp per destination vertex, vertices with
// more than kPprChunk in-edges split into chunks whose partial rows are
// folded in chunk order by the last warp to finish, so results are
// deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "gx_engine.h"
#include "gx_nvtx.h"

using namespace gx;

namespace {

constexpr int kPprCols = 64;
constexpr int kPprChunk = 1024;
constexpr int kPprThreads = 256;
constexpr int kPprWarps = kPprThreads / 32;

struct PprArgs {
  const int64_t* off;
  const int32_t* col;
  const int32_t* outdeg;
  const float* rs_in;
  float* rs_out;
  float* r_out;             // final R, written when non-null
  const int4* units;        // (v, chunk, n_chunks, partial base)
  int32_t n_units;
  unsigned int* ctr;        // kQueues cursors
  float* partial;           // [n_partial][64]
  unsigned int* ticket;     // per unit-owner with n_chunks > 1, indexed by partial base
  const int32_t* src;       // [64] source vertex of each column (-1 past k)
  float alpha, restart;
};

__device__ __forceinline__ void ppr_finish(const PprArgs& a, int v, float2 acc, int lane) {
  float2 r = make_float2(a.alpha * acc.x, a.alpha * acc.y);
  if (a.src[2 * lane] == v) r.x += a.restart;
  if (a.src[2 * lane + 1] == v) r.y += a.restart;
  const int32_t od = a.outdeg[v];
  const float inv = 1.0f / static_cast<float>(od > 0 ? od : 1);
  const size_t row = static_cast<size_t>(v) * kPprCols + 2 * lane;
  if (a.r_out) *reinterpret_cast<float2*>(a.r_out + row) = r;
  *reinterpret_cast<float2*>(a.rs_out + row) = make_float2(r.x * inv, r.y * inv);
}

__global__ void __launch_bounds__(kPprThreads) ppr_kernel(const PprArgs a) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int U = a.n_units;
  const int nq = U / 256 < 1 ? 1 : (U / 256 < kQueues ? U / 256 : kQueues);
  int q = (blockIdx.x * kPprWarps + wid) % nq;
  for (;;) {
    const int qb = static_cast<int>((static_cast<int64_t>(U) * q) / nq);
    const int qe = static_cast<int>((static_cast<int64_t>(U) * (q + 1)) / nq);
    int u0 = 0;
    if (lane == 0) u0 = qb + static_cast<int>(atomicAdd(a.ctr + q, 2u));
    u0 = __shfl_sync(0xffffffffu, u0, 0);
    if (u0 >= qe) {
      q = next_queue(a.ctr, q, nq, U, lane);
      if (q < 0) break;
      continue;
    }
    const int u1 = u0 + 2 < qe ? u0 + 2 : qe;
    for (int u = u0; u < u1; ++u) {
      const int4 un = a.units[u];
      const int v = un.x;
      const int64_t vb = a.off[v], ve = a.off[v + 1];
      const int64_t b = vb + static_cast<int64_t>(un.y) * kPprChunk;
      const int64_t e = ve < b + kPprChunk ? ve : b + kPprChunk;
      float2 acc = make_float2(0.f, 0.f);
      for (int64_t k0 = b; k0 < e; k0 += 32) {
        const int n = e - k0 < 32 ? static_cast<int>(e - k0) : 32;
        const int32_t mine = lane < n ? __ldcs(a.col + k0 + lane) : 0;
        int j = 0;
        for (; j + 8 <= n; j += 8) {
          float2 x[8];
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int32_t src = __shfl_sync(0xffffffffu, mine, j + t);
            x[t] = __ldg(reinterpret_cast<const float2*>(a.rs_in + static_cast<size_t>(src) * kPprCols) + lane);
          }
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            acc.x += x[t].x;
            acc.y += x[t].y;
          }
        }
        for (; j < n; ++j) {
          const int32_t src = __shfl_sync(0xffffffffu, mine, j);
          const float2 x = __ldg(reinterpret_cast<const float2*>(a.rs_in + static_cast<size_t>(src) * kPprCols) + lane);
          acc.x += x.x;
          acc.y += x.y;
        }
      }
      if (un.z == 1) {
        ppr_finish(a, v, acc, lane);
        continue;
      }
      float2* part = reinterpret_cast<float2*>(a.partial + static_cast<size_t>(un.w + un.y) * kPprCols);
      part[lane] = acc;
      __threadfence();
      __syncwarp();
      unsigned t = 0;
      if (lane == 0) t = atomicAdd(a.ticket + un.w, 1u);
      t = __shfl_sync(0xffffffffu, t, 0);
      if (t == static_cast<unsigned>(un.z) - 1) {
        __threadfence();
        float2 tot = make_float2(0.f, 0.f);
        for (int c = 0; c < un.z; ++c) {
          const volatile float* pp = a.partial + static_cast<size_t>(un.w + c) * kPprCols + 2 * lane;
          tot.x += pp[0];
          tot.y += pp[1];
        }
        ppr_finish(a, v, tot, lane);
        if (lane == 0) a.ticket[un.w] = 0;
      }
    }
  }
}

__global__ void ppr_init_kernel(float* rs, const int32_t* outdeg, const int32_t* src, int k) {
  const int j = threadIdx.x;
  if (j < k) {
    const int v = src[j];
    const int32_t od = outdeg[v];
    rs[static_cast<size_t>(v) * kPprCols + j] = 1.0f / static_cast<float>(od > 0 ? od : 1);
  }
}

}  // namespace

extern "C" gx_status gx_ppr(gx_engine* e, int32_t k, const int32_t* sources, int32_t iters, double restart,
                            float* host_out, gx_run_stats* stats) {
  gx::NvtxRange nvtx_range("gx_ppr");
  if (!e || !sources || k < 1 || k > kPprCols || iters < 0 || restart < 0 || restart > 1)
    return fail(GX_ERR_INVALID, "gx_ppr: bad arguments (k must be 1..64)");
  if (!e->loaded) return fail(GX_ERR_STATE, "gx_ppr: no graph loaded");
  if (!e->all_resident) return fail(GX_ERR_STATE, "gx_ppr: needs every shard resident (no shard-cache budget)");
  const int32_t V = e->V;
  for (int j = 0; j < k; ++j)
    if (sources[j] < 0 || sources[j] >= V) return fail(GX_ERR_INVALID, "gx_ppr: source %d outside [0, %d)", sources[j], V);
  GX_CUDA(cudaSetDevice(e->dev));
  cudaStream_t s = e->s_comp;
  // Units: one per vertex, heavy vertices in chunks.
  std::vector<int4> units;
  units.reserve(static_cast<size_t>(V) + 1024);
  int32_t n_part = 0;
  for (int32_t v = 0; v < V; ++v) {
    const int64_t d = e->off[v + 1] - e->off[v];
    const int32_t nch = d > kPprChunk ? static_cast<int32_t>((d + kPprChunk - 1) / kPprChunk) : 1;
    for (int32_t c = 0; c < nch; ++c) units.push_back(make_int4(v, c, nch, nch > 1 ? n_part : 0));
    if (nch > 1) n_part += nch;
  }
  const size_t rows = static_cast<size_t>(V) * kPprCols;
  float *rs0 = nullptr, *rs1 = nullptr, *r = nullptr, *partial = nullptr;
  int4* d_units = nullptr;
  int32_t* d_src = nullptr;
  unsigned int *ctr = nullptr, *ticket = nullptr;
  struct Guard {
    std::vector<void*> p;
    ~Guard() {
      for (void* x : p) gx::pool_free(x);
    }
  } guard;
  gx_status st = GX_OK;
  if ((st = dev_alloc(&rs0, rows)) != GX_OK) return st;
  guard.p.push_back(rs0);
  if ((st = dev_alloc(&rs1, rows)) != GX_OK) return st;
  guard.p.push_back(rs1);
  if ((st = dev_alloc(&r, rows)) != GX_OK) return st;
  guard.p.push_back(r);
  if ((st = dev_alloc(&partial, static_cast<size_t>(std::max(n_part, 1)) * kPprCols)) != GX_OK) return st;
  guard.p.push_back(partial);
  if ((st = dev_alloc(&d_units, units.size())) != GX_OK) return st;
  guard.p.push_back(d_units);
  if ((st = dev_alloc(&d_src, kPprCols)) != GX_OK) return st;
  guard.p.push_back(d_src);
  if ((st = dev_alloc(&ctr, static_cast<size_t>(kQueues) * std::max(iters, 1))) != GX_OK) return st;
  guard.p.push_back(ctr);
  if ((st = dev_alloc(&ticket, static_cast<size_t>(std::max(n_part, 1)))) != GX_OK) return st;
  guard.p.push_back(ticket);

  PprArgs a{};
  int32_t h_src[kPprCols];
  for (int j = 0; j < kPprCols; ++j) h_src[j] = j < k ? sources[j] : -1;
  a.src = d_src;
  GX_CUDA(cudaMemcpyAsync(d_units, units.data(), sizeof(int4) * units.size(), cudaMemcpyHostToDevice, s));
  GX_CUDA(cudaMemcpy(d_src, h_src, sizeof(h_src), cudaMemcpyHostToDevice));
  GX_CUDA(cudaMemsetAsync(rs0, 0, rows * sizeof(float), s));
  GX_CUDA(cudaMemsetAsync(ctr, 0, sizeof(unsigned int) * kQueues * std::max(iters, 1), s));
  GX_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned int) * std::max(n_part, 1), s));
  ppr_init_kernel<<<1, kPprCols, 0, s>>>(rs0, e->d_outdeg, d_src, k);
  if (iters == 0) {
    // R0 = S.
    GX_CUDA(cudaMemsetAsync(r, 0, rows * sizeof(float), s));
  }
  a.off = e->d_off;
  a.col = e->d_col;
  a.outdeg = e->d_outdeg;
  a.units = d_units;
  a.n_units = static_cast<int32_t>(units.size());
  a.partial = partial;
  a.ticket = ticket;
  a.alpha = static_cast<float>(1.0 - restart);
  a.restart = static_cast<float>(restart);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ppr_kernel, kPprThreads, 0);
  const int grid = std::max(1, per_sm) * e->n_sm;
  cudaEvent_t ev0, ev1;
  GX_CUDA(cudaEventCreate(&ev0));
  GX_CUDA(cudaEventCreate(&ev1));
  GX_CUDA(cudaEventRecord(ev0, s));
  for (int it = 0; it < iters; ++it) {
    a.rs_in = it & 1 ? rs1 : rs0;
    a.rs_out = it & 1 ? rs0 : rs1;
    a.r_out = it + 1 == iters ? r : nullptr;
    a.ctr = ctr + static_cast<size_t>(kQueues) * it;
    ppr_kernel<<<grid, kPprThreads, 0, s>>>(a);
  }
  GX_CUDA(cudaGetLastError());
  GX_CUDA(cudaEventRecord(ev1, s));
  GX_CUDA(cudaEventSynchronize(ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (host_out) {
    if (iters == 0) {
      std::vector<float> h(rows, 0.f);
      for (int j = 0; j < k; ++j) h[static_cast<size_t>(sources[j]) * kPprCols + j] = 1.f;
      for (int32_t v = 0; v < V; ++v) memcpy(host_out + static_cast<size_t>(v) * k, &h[static_cast<size_t>(v) * kPprCols], sizeof(float) * k);
    } else {
      GX_CUDA(cudaMemcpy2D(host_out, sizeof(float) * k, r, sizeof(float) * kPprCols, sizeof(float) * k, V,
                           cudaMemcpyDeviceToHost));
    }
  }
  if (stats) {
    *stats = gx_run_stats{};
    stats->iterations = iters;
    stats->edges_scanned = e->E * static_cast<int64_t>(iters);
    stats->ms_total = ms;
    stats->ms_compute = ms;
    stats->kernel_launches = iters + 1;
    stats->pull_launches = iters;
    stats->ms_pull = ms;
  }
  return GX_OK;
}

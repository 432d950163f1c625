// Multi-source personalized PageRank as a sparse-times-dense product over
// the loaded CSC:  R <- restart*S + (1-restart) * A^T D^-1 R,  R0 = S,
// with R a V x k FP32 matrix (k <= 64 sources) and S the one-hot source
// matrix.  No reference counterpart; the per-edge arithmetic is PageRank's
// pull (GraphMP/app/pagerank.cpp:44-48) applied to k rank vectors at once.
//
// HBM layout: rows of W = k rounded up to 8 columns (32..256 bytes).
// Rs[2][V][W] holds R[u,:]/outdeg[u] (double buffer, so an edge costs one
// coalesced row gather of W floats); the final R is written on the last step
// only.
//
// All steps run in ONE persistent cooperative launch, captured in a CUDA
// graph: CTAs sweep a step's work units, meet at a grid barrier (bounded by
// config.wait_limit polls; a timeout raises an abort flag every CTA honours
// and the call returns GX_ERR_TIMEOUT), and go on to the next step.  A unit
// is one destination vertex, or a chunk of kPprChunk in-edges of a vertex
// with more; its row is summed by a group of W/2 lanes (a float2 each), so a
// warp works on 64/W units at once, from claims of kPprClaim units.  Chunked
// vertices fold their partial rows in chunk order in the warp group that
// finishes last, so results are deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "gx_engine.h"
#include "gx_nvtx.h"

using namespace gx;

namespace {

constexpr int kPprMaxCols = 64;
constexpr int kPprChunk = 1024;
constexpr int kPprThreads = 256;
constexpr int kPprWarps = kPprThreads / 32;

struct PprArgs {
  const int64_t* off;
  const int32_t* col;
  const int32_t* outdeg;
  float* rs[2];             // R[u,:]/outdeg[u], double buffer [V][W]
  float* r_out;             // final R [V][W]
  const int4* units;        // (v, chunk, n_chunks, partial base)
  int32_t n_units;
  int32_t iters;
  unsigned int* ctr;        // kQueues work cursors per step
  unsigned int* arrive;     // grid-barrier arrival count per step
  unsigned int* abort;      // set when a grid barrier gives up
  unsigned int wait_limit;  // polls (of at least 64 ns) before it does
  float* partial;           // [n_partial][W]
  unsigned int* ticket;     // per chunked vertex, indexed by partial base
  const int32_t* src;       // [W] source vertex of each column (-1 past k)
  float alpha, restart;
};

// All CTAs of the (co-resident) grid meet after step `it`.  Returns false
// when the wait timed out or another CTA gave up.
__device__ bool ppr_grid_barrier(const PprArgs& a, int it) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(a.arrive + it, 1u);
    int ok = 1;
    volatile unsigned* c = a.arrive + it;
    volatile unsigned* ab = a.abort;
    for (unsigned i = 0; *c < gridDim.x; ++i) {
      if (*ab || i >= a.wait_limit) {
        atomicExch(a.abort, 1u);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_ok = ok && !*ab;
  }
  __syncthreads();
  return s_ok != 0;
}

template <int W>
__device__ __forceinline__ void ppr_finish(const PprArgs& a, float* rs_out, float* r_out, int v, float2 acc,
                                           int gl) {
  float2 r = make_float2(a.alpha * acc.x, a.alpha * acc.y);
  if (a.src[2 * gl] == v) r.x += a.restart;
  if (a.src[2 * gl + 1] == v) r.y += a.restart;
  const int32_t od = a.outdeg[v];
  const float inv = 1.0f / static_cast<float>(od > 0 ? od : 1);
  const size_t row = static_cast<size_t>(v) * W + 2 * gl;
  if (r_out) *reinterpret_cast<float2*>(r_out + row) = r;
  *reinterpret_cast<float2*>(rs_out + row) = make_float2(r.x * inv, r.y * inv);
}

// Units a warp claims per cursor atomic: most vertices of an R-MAT graph
// have no in-edges, so a claim per unit would cost a round trip per empty row.
constexpr int kPprClaim = 16;

template <int W>
__global__ void __launch_bounds__(kPprThreads) ppr_kernel(const PprArgs a) {
  constexpr int L = W / 2;   // lanes per row, a float2 each
  constexpr int G = 32 / L;  // units a warp works on at once
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int gl = lane % L, grp = lane / L;
  const unsigned gmask = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << (grp * L));
  const int U = a.n_units;
  const int nq = U / 256 < 1 ? 1 : (U / 256 < kQueues ? U / 256 : kQueues);
  for (int it = 0; it < a.iters; ++it) {
    const float* rs_in = (it & 1) ? a.rs[1] : a.rs[0];
    float* rs_out = (it & 1) ? a.rs[0] : a.rs[1];
    float* r_out = it + 1 == a.iters ? a.r_out : nullptr;
    unsigned int* ctr = a.ctr + static_cast<size_t>(kQueues) * it;
    int q = (blockIdx.x * kPprWarps + wid) % nq;
    for (;;) {
      const int qb = static_cast<int>((static_cast<int64_t>(U) * q) / nq);
      const int qe = static_cast<int>((static_cast<int64_t>(U) * (q + 1)) / nq);
      int u0 = 0;
      if (lane == 0) u0 = qb + static_cast<int>(atomicAdd(ctr + q, static_cast<unsigned>(kPprClaim)));
      u0 = __shfl_sync(0xffffffffu, u0, 0);
      if (u0 >= qe) {
        q = next_queue(ctr, q, nq, U, lane);
        if (q < 0) break;
        continue;
      }
      // Group grp takes units u0 + grp, u0 + grp + G, ... of the claim.
      for (int u = u0 + grp; u < u0 + kPprClaim && u < qe; u += G) {
        const int4 un = a.units[u];
        const int v = un.x;
        const int64_t vb = a.off[v], ve = a.off[v + 1];
        const int64_t b = vb + static_cast<int64_t>(un.y) * kPprChunk;
        const int64_t e = ve < b + kPprChunk ? ve : b + kPprChunk;
        float2 acc = make_float2(0.f, 0.f);
        for (int64_t k0 = b; k0 < e; k0 += L) {
          const int n = e - k0 < L ? static_cast<int>(e - k0) : L;
          const int32_t mine = gl < n ? __ldcs(a.col + k0 + gl) : 0;
          int j = 0;
          for (; j + 8 <= n; j += 8) {
            float2 x[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
              const int32_t s = __shfl_sync(gmask, mine, j + t, L);
              x[t] = __ldg(reinterpret_cast<const float2*>(rs_in + static_cast<size_t>(s) * W) + gl);
            }
#pragma unroll
            for (int t = 0; t < 8; ++t) {
              acc.x += x[t].x;
              acc.y += x[t].y;
            }
          }
          for (; j < n; ++j) {
            const int32_t s = __shfl_sync(gmask, mine, j, L);
            const float2 x = __ldg(reinterpret_cast<const float2*>(rs_in + static_cast<size_t>(s) * W) + gl);
            acc.x += x.x;
            acc.y += x.y;
          }
        }
        if (un.z == 1) {
          ppr_finish<W>(a, rs_out, r_out, v, acc, gl);
        } else {
          float2* part = reinterpret_cast<float2*>(a.partial + static_cast<size_t>(un.w + un.y) * W);
          part[gl] = acc;
          __threadfence();
          __syncwarp(gmask);
          unsigned t = 0;
          if (gl == 0) t = atomicAdd(a.ticket + un.w, 1u);
          t = __shfl_sync(gmask, t, 0, L);
          if (t == static_cast<unsigned>(un.z) - 1) {
            __threadfence();
            float2 tot = make_float2(0.f, 0.f);
            for (int c = 0; c < un.z; ++c) {
              const volatile float* pp = a.partial + static_cast<size_t>(un.w + c) * W + 2 * gl;
              tot.x += pp[0];
              tot.y += pp[1];
            }
            ppr_finish<W>(a, rs_out, r_out, v, tot, gl);
            if (gl == 0) a.ticket[un.w] = 0;
          }
        }
      }
      __syncwarp();
    }
    if (!ppr_grid_barrier(a, it)) return;
  }
}

__global__ void ppr_init_kernel(float* rs, const int32_t* outdeg, const int32_t* src, int k, int W) {
  const int j = threadIdx.x;
  if (j < k) {
    const int v = src[j];
    const int32_t od = outdeg[v];
    rs[static_cast<size_t>(v) * W + j] = 1.0f / static_cast<float>(od > 0 ? od : 1);
  }
}

template <int W>
const void* ppr_kernel_for() {
  return reinterpret_cast<const void*>(ppr_kernel<W>);
}

}  // namespace

extern "C" gx_status gx_ppr(gx_engine* e, int32_t k, const int32_t* sources, int32_t iters, double restart,
                            float* host_out, gx_run_stats* stats) {
  gx::NvtxRange nvtx_range("gx_ppr");
  if (!e || !sources || k < 1 || k > kPprMaxCols || iters < 0 || restart < 0 || restart > 1)
    return fail(GX_ERR_INVALID, "gx_ppr: bad arguments (k must be 1..64)");
  if (!e->loaded) return fail(GX_ERR_STATE, "gx_ppr: no graph loaded");
  if (!e->all_resident) return fail(GX_ERR_STATE, "gx_ppr: needs every shard resident (no shard-cache budget)");
  const int32_t V = e->V;
  for (int j = 0; j < k; ++j)
    if (sources[j] < 0 || sources[j] >= V) return fail(GX_ERR_INVALID, "gx_ppr: source %d outside [0, %d)", sources[j], V);
  GX_CUDA(cudaSetDevice(e->dev));
  cudaStream_t s = e->s_comp;
  const int W = k <= 8 ? 8 : k <= 16 ? 16 : k <= 32 ? 32 : 64;
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
  const size_t rows = static_cast<size_t>(V) * W;
  const size_t steps = static_cast<size_t>(std::max(iters, 1));
  float *rs0 = nullptr, *rs1 = nullptr, *r = nullptr, *partial = nullptr;
  int4* d_units = nullptr;
  int32_t* d_src = nullptr;
  unsigned int *ctr = nullptr, *ticket = nullptr, *arrive = nullptr, *abort_flag = nullptr;
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
  if ((st = dev_alloc(&partial, static_cast<size_t>(std::max(n_part, 1)) * W)) != GX_OK) return st;
  guard.p.push_back(partial);
  if ((st = dev_alloc(&d_units, units.size())) != GX_OK) return st;
  guard.p.push_back(d_units);
  if ((st = dev_alloc(&d_src, kPprMaxCols)) != GX_OK) return st;
  guard.p.push_back(d_src);
  if ((st = dev_alloc(&ctr, static_cast<size_t>(kQueues) * steps)) != GX_OK) return st;
  guard.p.push_back(ctr);
  if ((st = dev_alloc(&ticket, static_cast<size_t>(std::max(n_part, 1)))) != GX_OK) return st;
  guard.p.push_back(ticket);
  if ((st = dev_alloc(&arrive, steps)) != GX_OK) return st;
  guard.p.push_back(arrive);
  if ((st = dev_alloc(&abort_flag, 1)) != GX_OK) return st;
  guard.p.push_back(abort_flag);

  int32_t h_src[kPprMaxCols];
  for (int j = 0; j < kPprMaxCols; ++j) h_src[j] = j < k ? (e->relabeled ? e->h_perm[sources[j]] : sources[j]) : -1;
  GX_CUDA(cudaMemcpyAsync(d_units, units.data(), sizeof(int4) * units.size(), cudaMemcpyHostToDevice, s));
  GX_CUDA(cudaMemcpyAsync(d_src, h_src, sizeof(h_src), cudaMemcpyHostToDevice, s));
  GX_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned int) * std::max(n_part, 1), s));

  PprArgs a{};
  a.off = e->d_off;
  a.col = e->d_col;
  a.outdeg = e->d_outdeg;
  a.rs[0] = rs0;
  a.rs[1] = rs1;
  a.r_out = r;
  a.units = d_units;
  a.n_units = static_cast<int32_t>(units.size());
  a.iters = iters;
  a.ctr = ctr;
  a.arrive = arrive;
  a.abort = abort_flag;
  a.wait_limit = e->cfg.wait_limit;
  a.partial = partial;
  a.ticket = ticket;
  a.src = d_src;
  a.alpha = static_cast<float>(1.0 - restart);
  a.restart = static_cast<float>(restart);
  const void* fn = W == 8 ? ppr_kernel_for<8>() : W == 16 ? ppr_kernel_for<16>() : W == 32 ? ppr_kernel_for<32>()
                                                                                           : ppr_kernel_for<64>();
  int per_sm = 0;
  GX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kPprThreads, 0));
  // Co-resident CTAs only: the grid barrier waits for every one of them.
  const int grid = std::max(1, per_sm) * e->n_sm;
  cudaLaunchConfig_t lc{};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  lc.gridDim = dim3(grid);
  lc.blockDim = dim3(kPprThreads);
  lc.dynamicSmemBytes = 0;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  void* kargs[] = {&a};
  // The step's resets, R0 = S and the persistent launch, as one graph.
  auto enqueue = [&]() -> cudaError_t {
    cudaError_t err = cudaMemsetAsync(rs0, 0, rows * sizeof(float), s);
    if (err == cudaSuccess) err = cudaMemsetAsync(ctr, 0, sizeof(unsigned int) * kQueues * steps, s);
    if (err == cudaSuccess) err = cudaMemsetAsync(arrive, 0, sizeof(unsigned int) * steps, s);
    if (err == cudaSuccess) err = cudaMemsetAsync(abort_flag, 0, sizeof(unsigned int), s);
    if (err != cudaSuccess) return err;
    ppr_init_kernel<<<1, kPprMaxCols, 0, s>>>(rs0, e->d_outdeg, d_src, k, W);
    err = cudaGetLastError();
    if (err == cudaSuccess && iters > 0) err = cudaLaunchKernelExC(&lc, fn, kargs);
    return err;
  };
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  GX_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaError_t cap_err = enqueue();
  cudaError_t end_err = cudaStreamEndCapture(s, &graph);
  if (cap_err != cudaSuccess || end_err != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return fail(GX_ERR_CUDA, "gx_ppr: capture: %s", cudaGetErrorString(cap_err != cudaSuccess ? cap_err : end_err));
  }
  cudaError_t err = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (err != cudaSuccess) return fail(GX_ERR_CUDA, "gx_ppr: graph instantiate: %s", cudaGetErrorString(err));
  cudaEvent_t ev0, ev1;
  GX_CUDA(cudaEventCreate(&ev0));
  GX_CUDA(cudaEventCreate(&ev1));
  GX_CUDA(cudaEventRecord(ev0, s));
  err = cudaGraphLaunch(exec, s);
  if (err == cudaSuccess) err = cudaEventRecord(ev1, s);
  if (err == cudaSuccess) err = cudaEventSynchronize(ev1);
  float ms = 0;
  if (err == cudaSuccess) cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  cudaGraphExecDestroy(exec);
  if (err != cudaSuccess) return fail(GX_ERR_CUDA, "gx_ppr: run failed: %s", cudaGetErrorString(err));
  unsigned int aborted = 0;
  GX_CUDA(cudaMemcpy(&aborted, abort_flag, sizeof(aborted), cudaMemcpyDeviceToHost));
  if (aborted) return fail(GX_ERR_TIMEOUT, "gx_ppr: a grid barrier timed out");
  if (host_out) {
    if (iters == 0) {
      memset(host_out, 0, sizeof(float) * static_cast<size_t>(V) * k);
      for (int j = 0; j < k; ++j) host_out[static_cast<size_t>(sources[j]) * k + j] = 1.f;
    } else if (!e->relabeled) {
      GX_CUDA(cudaMemcpy2D(host_out, sizeof(float) * k, r, sizeof(float) * W, sizeof(float) * k, V,
                           cudaMemcpyDeviceToHost));
    } else {
      // Rows in the engine's numbering: row v of the result is row perm[v].
      std::vector<float> rows(static_cast<size_t>(V) * k);
      GX_CUDA(cudaMemcpy2D(rows.data(), sizeof(float) * k, r, sizeof(float) * W, sizeof(float) * k, V,
                           cudaMemcpyDeviceToHost));
      const int32_t* perm = e->h_perm.data();
#pragma omp parallel for schedule(static)
      for (int32_t v = 0; v < V; ++v)
        memcpy(host_out + static_cast<size_t>(v) * k, rows.data() + static_cast<size_t>(perm[v]) * k,
               sizeof(float) * k);
    }
  }
  if (stats) {
    *stats = gx_run_stats{};
    stats->iterations = iters;
    stats->edges_scanned = e->E * static_cast<int64_t>(iters);
    stats->ms_total = ms;
    stats->ms_compute = ms;
    stats->kernel_launches = iters > 0 ? 2 : 1;
    stats->pull_launches = iters > 0 ? 1 : 0;
    stats->ms_pull = ms;
  }
  return GX_OK;
}

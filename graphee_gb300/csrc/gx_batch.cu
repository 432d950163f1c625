// Batched independent instances in one persistent launch.
//
// The loaded CSC holds many graphs side by side (instance i owns vertices
// [vbeg[i], vbeg[i+1]) and only edges among them).  One persistent kernel,
// replayed as a CUDA graph, runs for every instance the reference's
// PageRank (comp_pagerank<float>, GraphMP/app/pagerank.cpp:20-84, with
// N = the instance's vertex count) for up to pr_iters supersteps and then
// its min-label CC (comp_cc, GraphMP/app/cc.cpp:20-75) to convergence, each
// with GraphPS::run's stop rule per instance (GraphMP/system/GraphPS.h:383).
// A CTA owns an instance at a time, so a superstep's barrier is a CTA
// barrier; CTAs claim instances longest first.  Inside a CTA, warps sweep
// 32-vertex tiles: lanes walk lists of up to `lane_max` edges alone (edge
// order), longer lists are swept by the whole warp.
// Threads per CTA, lane_max and CTAs per SM come from the autotuner
// (gx_batch_autotune), which times candidate schedules on the batch and
// records the winner in a table file.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <numeric>
#include <string>
#include <vector>

#include "gx_engine.h"

using namespace gx;

namespace {

struct BatchArgs {
  const int64_t* off;
  const int32_t* col;
  const int32_t* outdeg;
  const int32_t* vbeg;      // n_inst + 1
  const int32_t* order;     // claim order (longest first)
  int32_t n_inst;
  unsigned int* ctr;
  float *pr0, *pr1;
  float *con0, *con1;
  int32_t *lab0, *lab1;
  float* pr_out;
  int32_t* cc_out;
  int32_t* pr_steps;        // per instance
  int32_t* cc_steps;
  int32_t pr_iters, cc_max;
  int32_t lane_max;
  double damping;
};

// Gathers a vertex's in-edge values: PR contributions (sum) or labels (min).
// Lanes walk lists of up to lane_max edges alone, 8 edges per step from two
// 128-bit index loads (edge order kept: positions outside the list are
// masked), so each lane has 8 gathers in flight; longer lists are swept by the
// whole warp, 4 consecutive edges per lane per round.
template <bool PR>
__device__ __forceinline__ void batch_vertex_lists(const BatchArgs& a, const float* con, const int32_t* lab,
                                                   int64_t beg, int64_t end, bool valid, float& facc, int32_t& iacc,
                                                   int lane) {
  const bool longl = valid && end - beg > a.lane_max;
  if (valid && !longl && end > beg) {
    for (int64_t k = beg & ~3ll; k < end; k += 8) {
      const int4 c0 = __ldg(reinterpret_cast<const int4*>(a.col + k));
      int4 c1 = make_int4(0, 0, 0, 0);
      if (k + 4 < end) c1 = __ldg(reinterpret_cast<const int4*>(a.col + k + 4));
      const int32_t cs[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
      float fv[8];
      int32_t iv[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const bool in = k + j >= beg && k + j < end;
        if (PR) fv[j] = in ? __ldg(con + cs[j]) : 0.f;
        else iv[j] = in ? __ldg(lab + cs[j]) : 0x7fffffff;
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (PR) {
          if (k + j >= beg && k + j < end) facc += fv[j];
        } else {
          iacc = min(iacc, iv[j]);
        }
      }
    }
  }
  for (unsigned m = __ballot_sync(0xffffffffu, longl); m; m &= m - 1) {
    const int l = __ffs(m) - 1;
    const int64_t bl = __shfl_sync(0xffffffffu, beg, l), el = __shfl_sync(0xffffffffu, end, l);
    float fs = 0.f;
    int32_t is = 0x7fffffff;
    for (int64_t q = (bl & ~3ll) + 4 * lane; q < el; q += 128) {
      const int4 c = __ldg(reinterpret_cast<const int4*>(a.col + q));
      const int32_t cs[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (q + j >= bl && q + j < el) {
          if (PR) fs += __ldg(con + cs[j]);
          else is = min(is, __ldg(lab + cs[j]));
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      if (PR) fs += __shfl_xor_sync(0xffffffffu, fs, o);
      else is = min(is, __shfl_xor_sync(0xffffffffu, is, o));
    }
    if (lane == l) {
      if (PR) facc += fs;
      else iacc = min(iacc, is);
    }
  }
}

__global__ void batch_kernel(BatchArgs a) {
  __shared__ int s_inst;
  __shared__ unsigned int s_changed;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) s_inst = static_cast<int>(atomicAdd(a.ctr, 1u));
    __syncthreads();
    const int slot = s_inst;
    __syncthreads();
    if (slot >= a.n_inst) break;
    const int inst = a.order[slot];
    const int32_t vb = a.vbeg[inst], ve = a.vbeg[inst + 1], n = ve - vb;
    const int tiles = (n + 31) / 32;
    const double inv_n = 1.0 / n;
    // ---- PageRank ----
    for (int v = vb + threadIdx.x; v < ve; v += blockDim.x) {
      const float r0 = static_cast<float>(inv_n);
      const int32_t od = a.outdeg[v];
      a.pr0[v] = r0;
      a.con0[v] = r0 / static_cast<float>(od > 0 ? od : 1);
    }
    __syncthreads();
    int cur = 0, step = 0;
    for (step = 0; step < a.pr_iters; ++step) {
      if (threadIdx.x == 0) s_changed = 0;
      __syncthreads();
      // Ternaries, not a[cur]: runtime indexing of a parameter array would
      // copy the parameter block to local memory.
      const float* con = cur ? a.con1 : a.con0;
      const float* src = cur ? a.pr1 : a.pr0;
      float* dst = cur ? a.pr0 : a.pr1;
      float* dcon = cur ? a.con0 : a.con1;
      unsigned changed = 0;
      for (int t = wid; t < tiles; t += nw) {
        const int v = vb + 32 * t + lane;
        const bool valid = v < ve;
        int64_t beg = 0, end = 0;
        if (valid) {
          beg = a.off[v];
          end = a.off[v + 1];
        }
        float acc = 0.f;
        int32_t dummy = 0;
        batch_vertex_lists<true>(a, con, nullptr, beg, end, valid, acc, dummy, lane);
        if (valid) {
          const float nv = static_cast<float>(__dadd_rn(__dmul_rn(static_cast<double>(acc), a.damping), inv_n));
          const float old = src[v];
          changed += nv != (step == 0 ? 0.f : old);
          dst[v] = nv;
          const int32_t od = a.outdeg[v];
          dcon[v] = nv / static_cast<float>(od > 0 ? od : 1);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) changed += __shfl_xor_sync(0xffffffffu, changed, o);
      if (lane == 0 && changed) atomicAdd(&s_changed, changed);
      __syncthreads();
      cur ^= 1;
      const unsigned ch = s_changed;
      __syncthreads();
      if (ch == 0 && step > 1) {
        ++step;
        break;
      }
    }
    for (int v = vb + threadIdx.x; v < ve; v += blockDim.x) a.pr_out[v] = (cur ? a.pr1 : a.pr0)[v];
    if (threadIdx.x == 0) a.pr_steps[inst] = step < a.pr_iters ? step : a.pr_iters;
    // ---- CC ----
    for (int v = vb + threadIdx.x; v < ve; v += blockDim.x) a.lab0[v] = v - vb;
    __syncthreads();
    cur = 0;
    for (step = 0; step < a.cc_max; ++step) {
      if (threadIdx.x == 0) s_changed = 0;
      __syncthreads();
      const int32_t* src = cur ? a.lab1 : a.lab0;
      int32_t* dst = cur ? a.lab0 : a.lab1;
      unsigned changed = 0;
      for (int t = wid; t < tiles; t += nw) {
        const int v = vb + 32 * t + lane;
        const bool valid = v < ve;
        int64_t beg = 0, end = 0;
        int32_t old = 0;
        if (valid) {
          beg = a.off[v];
          end = a.off[v + 1];
          old = src[v];
        }
        float dummy = 0.f;
        int32_t acc = old;
        batch_vertex_lists<false>(a, nullptr, src, beg, end, valid, dummy, acc, lane);
        if (valid) {
          changed += acc != (step == 0 ? 0 : old);
          dst[v] = acc;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) changed += __shfl_xor_sync(0xffffffffu, changed, o);
      if (lane == 0 && changed) atomicAdd(&s_changed, changed);
      __syncthreads();
      cur ^= 1;
      const unsigned ch = s_changed;
      __syncthreads();
      if (ch == 0 && step > 1) {
        ++step;
        break;
      }
    }
    for (int v = vb + threadIdx.x; v < ve; v += blockDim.x) a.cc_out[v] = (cur ? a.lab1 : a.lab0)[v];
    if (threadIdx.x == 0) a.cc_steps[inst] = step < a.cc_max ? step : a.cc_max;
    __syncthreads();
  }
}

__global__ void batch_check_kernel(const int64_t* off, const int32_t* col, const int32_t* vbeg, int32_t n,
                                   int32_t V, unsigned int* bad) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    int lo = 0, hi = n;  // instance of v: vbeg[lo] <= v < vbeg[lo + 1]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (vbeg[mid] <= v) lo = mid;
      else hi = mid;
    }
    const int32_t b = vbeg[lo], e = vbeg[lo + 1];
    unsigned c = 0;
    for (int64_t k = off[v]; k < off[v + 1]; ++k) c += (col[k] < b || col[k] >= e);
    if (c) atomicAdd(bad, c);
  }
}

struct BatchDev {
  int32_t *vbeg = nullptr, *order = nullptr, *lab0 = nullptr, *lab1 = nullptr, *cc_out = nullptr;
  int32_t *pr_steps = nullptr, *cc_steps = nullptr;
  float *pr0 = nullptr, *pr1 = nullptr, *con0 = nullptr, *con1 = nullptr, *pr_out = nullptr;
  unsigned int* ctr = nullptr;
  ~BatchDev() {
    dev_free(&vbeg);
    dev_free(&order);
    dev_free(&lab0);
    dev_free(&lab1);
    dev_free(&cc_out);
    dev_free(&pr_steps);
    dev_free(&cc_steps);
    dev_free(&pr0);
    dev_free(&pr1);
    dev_free(&con0);
    dev_free(&con1);
    dev_free(&pr_out);
    dev_free(&ctr);
  }
};

gx_status batch_prepare(gx_engine* e, int32_t n, const int32_t* vbeg, BatchDev& d, BatchArgs& a) {
  const int32_t V = e->V;
  if (vbeg[0] != 0 || vbeg[n] != V) return fail(GX_ERR_INVALID, "gx_batch: instance ranges must cover [0, V)");
  for (int32_t i = 0; i < n; ++i)
    if (vbeg[i + 1] <= vbeg[i]) return fail(GX_ERR_INVALID, "gx_batch: instance %d is empty or out of order", i);
  std::vector<int32_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
    return e->off[vbeg[x + 1]] - e->off[vbeg[x]] > e->off[vbeg[y + 1]] - e->off[vbeg[y]];
  });
  GX_TRY(dev_alloc(&d.vbeg, static_cast<size_t>(n) + 1));
  GX_TRY(dev_alloc(&d.order, static_cast<size_t>(n)));
  GX_TRY(dev_alloc(&d.lab0, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&d.lab1, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&d.cc_out, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&d.pr0, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&d.pr1, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&d.con0, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&d.con1, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&d.pr_out, static_cast<size_t>(V)));
  GX_TRY(dev_alloc(&d.pr_steps, static_cast<size_t>(n)));
  GX_TRY(dev_alloc(&d.cc_steps, static_cast<size_t>(n)));
  GX_TRY(dev_alloc(&d.ctr, 1));
  GX_CUDA(cudaMemcpy(d.vbeg, vbeg, sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice));
  GX_CUDA(cudaMemcpy(d.order, order.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
  // Every edge must stay inside its instance (a block-diagonal CSC).
  GX_CUDA(cudaMemset(d.ctr, 0, sizeof(unsigned int)));
  batch_check_kernel<<<e->n_sm * 8, 256, 0, e->s_comp>>>(e->d_off, e->d_col, d.vbeg, n, V, d.ctr);
  unsigned int bad = 0;
  GX_CUDA(cudaMemcpyAsync(&bad, d.ctr, sizeof(bad), cudaMemcpyDeviceToHost, e->s_comp));
  GX_CUDA(cudaStreamSynchronize(e->s_comp));
  if (bad) return fail(GX_ERR_INVALID, "gx_batch: %u edges cross instance boundaries", bad);
  a = BatchArgs{};
  a.off = e->d_off;
  a.col = e->d_col;
  a.outdeg = e->d_outdeg;
  a.vbeg = d.vbeg;
  a.order = d.order;
  a.n_inst = n;
  a.ctr = d.ctr;
  a.pr0 = d.pr0;
  a.pr1 = d.pr1;
  a.con0 = d.con0;
  a.con1 = d.con1;
  a.lab0 = d.lab0;
  a.lab1 = d.lab1;
  a.pr_out = d.pr_out;
  a.cc_out = d.cc_out;
  a.pr_steps = d.pr_steps;
  a.cc_steps = d.cc_steps;
  return GX_OK;
}

// One persistent launch (plus its cursor reset), captured as a CUDA graph.
gx_status batch_launch(gx_engine* e, const BatchArgs& a, const gx_batch_tuning& t, float* ms) {
  cudaStream_t s = e->s_comp;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel, t.threads, 0);
  const int blocks = std::max(1, std::min(per_sm, t.ctas_per_sm)) * e->n_sm;
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  GX_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(a.ctr, 0, sizeof(unsigned int), s);
  batch_kernel<<<blocks, t.threads, 0, s>>>(a);
  GX_CUDA(cudaStreamEndCapture(s, &graph));
  cudaError_t err = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (err != cudaSuccess) return fail(GX_ERR_CUDA, "gx_batch: graph instantiate: %s", cudaGetErrorString(err));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  cudaGraphLaunch(exec, s);
  cudaEventRecord(e1, s);
  err = cudaEventSynchronize(e1);
  float t_ms = 0;
  cudaEventElapsedTime(&t_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGraphExecDestroy(exec);
  if (err != cudaSuccess) return fail(GX_ERR_CUDA, "gx_batch: run failed: %s", cudaGetErrorString(err));
  *ms = t_ms;
  return GX_OK;
}

gx_status check_tuning(const gx_batch_tuning& t) {
  if (t.threads < 64 || t.threads > 1024 || t.threads % 32 || t.lane_max < 0 || t.ctas_per_sm < 1)
    return fail(GX_ERR_INVALID, "gx_batch: bad tuning (threads %d, lane_max %d, ctas_per_sm %d)", t.threads,
                t.lane_max, t.ctas_per_sm);
  return GX_OK;
}

}  // namespace

extern "C" {

void gx_batch_tuning_default(gx_batch_tuning* t) {
  if (!t) return;
  t->threads = 512;
  t->lane_max = 32;
  t->ctas_per_sm = 2;
}

gx_status gx_batch_run(gx_engine* e, int32_t n_inst, const int32_t* inst_vbegin, int32_t pr_iters, int32_t cc_max_iter,
                       double damping, const gx_batch_tuning* tuning, float* pr_out, int32_t* cc_out,
                       int32_t* pr_steps, int32_t* cc_steps, gx_run_stats* stats) {
  if (!e || n_inst < 1 || !inst_vbegin || pr_iters < 0 || cc_max_iter < 0)
    return fail(GX_ERR_INVALID, "gx_batch_run: bad arguments");
  if (!e->loaded || !e->all_resident) return fail(GX_ERR_STATE, "gx_batch_run: load the packed graph first (all resident)");
  gx_batch_tuning t;
  gx_batch_tuning_default(&t);
  if (tuning) t = *tuning;
  GX_TRY(check_tuning(t));
  GX_CUDA(cudaSetDevice(e->dev));
  BatchDev d;
  BatchArgs a;
  GX_TRY(batch_prepare(e, n_inst, inst_vbegin, d, a));
  a.pr_iters = pr_iters;
  a.cc_max = cc_max_iter;
  a.lane_max = t.lane_max;
  a.damping = damping;
  float ms = 0;
  GX_TRY(batch_launch(e, a, t, &ms));
  const int32_t V = e->V;
  if (pr_out) GX_CUDA(cudaMemcpy(pr_out, d.pr_out, sizeof(float) * V, cudaMemcpyDeviceToHost));
  if (cc_out) GX_CUDA(cudaMemcpy(cc_out, d.cc_out, sizeof(int32_t) * V, cudaMemcpyDeviceToHost));
  std::vector<int32_t> ps(n_inst), cs(n_inst);
  GX_CUDA(cudaMemcpy(ps.data(), d.pr_steps, sizeof(int32_t) * n_inst, cudaMemcpyDeviceToHost));
  GX_CUDA(cudaMemcpy(cs.data(), d.cc_steps, sizeof(int32_t) * n_inst, cudaMemcpyDeviceToHost));
  if (pr_steps) memcpy(pr_steps, ps.data(), sizeof(int32_t) * n_inst);
  if (cc_steps) memcpy(cc_steps, cs.data(), sizeof(int32_t) * n_inst);
  if (stats) {
    *stats = gx_run_stats{};
    int64_t edges = 0;
    for (int32_t i = 0; i < n_inst; ++i)
      edges += (e->off[inst_vbegin[i + 1]] - e->off[inst_vbegin[i]]) * static_cast<int64_t>(ps[i] + cs[i]);
    stats->iterations = *std::max_element(ps.begin(), ps.end()) + *std::max_element(cs.begin(), cs.end());
    stats->edges_scanned = edges;
    stats->ms_total = ms;
    stats->ms_compute = ms;
    stats->kernel_launches = 1;
  }
  return GX_OK;
}

gx_status gx_batch_autotune(gx_engine* e, int32_t n_inst, const int32_t* inst_vbegin, int32_t pr_iters,
                            int32_t cc_max_iter, const char* table_path, gx_batch_tuning* best, double* best_ms) {
  if (!e || !best || n_inst < 1 || !inst_vbegin) return fail(GX_ERR_INVALID, "gx_batch_autotune: bad arguments");
  if (!e->loaded || !e->all_resident) return fail(GX_ERR_STATE, "gx_batch_autotune: load the packed graph first");
  GX_CUDA(cudaSetDevice(e->dev));
  BatchDev d;
  BatchArgs a;
  GX_TRY(batch_prepare(e, n_inst, inst_vbegin, d, a));
  a.pr_iters = pr_iters;
  a.cc_max = cc_max_iter;
  a.damping = 0.85;
  const int threads_c[] = {256, 512, 1024};
  const int lane_c[] = {16, 32, 64};
  const int cps_c[] = {1, 2, 4};
  float best_t = 0;
  bool have = false;
  std::string log;
  for (int th : threads_c)
    for (int lm : lane_c)
      for (int cp : cps_c) {
        if (th * cp > 2048) continue;
        gx_batch_tuning t{th, lm, cp};
        a.lane_max = lm;
        float ms = 0, ms2 = 0;
        GX_TRY(batch_launch(e, a, t, &ms));   // warm
        GX_TRY(batch_launch(e, a, t, &ms2));
        ms = std::min(ms, ms2);
        char buf[160];
        snprintf(buf, sizeof(buf), "{\"threads\": %d, \"lane_max\": %d, \"ctas_per_sm\": %d, \"ms\": %.4f}", th, lm, cp,
                 ms);
        log += std::string(log.empty() ? "" : ", ") + buf;
        if (!have || ms < best_t) {
          best_t = ms;
          *best = t;
          have = true;
        }
      }
  if (best_ms) *best_ms = best_t;
  if (table_path && *table_path) {
    FILE* f = fopen(table_path, "a");
    if (!f) return fail(GX_ERR_IO, "gx_batch_autotune: cannot append to %s", table_path);
    fprintf(f,
            "{\"instances\": %d, \"vertices\": %d, \"edges\": %lld, \"pr_iters\": %d, \"best\": {\"threads\": %d, "
            "\"lane_max\": %d, \"ctas_per_sm\": %d, \"ms\": %.4f}, \"candidates\": [%s]}\n",
            n_inst, e->V, static_cast<long long>(e->E), pr_iters, best->threads, best->lane_max, best->ctas_per_sm,
            best_t, log.c_str());
    fclose(f);
  }
  return GX_OK;
}

}  // extern "C"

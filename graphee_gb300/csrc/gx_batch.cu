// Batched independent instances in one persistent launch.
//
// The loaded CSC holds many graphs side by side (instance i owns vertices
// [vbeg[i], vbeg[i+1]) and only edges among them).  One persistent kernel,
// replayed as a CUDA graph, runs for every instance the reference's
// PageRank (comp_pagerank<float>, GraphMP/app/pagerank.cpp:20-84, with
// N = the instance's vertex count) for up to pr_iters supersteps and then
// its min-label CC (comp_cc, GraphMP/app/cc.cpp:20-75) to convergence, each
// with GraphPS::run's stop rule per instance (GraphMP/system/GraphPS.h:383).
// CTAs claim work slots longest instance first.  A small instance is one slot
// and its superstep barrier a CTA barrier; an instance larger than about half
// a CTA's fair share of the batch is split over a team of CTAs (one slot per
// member, claimed consecutively), whose members sweep interleaved tiles and
// meet at a global barrier after every superstep: an arrival counter and
// triple-buffered change counts per instance, polled with a bounded spin (a
// timeout raises an abort flag that every CTA honours, and the host reports
// GX_ERR_TIMEOUT).  The launch holds no more CTAs than fit on the GPU at
// once, so every member of a claimed team is running.  Inside a CTA, warps
// sweep 32-vertex tiles: lanes walk lists of up to `lane_max` edges alone
// (edge order), longer lists are swept by the whole warp.
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
#include "gx_nvtx.h"

using namespace gx;

namespace {

struct BatchArgs {
  const int64_t* off;
  const int32_t* col;
  const int32_t* outdeg;
  const int32_t* vbeg;      // n_inst + 1
  const int2* slots;        // claim order: (instance, member << 16 | team size), longest first
  int32_t n_slots;
  int32_t n_inst;
  unsigned int* ctr;
  unsigned int* team;       // per instance: arrivals, change counts [3]
  unsigned int* abort;      // set when a team barrier times out
  unsigned int spin_limit;
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

// Barrier b of a team of `team` CTAs on instance state t[0..3]: adds this
// CTA's change count to t[1 + b % 3] (member 0 first clears the slot barrier
// b + 1 will use) and returns the team's total.  Every thread of the CTA
// calls it.  Returns false when the wait timed out or another team aborted.
__device__ bool team_barrier(const BatchArgs& a, unsigned int* t, int team, int member, int b, unsigned changed,
                             unsigned* total) {
  __shared__ unsigned s_tot;
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    if (member == 0) atomicExch(t + 1 + (b + 1) % 3, 0u);
    if (changed) atomicAdd(t + 1 + b % 3, changed);
    __threadfence();
    atomicAdd(t, 1u);
    const unsigned target = static_cast<unsigned>(b + 1) * static_cast<unsigned>(team);
    volatile unsigned* arr = t;
    volatile unsigned* ab = a.abort;
    for (unsigned it = 0; *arr < target; ++it) {
      if (*ab || it >= a.spin_limit) {
        atomicExch(a.abort, 1u);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_tot = *reinterpret_cast<volatile unsigned*>(t + 1 + b % 3);
    s_ok = ok;
  }
  __syncthreads();
  *total = s_tot;
  return s_ok != 0;
}

__global__ void batch_kernel(BatchArgs a) {
  __shared__ int s_slot;
  __shared__ unsigned int s_changed;
  __shared__ int s_next;  // next tile of this CTA's share, claimed by warps as they finish
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) s_slot = static_cast<int>(atomicAdd(a.ctr, 1u));
    __syncthreads();
    const int slot = s_slot;
    __syncthreads();
    if (slot >= a.n_slots) break;
    if (*reinterpret_cast<volatile unsigned*>(a.abort)) break;
    const int2 sl = a.slots[slot];
    const int inst = sl.x, member = sl.y >> 16, team = sl.y & 0xffff;
    unsigned int* tstate = a.team + 4 * static_cast<int64_t>(inst);
    const int32_t vb = a.vbeg[inst], ve = a.vbeg[inst + 1], n = ve - vb;
    const int tiles = (n + 31) / 32;
    const double inv_n = 1.0 / n;
    const int vt0 = member * blockDim.x + threadIdx.x, vstride = blockDim.x * team;
    int bar = 0;
    // The barrier that ends a phase: a CTA barrier, or the team's.
    auto sync_count = [&](unsigned mine, unsigned* total) -> bool {
      if (team == 1) {
        if (threadIdx.x == 0) s_changed = 0;
        __syncthreads();
        if (threadIdx.x == 0) s_next = 0;
        if (lane == 0 && mine) atomicAdd(&s_changed, mine);
        __syncthreads();
        *total = s_changed;
        __syncthreads();
        return true;
      }
      if (threadIdx.x == 0) s_changed = 0;
      __syncthreads();
      if (threadIdx.x == 0) s_next = 0;
      if (lane == 0 && mine) atomicAdd(&s_changed, mine);
      __syncthreads();
      const unsigned cta = s_changed;
      return team_barrier(a, tstate, team, member, bar++, threadIdx.x == 0 ? cta : 0u, total);
    };
    unsigned tot = 0;
    // ---- PageRank ----
    for (int v = vb + vt0; v < ve; v += vstride) {
      const float r0 = static_cast<float>(inv_n);
      const int32_t od = a.outdeg[v];
      a.pr0[v] = r0;
      a.con0[v] = r0 / static_cast<float>(od > 0 ? od : 1);
    }
    if (!sync_count(0, &tot)) return;
    int cur = 0, step = 0;
    for (step = 0; step < a.pr_iters; ++step) {
      // Ternaries, not a[cur]: runtime indexing of a parameter array would
      // copy the parameter block to local memory.
      const float* con = cur ? a.con1 : a.con0;
      const float* src = cur ? a.pr1 : a.pr0;
      float* dst = cur ? a.pr0 : a.pr1;
      float* dcon = cur ? a.con0 : a.con1;
      unsigned changed = 0;
      for (;;) {
        int k = 0;
        if (lane == 0) k = atomicAdd(&s_next, 1);
        k = __shfl_sync(0xffffffffu, k, 0);
        const int t = member + k * team;  // this CTA's tiles: member, member + team, ...
        if (t >= tiles) break;
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
      if (!sync_count(changed, &tot)) return;
      cur ^= 1;
      if (tot == 0 && step > 1) {
        ++step;
        break;
      }
    }
    for (int v = vb + vt0; v < ve; v += vstride) a.pr_out[v] = (cur ? a.pr1 : a.pr0)[v];
    if (threadIdx.x == 0 && member == 0) a.pr_steps[inst] = step < a.pr_iters ? step : a.pr_iters;
    // ---- CC ----
    for (int v = vb + vt0; v < ve; v += vstride) a.lab0[v] = v - vb;
    if (!sync_count(0, &tot)) return;
    cur = 0;
    for (step = 0; step < a.cc_max; ++step) {
      const int32_t* src = cur ? a.lab1 : a.lab0;
      int32_t* dst = cur ? a.lab0 : a.lab1;
      unsigned changed = 0;
      for (;;) {
        int k = 0;
        if (lane == 0) k = atomicAdd(&s_next, 1);
        k = __shfl_sync(0xffffffffu, k, 0);
        const int t = member + k * team;
        if (t >= tiles) break;
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
      if (!sync_count(changed, &tot)) return;
      cur ^= 1;
      if (tot == 0 && step > 1) {
        ++step;
        break;
      }
    }
    for (int v = vb + vt0; v < ve; v += vstride) a.cc_out[v] = (cur ? a.lab1 : a.lab0)[v];
    if (threadIdx.x == 0 && member == 0) a.cc_steps[inst] = step < a.cc_max ? step : a.cc_max;
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
  int32_t *vbeg = nullptr, *lab0 = nullptr, *lab1 = nullptr, *cc_out = nullptr;
  int32_t *pr_steps = nullptr, *cc_steps = nullptr;
  float *pr0 = nullptr, *pr1 = nullptr, *con0 = nullptr, *con1 = nullptr, *pr_out = nullptr;
  unsigned int* ctr = nullptr;
  int2* slots = nullptr;
  unsigned int* team = nullptr;     // 4 per instance
  unsigned int* abort = nullptr;
  std::vector<int32_t> order;       // instances, longest first
  std::vector<int64_t> work;        // per instance: edges + vertices
  ~BatchDev() {
    dev_free(&vbeg);
    dev_free(&slots);
    dev_free(&team);
    dev_free(&abort);
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
  std::vector<int32_t>& order = d.order;
  order.resize(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
    return e->off[vbeg[x + 1]] - e->off[vbeg[x]] > e->off[vbeg[y + 1]] - e->off[vbeg[y]];
  });
  d.work.resize(n);
  for (int32_t i = 0; i < n; ++i) d.work[i] = (e->off[vbeg[i + 1]] - e->off[vbeg[i]]) + (vbeg[i + 1] - vbeg[i]);
  GX_TRY(dev_alloc(&d.vbeg, static_cast<size_t>(n) + 1));
  GX_TRY(dev_alloc(&d.team, 4 * static_cast<size_t>(n)));
  GX_TRY(dev_alloc(&d.abort, 1));
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
  a.n_inst = n;
  a.ctr = d.ctr;
  a.team = d.team;
  a.abort = d.abort;
  a.spin_limit = e->cfg.wait_limit;  // polls of at least 64 ns each
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

// One persistent launch (plus its cursor and team-state resets), captured as
// a CUDA graph.  The grid holds no more CTAs than are resident at once.
gx_status batch_launch(gx_engine* e, BatchDev& d, BatchArgs& a, const gx_batch_tuning& t, float* ms) {
  cudaStream_t s = e->s_comp;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel, t.threads, 0);
  if (per_sm < 1) return fail(GX_ERR_INVALID, "gx_batch: %d threads per CTA do not fit an SM", t.threads);
  const int blocks = std::min(per_sm, t.ctas_per_sm) * e->n_sm;
  // Work slots: an instance above half a CTA's fair share gets a team of up
  // to 32 CTAs (never more than the grid).
  int64_t total = 0;
  for (int64_t w : d.work) total += w;
  const int64_t share = std::max<int64_t>(1, total / (2 * static_cast<int64_t>(blocks)));
  std::vector<int2> slots;
  slots.reserve(d.order.size());
  for (int32_t inst : d.order) {
    const int team = static_cast<int>(std::min<int64_t>({(d.work[inst] + share - 1) / share, 32, blocks}));
    for (int m = 0; m < std::max(team, 1); ++m) slots.push_back(make_int2(inst, (m << 16) | std::max(team, 1)));
  }
  dev_free(&d.slots);
  GX_TRY(dev_alloc(&d.slots, slots.size()));
  GX_CUDA(cudaMemcpy(d.slots, slots.data(), sizeof(int2) * slots.size(), cudaMemcpyHostToDevice));
  a.slots = d.slots;
  a.n_slots = static_cast<int32_t>(slots.size());
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  GX_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(a.ctr, 0, sizeof(unsigned int), s);
  cudaMemsetAsync(a.team, 0, sizeof(unsigned int) * 4 * static_cast<size_t>(a.n_inst), s);
  cudaMemsetAsync(a.abort, 0, sizeof(unsigned int), s);
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
  unsigned int aborted = 0;
  GX_CUDA(cudaMemcpy(&aborted, a.abort, sizeof(aborted), cudaMemcpyDeviceToHost));
  if (aborted) return fail(GX_ERR_TIMEOUT, "gx_batch: a CTA team barrier timed out");
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
  gx::NvtxRange nvtx_range("gx_batch_run");
  if (!e || n_inst < 1 || !inst_vbegin || pr_iters < 0 || cc_max_iter < 0)
    return fail(GX_ERR_INVALID, "gx_batch_run: bad arguments");
  if (!e->loaded || !e->all_resident) return fail(GX_ERR_STATE, "gx_batch_run: load the packed graph first (all resident)");
  if (e->relabeled) return fail(GX_ERR_STATE, "gx_batch_run: the engine renumbered the vertices (config.relabel)");
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
  GX_TRY(batch_launch(e, d, a, t, &ms));
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
  gx::NvtxRange nvtx_range("gx_batch_autotune");
  if (!e || !best || n_inst < 1 || !inst_vbegin) return fail(GX_ERR_INVALID, "gx_batch_autotune: bad arguments");
  if (!e->loaded || !e->all_resident) return fail(GX_ERR_STATE, "gx_batch_autotune: load the packed graph first");
  if (e->relabeled) return fail(GX_ERR_STATE, "gx_batch_autotune: the engine renumbered the vertices (config.relabel)");
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
        GX_TRY(batch_launch(e, d, a, t, &ms));   // warm
        GX_TRY(batch_launch(e, d, a, t, &ms2));
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

// CPU restatement of GraphMP's engine loop and vertex programs.
//
// TEST INFRASTRUCTURE ONLY: the correctness reference for the CUDA path and the timed CPU
// baseline.  Never linked into the product.  Built with -ffp-contract=off so
// the float PageRank matches the reference bit for bit on x86 and on Arm.
//
// Follows, step by step:
//   engine  GraphPS<T>::run            GraphMP/system/GraphPS.h:171-387
//   shard   init_comp / end_comp       GraphMP/system/Comp.h:21-72
//   PR      comp_pagerank + init       GraphMP/app/pagerank.cpp:20-84
//   SSSP    comp_sssp + init           GraphMP/app/sssp.cpp:20-75
//   CC      comp_cc + init             GraphMP/app/cc.cpp:20-75
//   in-deg  comp_pagerank (cal)        GraphMP/app/cal.cpp:20-79
// One deliberate difference: partition activation under selective
// scheduling uses an exact source test where the reference uses a bloom
// filter (GraphPS.h:349-368).  A bloom filter only adds false positives, and
// re-running a partition none of whose sources changed reproduces its
// values, so the outputs and per-step counts are the same.
#include "gx_oracle.h"

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

namespace {

constexpr int32_t kGpsInf = 10000;   // GPS_INF, GraphMP/system/Global.h:50
constexpr double kBfThre = 0.001;    // BF_THRE, GraphMP/system/Global.h:57

struct Graph {
  int32_t V, P;
  const int32_t* bounds;
  const int64_t* off;
  const int32_t* col;
  const int32_t* outdeg;  // clamped copy where the app clamps
  const uint32_t* w;
};

// GraphPS<T>::run with a per-shard compute functor.  `Comp(p, Msg, MsgNew,
// Value, changed)` processes shard p like the app's _comp.
template <class T, class Comp, class StepHook>
int run_engine(const Graph& g, std::vector<T>& Msg, int32_t max_iter, int threads, Comp comp,
               StepHook after_step, int64_t* changed_out, double* ms_out, int32_t* iters_out) {
  const int32_t V = g.V, P = g.P;
  std::vector<T> Value(V, T(0));        // _VertexValue.assign(V, 0) in every init_vertex
  std::vector<T> MsgNew(Msg);           // GraphPS.h:248
  std::vector<int32_t> parts(P);
  std::vector<char> part_active(P, 1);  // PartitionActive_Bool, GraphPS.h:216
  std::vector<uint8_t> vactive;
  std::mt19937 shuffle_rng(12345);
  int32_t step = 0, executed = 0;
  for (step = 0; step < max_iter; ++step) {
    auto t0 = std::chrono::steady_clock::now();
    std::iota(parts.begin(), parts.end(), 0);
    std::shuffle(parts.begin(), parts.end(), shuffle_rng);  // GraphPS.h:263
    std::atomic<int64_t> changed{0};
#pragma omp parallel for num_threads(threads) schedule(guided)
    for (int32_t k = 0; k < P; ++k) {
      const int32_t p = parts[k];
      if (!part_active[p]) continue;  // GraphPS.h:271-272
      int64_t c = comp(p, Msg.data(), MsgNew.data(), Value.data());
      changed.fetch_add(c, std::memory_order_relaxed);
    }
    const int64_t changed_num = changed.load();
    const double ratio = static_cast<double>(changed_num) / V;  // GraphPS.h:297
    const bool selective = ratio < kBfThre;                      // GraphPS.h:318
    if (selective) {
      vactive.assign(V, 0);
#pragma omp parallel for num_threads(threads) schedule(static)
      for (int32_t v = 0; v < V; ++v) vactive[v] = MsgNew[v] != Msg[v];  // GraphPS.h:325-329
    }
    std::copy(MsgNew.begin(), MsgNew.end(), Msg.begin());  // GraphPS.h:338-345
    if (selective) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
      for (int32_t p = 0; p < P; ++p) {
        char act = 0;
        for (int64_t e = g.off[g.bounds[p]]; e < g.off[g.bounds[p + 1]] && !act; ++e) act = vactive[g.col[e]];
        part_active[p] = act;
      }
    } else {
      std::fill(part_active.begin(), part_active.end(), 1);
    }
    auto t1 = std::chrono::steady_clock::now();
    if (changed_out) changed_out[step] = changed_num;
    if (ms_out) ms_out[step] = std::chrono::duration<double, std::milli>(t1 - t0).count();
    executed = step + 1;
    if (changed_num == 0 && step > 1) break;  // GraphPS.h:383-385
    if (after_step(step)) break;
  }
  if (iters_out) *iters_out = executed;
  return 0;
}

struct NoHook {
  bool operator()(int32_t) const { return false; }
};

}  // namespace

extern "C" int gxo_run(int app, int32_t V, int32_t P, const int32_t* bounds, const int64_t* off,
                       const int32_t* col, const int32_t* outdeg, const uint32_t* w, int32_t max_iter,
                       double damping, int32_t source, double tolerance, int threads,
                       const void* init_vals, void* out_vals, int64_t* changed, double* ms,
                       int32_t* iters_out) {
  if (V <= 0 || P <= 0 || !bounds || !off || !out_vals || max_iter < 0) return 1;
  if (threads <= 0) threads = omp_get_max_threads();
  Graph g{V, P, bounds, off, col, outdeg, w};

  if (app == GXO_PAGERANK_REF) {
    // init_vertex: outdeg 0 -> 1, Msg = 1/N (pagerank.cpp:74-83).
    std::vector<int32_t> od(outdeg, outdeg + V);
    for (auto& d : od)
      if (d == 0) d = 1;
    std::vector<float> Msg(V, static_cast<float>(1.0 / V));
    if (init_vals) memcpy(Msg.data(), init_vals, sizeof(float) * V);
    auto comp = [&](int32_t p, float* M, float* MN, float* Val) -> int64_t {
      int64_t ch = 0;
      const int32_t s = bounds[p], e = bounds[p + 1];
      for (int32_t v = s; v < e; ++v) {
        float rel = 0;
        for (int64_t k = off[v]; k < off[v + 1]; ++k) {
          const int32_t u = col[k];
          rel += M[u] / od[u];  // pagerank.cpp:45-46
        }
        rel = rel * damping + 1.0 / V;  // pagerank.cpp:48 (double, stored as float)
        MN[v] = rel;                    // result[i] -> end_comp, Comp.h:65-67
        if (rel != Val[v]) {            // pagerank.cpp:56-59
          ++ch;
          Val[v] = rel;
        }
      }
      return ch;
    };
    run_engine<float>(g, Msg, max_iter, threads, comp, NoHook{}, changed, ms, iters_out);
    memcpy(out_vals, Msg.data(), sizeof(float) * V);
    return 0;
  }

  if (app == GXO_PAGERANK_REF64) {
    std::vector<int32_t> od(outdeg, outdeg + V);
    for (auto& d : od)
      if (d == 0) d = 1;
    std::vector<double> Msg(V, 1.0 / V);
    if (init_vals) memcpy(Msg.data(), init_vals, sizeof(double) * V);
    auto comp = [&](int32_t p, double* M, double* MN, double* Val) -> int64_t {
      int64_t ch = 0;
      for (int32_t v = bounds[p]; v < bounds[p + 1]; ++v) {
        double rel = 0;
        for (int64_t k = off[v]; k < off[v + 1]; ++k) rel += M[col[k]] / od[col[k]];
        rel = rel * damping + 1.0 / V;
        MN[v] = rel;
        if (rel != Val[v]) {
          ++ch;
          Val[v] = rel;
        }
      }
      return ch;
    };
    run_engine<double>(g, Msg, max_iter, threads, comp, NoHook{}, changed, ms, iters_out);
    memcpy(out_vals, Msg.data(), sizeof(double) * V);
    return 0;
  }

  if (app == GXO_PAGERANK_STD) {
    // r' = (1-d)/N + d*(sum r[u]/outdeg[u] + D/N), D = rank on out-degree-0
    // vertices.  No reference counterpart; FP64 oracle.
    std::vector<double> Msg(V, 1.0 / V);
    if (init_vals) memcpy(Msg.data(), init_vals, sizeof(double) * V);
    double D = 0;
    auto dangling = [&](const std::vector<double>& r) {
      double s = 0;
      for (int32_t v = 0; v < V; ++v)
        if (outdeg[v] == 0) s += r[v];
      return s;
    };
    D = dangling(Msg);
    auto comp = [&](int32_t p, double* M, double* MN, double* Val) -> int64_t {
      int64_t ch = 0;
      const double base = (1.0 - damping) / V + damping * D / V;
      for (int32_t v = bounds[p]; v < bounds[p + 1]; ++v) {
        double acc = 0;
        for (int64_t k = off[v]; k < off[v + 1]; ++k) acc += M[col[k]] / outdeg[col[k]];
        double rel = base + damping * acc;
        MN[v] = rel;
        if (rel != Val[v]) {
          ++ch;
          Val[v] = rel;
        }
      }
      return ch;
    };
    std::vector<double> prev(Msg);
    auto hook = [&](int32_t) -> bool {
      double l1 = 0;
      for (int32_t v = 0; v < V; ++v) l1 += std::fabs(Msg[v] - prev[v]);
      prev = Msg;
      D = dangling(Msg);
      return tolerance > 0 && l1 < tolerance;
    };
    run_engine<double>(g, Msg, max_iter, threads, comp, hook, changed, ms, iters_out);
    memcpy(out_vals, Msg.data(), sizeof(double) * V);
    return 0;
  }

  if (app == GXO_SSSP && !w) {
    // Unit weight, INF = GPS_INF (sssp.cpp:40-47, 68-73).
    std::vector<int32_t> Msg(V, kGpsInf);
    if (source >= 0 && source < V) Msg[source] = 0;
    if (init_vals) memcpy(Msg.data(), init_vals, sizeof(int32_t) * V);
    auto comp = [&](int32_t p, int32_t* M, int32_t* MN, int32_t* Val) -> int64_t {
      int64_t ch = 0;
      for (int32_t v = bounds[p]; v < bounds[p + 1]; ++v) {
        int32_t mn = M[v];
        for (int64_t k = off[v]; k < off[v + 1]; ++k) {
          int32_t tmp = M[col[k]] + 1;
          if (mn > tmp) mn = tmp;
        }
        MN[v] = mn;
        if (mn != Val[v]) {
          ++ch;
          Val[v] = mn;
        }
      }
      return ch;
    };
    run_engine<int32_t>(g, Msg, max_iter, threads, comp, NoHook{}, changed, ms, iters_out);
    memcpy(out_vals, Msg.data(), sizeof(int32_t) * V);
    return 0;
  }

  if (app == GXO_SSSP && w) {
    // uint32 weights, INF = 0xFFFFFFFF, saturating add.  Same pull min-plus.
    std::vector<uint32_t> Msg(V, 0xFFFFFFFFu);
    if (source >= 0 && source < V) Msg[source] = 0;
    if (init_vals) memcpy(Msg.data(), init_vals, sizeof(uint32_t) * V);
    auto comp = [&](int32_t p, uint32_t* M, uint32_t* MN, uint32_t* Val) -> int64_t {
      int64_t ch = 0;
      for (int32_t v = bounds[p]; v < bounds[p + 1]; ++v) {
        uint32_t mn = M[v];
        for (int64_t k = off[v]; k < off[v + 1]; ++k) {
          uint64_t t = static_cast<uint64_t>(M[col[k]]) + w[k];
          uint32_t tmp = t > 0xFFFFFFFFull ? 0xFFFFFFFFu : static_cast<uint32_t>(t);
          if (mn > tmp) mn = tmp;
        }
        MN[v] = mn;
        if (mn != Val[v]) {
          ++ch;
          Val[v] = mn;
        }
      }
      return ch;
    };
    run_engine<uint32_t>(g, Msg, max_iter, threads, comp, NoHook{}, changed, ms, iters_out);
    memcpy(out_vals, Msg.data(), sizeof(uint32_t) * V);
    return 0;
  }

  if (app == GXO_CC) {
    std::vector<int32_t> Msg(V);
    std::iota(Msg.begin(), Msg.end(), 0);  // cc.cpp:70-73
    if (init_vals) memcpy(Msg.data(), init_vals, sizeof(int32_t) * V);
    auto comp = [&](int32_t p, int32_t* M, int32_t* MN, int32_t* Val) -> int64_t {
      int64_t ch = 0;
      for (int32_t v = bounds[p]; v < bounds[p + 1]; ++v) {
        int32_t mn = M[v];
        for (int64_t k = off[v]; k < off[v + 1]; ++k)
          if (mn > M[col[k]]) mn = M[col[k]];  // cc.cpp:41-44
        MN[v] = mn;
        if (mn != Val[v]) {
          ++ch;
          Val[v] = mn;
        }
      }
      return ch;
    };
    run_engine<int32_t>(g, Msg, max_iter, threads, comp, NoHook{}, changed, ms, iters_out);
    memcpy(out_vals, Msg.data(), sizeof(int32_t) * V);
    return 0;
  }

  if (app == GXO_INDEGREE) {
    std::vector<int32_t> Msg(V, 0);  // cal.cpp:77
    auto comp = [&](int32_t p, int32_t* /*Msg: unused, the in-degree reads no values*/, int32_t* MN, int32_t* Val) -> int64_t {
      int64_t ch = 0;
      for (int32_t v = bounds[p]; v < bounds[p + 1]; ++v) {
        int32_t rel = static_cast<int32_t>(off[v + 1] - off[v]);  // cal.cpp:43
        MN[v] = rel;
        if (rel != Val[v]) {
          ++ch;
          Val[v] = rel;
        }
      }
      return ch;
    };
    run_engine<int32_t>(g, Msg, max_iter, threads, comp, NoHook{}, changed, ms, iters_out);
    memcpy(out_vals, Msg.data(), sizeof(int32_t) * V);
    return 0;
  }
  return 2;
}

extern "C" uint64_t gxo_triangles(int32_t V, const int64_t* off, const int32_t* col, int threads) {
  if (threads <= 0) threads = omp_get_max_threads();
  // Orient u -> v iff (deg u, u) < (deg v, v); count |N+(u) ∩ N+(v)| per
  // oriented edge with sorted merges.
  std::vector<int64_t> doff(static_cast<size_t>(V) + 1, 0);
  auto less = [&](int32_t a, int32_t b) {
    int64_t da = off[a + 1] - off[a], db = off[b + 1] - off[b];
    return da < db || (da == db && a < b);
  };
  for (int32_t u = 0; u < V; ++u) {
    int64_t c = 0;
    for (int64_t k = off[u]; k < off[u + 1]; ++k)
      if (col[k] != u && less(u, col[k])) ++c;
    doff[u + 1] = doff[u] + c;
  }
  std::vector<int32_t> dcol(static_cast<size_t>(doff[V]));
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1024)
  for (int32_t u = 0; u < V; ++u) {
    int64_t p = doff[u];
    for (int64_t k = off[u]; k < off[u + 1]; ++k)
      if (col[k] != u && less(u, col[k])) dcol[p++] = col[k];
    std::sort(dcol.begin() + doff[u], dcol.begin() + doff[u + 1]);
  }
  uint64_t total = 0;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256) reduction(+ : total)
  for (int32_t u = 0; u < V; ++u) {
    for (int64_t k = doff[u]; k < doff[u + 1]; ++k) {
      const int32_t v = dcol[k];
      int64_t i = doff[u], ie = doff[u + 1], j = doff[v], je = doff[v + 1];
      while (i < ie && j < je) {
        if (dcol[i] < dcol[j]) ++i;
        else if (dcol[i] > dcol[j]) ++j;
        else {
          ++total;
          ++i;
          ++j;
        }
      }
    }
  }
  return total;
}

extern "C" int gxo_ppr(int32_t V, const int64_t* off, const int32_t* col, const int32_t* outdeg, int32_t k,
                       const int32_t* sources, int32_t iters, double restart, int threads, double* out) {
  if (threads <= 0) threads = omp_get_max_threads();
  const size_t n = static_cast<size_t>(V) * k;
  std::vector<double> R(n, 0.0), Rn(n);
  for (int32_t j = 0; j < k; ++j) R[static_cast<size_t>(sources[j]) * k + j] = 1.0;
  for (int32_t it = 0; it < iters; ++it) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
    for (int32_t v = 0; v < V; ++v) {
      double* dst = &Rn[static_cast<size_t>(v) * k];
      for (int32_t j = 0; j < k; ++j) dst[j] = 0;
      for (int64_t e = off[v]; e < off[v + 1]; ++e) {
        const int32_t u = col[e];
        const double inv = 1.0 / outdeg[u];
        const double* src = &R[static_cast<size_t>(u) * k];
        for (int32_t j = 0; j < k; ++j) dst[j] += src[j] * inv;
      }
      for (int32_t j = 0; j < k; ++j) dst[j] *= (1.0 - restart);
    }
    for (int32_t j = 0; j < k; ++j) Rn[static_cast<size_t>(sources[j]) * k + j] += restart;
    R.swap(Rn);
  }
  memcpy(out, R.data(), n * sizeof(double));
  return 0;
}

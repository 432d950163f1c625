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

// ---------------------------------------------------------------------------
// Graph construction, restated so that the benchmark's reference arm builds
// its input without the product library.  The generator is the library's
// seeded R-MAT: edge i of (seed, scale, a, b, c) draws one 16-bit uniform per
// level from the SplitMix64 finaliser (Steele, Lea and Flood, OOPSLA 2014)
// applied to a per-edge key, four levels per 64-bit draw, and picks the
// quadrant a = (row 0, col 0), b = (0, 1), c = (1, 0), d = (1, 1), row =
// source.  The CSC keeps each destination's sources ascending and unique, as
// GraphMP/tools/format_spark.py:111-157 produces them with scipy's
// csr_matrix; the partition rule is format_spark.py:91-108.
// ---------------------------------------------------------------------------
namespace {

uint64_t splitmix_final(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

}  // namespace

extern "C" int gxo_rmat_csc(int32_t scale, int64_t n, double a, double b, double c, uint64_t seed, int32_t drop_self,
                            int32_t dedup, int32_t symmetric, int threads, int64_t* off, int32_t* col,
                            int64_t* n_out) {
  if (scale < 1 || scale > 30 || n < 0 || !off || !n_out || (n > 0 && !col)) return 1;
  if (threads <= 0) threads = omp_get_max_threads();
  const int64_t V = int64_t(1) << scale;
  const uint32_t qa = static_cast<uint32_t>(std::llround(a * 65536.0));
  const uint32_t qb = qa + static_cast<uint32_t>(std::llround(b * 65536.0));
  const uint32_t qc = qb + static_cast<uint32_t>(std::llround(c * 65536.0));
  const uint64_t base = splitmix_final(seed ^ 0x5ca1ab1e0ddba11ull);
  auto edge = [&](int64_t i, uint32_t* s_out, uint32_t* d_out) {
    const uint64_t key = base ^ (static_cast<uint64_t>(i) * 0xd1b54a32d192ed03ull);
    uint32_t s = 0, d = 0;
    for (int level = 0; level < scale; ++level) {
      const uint64_t draw = splitmix_final(key + static_cast<uint64_t>(level / 4 + 1) * 0x9e3779b97f4a7c15ull);
      const uint32_t x = static_cast<uint32_t>(draw >> (16 * (level % 4))) & 0xffffu;
      const uint32_t bit = 1u << (scale - 1 - level);
      if (x >= qa) {
        if (x < qb) d |= bit;
        else if (x < qc) s |= bit;
        else s |= bit, d |= bit;
      }
    }
    *s_out = s;
    *d_out = d;
  };
  // The edges once, then in-degree counts (with the reverse direction when
  // symmetric), the fill, and per destination a sort and deduplication.
  std::vector<uint32_t> es(static_cast<size_t>(n)), ed(static_cast<size_t>(n));
  std::vector<std::atomic<int64_t>> cnt(static_cast<size_t>(V));
  for (auto& x : cnt) x.store(0, std::memory_order_relaxed);
#pragma omp parallel for num_threads(threads) schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    uint32_t s, d;
    edge(i, &s, &d);
    es[i] = s;
    ed[i] = d;
    if (drop_self && s == d) continue;
    cnt[d].fetch_add(1, std::memory_order_relaxed);
    if (symmetric) cnt[s].fetch_add(1, std::memory_order_relaxed);
  }
  off[0] = 0;
  for (int64_t v = 0; v < V; ++v) off[v + 1] = off[v] + cnt[v].load(std::memory_order_relaxed);
#pragma omp parallel for num_threads(threads) schedule(static)
  for (int64_t v = 0; v < V; ++v) cnt[v].store(off[v], std::memory_order_relaxed);
#pragma omp parallel for num_threads(threads) schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t s = es[i], d = ed[i];
    if (drop_self && s == d) continue;
    col[cnt[d].fetch_add(1, std::memory_order_relaxed)] = static_cast<int32_t>(s);
    if (symmetric) col[cnt[s].fetch_add(1, std::memory_order_relaxed)] = static_cast<int32_t>(d);
  }
  std::vector<int64_t> kept(static_cast<size_t>(V));
#pragma omp parallel for num_threads(threads) schedule(dynamic, 4096)
  for (int64_t v = 0; v < V; ++v) {
    int32_t* lo = col + off[v];
    int32_t* hi = col + off[v + 1];
    std::sort(lo, hi);
    kept[v] = dedup ? std::unique(lo, hi) - lo : hi - lo;
  }
  // Compact in order (kept[v] <= the old list length, so moves go left).
  int64_t w = 0;
  for (int64_t v = 0; v < V; ++v) {
    const int64_t from = off[v];
    if (w != from) memmove(col + w, col + from, sizeof(int32_t) * static_cast<size_t>(kept[v]));
    off[v] = w;
    w += kept[v];
  }
  off[V] = w;
  *n_out = w;
  return 0;
}

extern "C" int gxo_partition_bounds(int32_t V, const int64_t* off, int32_t P, int32_t* bounds) {
  if (V < 0 || P < 1 || !off || !bounds) return 1;
  const int64_t per = (off[V] + P - 1) / P;  // ceil(E/P), format_spark.py:91
  bounds[0] = 0;
  for (int32_t i = 1; i < P; ++i) {
    // First vertex whose cumulative in-degree reaches per*i (format_spark.py:100-101).
    const int64_t* it = std::lower_bound(off, off + V + 1, per * i);
    bounds[i] = std::max(bounds[i - 1], static_cast<int32_t>(std::min<int64_t>(it - off, V)));
  }
  bounds[P] = V;
  return 0;
}

extern "C" int gxo_out_degree(int32_t V, const int64_t* off, const int32_t* col, int threads, int32_t* outdeg) {
  if (V < 0 || !off || !outdeg) return 1;
  if (threads <= 0) threads = omp_get_max_threads();
  std::vector<std::atomic<int32_t>> od(static_cast<size_t>(V));
  for (auto& x : od) x.store(0, std::memory_order_relaxed);
#pragma omp parallel for num_threads(threads) schedule(static)
  for (int64_t k = 0; k < off[V]; ++k) od[col[k]].fetch_add(1, std::memory_order_relaxed);
  for (int32_t v = 0; v < V; ++v) outdeg[v] = od[v].load(std::memory_order_relaxed);
  return 0;
}

// SSSP weight of edge u -> v in [1, 255], a pure function of (seed, u, v).
extern "C" int gxo_edge_weights(uint64_t seed, int32_t V, const int64_t* off, const int32_t* col, int threads,
                                uint32_t* w) {
  if (V < 0 || !off || (off[V] > 0 && (!col || !w))) return 1;
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for num_threads(threads) schedule(dynamic, 4096)
  for (int32_t v = 0; v < V; ++v)
    for (int64_t k = off[v]; k < off[v + 1]; ++k) {
      const uint64_t pair = (static_cast<uint64_t>(static_cast<uint32_t>(col[k])) << 32) | static_cast<uint32_t>(v);
      w[k] = 1u + static_cast<uint32_t>(splitmix_final(seed ^ splitmix_final(pair)) % 255u);
    }
  return 0;
}

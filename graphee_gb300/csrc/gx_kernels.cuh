// Device kernels of the superstep loop (GraphPS<T>::run,
// GraphMP/system/GraphPS.h:256-386) for one GB300.
//
// One superstep is three launches that read a device control block, so a
// run of K supersteps can be replayed as one CUDA graph with no host sync:
//   pull_kernel<APP>      gather-apply over in-edges (CSC) of the swept shards
//   push_kernel<APP>      sparse min-plus / min-label over out-edges of the frontier
//   finalize_kernel<APP>  step statistics, frontier compaction, shard activation,
//                         termination, buffer swap
// Each kernel returns at once when the control block says the step is not
// its mode, or that the run is done.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gx {

enum AppKind : int { K_PR_REF = 0, K_PR_STD = 1, K_SSSP_UNIT = 2, K_SSSP_W = 3, K_CC = 4, K_INDEG = 5 };
enum StepMode : int { MODE_DENSE = 0, MODE_SELECTIVE = 1, MODE_PUSH = 2 };

constexpr int kThreads = 256;           // threads per CTA of pull/push kernels
constexpr int kWarps = kThreads / 32;
constexpr int kChunk = 256;             // edges staged per warp per round
constexpr int kGpsInf = 10000;          // GPS_INF, GraphMP/system/Global.h:50
constexpr uint32_t kInfW = 0xFFFFFFFFu; // INF of weighted SSSP
constexpr int kPushChunk = 256;         // out-edges per push frontier entry (longer lists get several)

struct StepStats {
  unsigned long long changed;  // reference _Changed_Vertex
  unsigned long long active;   // |{v : new != old}|
  unsigned long long edges;    // edges read
  unsigned long long resid_fx; // PageRank: sum |new-old| in fixed point
  unsigned long long dangl_fx; // PageRank STD: rank on out-degree-0 vertices, fixed point
  int shards_active;
  int mode;
};

// Which shards a selective step sweeps (the partition activation of
// GraphPS.h:349-368, exact per shard instead of a bloom filter):
enum MarkMode : int {
  MARK_NONE = 0,     // selective steps sweep every shard
  MARK_OUT = 1,      // finalize marks the shards of the changed vertices' out-neighbours (out-edge CSR)
  MARK_LIST = 2      // finalize lists the changed vertices; the host marks their shards (streamed graphs)
};

// Control block.  Fields above `step` are set by the host before a run; the
// rest evolve on the device.
struct Ctl {
  int max_iter;
  int n_vertices;
  int n_shards;
  int shard_words;          // 32-bit words of one shard bitmap, (P + 31) / 32
  int push_ok;              // out-edges resident: sparse steps may push
  int step0_push;           // SSSP from init_vertex: step 0 pushes from the source alone
  int async_mode;           // min apps: pull updates values in place (no buffer swap)
  int mark_mode;            // MarkMode
  unsigned long long push_edge_limit;  // push when the frontier has at most this many out-edges
  uint32_t* shard_bm;       // MARK_OUT: two shard bitmaps of shard_words words; [shard_cur] is current
  const int64_t* ooff;      // MARK_OUT: out-edge CSR and the shards' vertex bounds (P+1)
  const int32_t* ocol;
  const int32_t* bounds;
  int32_t* changed_list;    // MARK_LIST: the changed vertices of the last step
  unsigned int changed_cap;
  int pad0;
  double damping;
  double inv_n;             // 1.0 / N, as the reference computes it
  double fx_scale;          // fixed-point scale of resid_fx / dangl_fx
  double tolerance;         // PageRank L1 stop (0 = off)
  double sel_threshold;     // BF_THRE
  // evolving
  int step;
  int cur;                  // index of the buffer holding the current values
  int mode;                 // StepMode of the current step
  int done;
  int n_frontier;           // frontier entries for the current push step
  int error;
  double base;              // PageRank STD: (1-d)/N + d*D/N of the current step
  int shard_cur;            // MARK_OUT: index of the current step's shard bitmap
  int shard_valid;          // MARK_OUT: the current bitmap was marked for this (selective) step
  unsigned int n_changed_list;  // MARK_LIST: entries written (the host resets it)
  int list_overflow;        // MARK_LIST: more changed vertices than changed_cap
  unsigned long long changed, active, edges, resid_fx, dangl_fx;  // current-step accumulators
  unsigned long long front_edges;      // out-edges of the vertices that changed this step
  unsigned int next_frontier;
  unsigned int fin_ticket;
};

struct PullArgs {
  Ctl* ctl;
  const int64_t* off;       // global in-edge offsets, V+1
  const int32_t* col;       // source ids, indexed by global edge id (may be rebased for a streamed shard)
  const uint32_t* w;        // weights aligned with col (SSSP weighted)
  const int32_t* outdeg;    // raw out-degree
  void* val[2];             // T[V] double buffer
  float* con[2];            // PageRank contributions r[u]/outdeg[u], double buffer
  const int2* units;        // work units: tile (vb, ve) or heavy chunk (-(h+1), chunk)
  const int32_t* unit_shard;
  int32_t u_begin, u_end;   // units of this launch
  const int4* heavy;        // heavy vertex h: (v, n_chunks, partial base, shard)
  void* partial;            // per-chunk partial results (T)
  unsigned int* hticket;    // per heavy vertex: chunks finished this step
  unsigned int* ctr;        // kQueues work-unit cursors of this launch (reset by finalize)
  int32_t heavy_deg;        // lists longer than this are swept by their own units
  uint32_t* bm;             // next-frontier bitmap
  // Compressed shard (COMP launches): chunk headers indexed by global chunk
  // id (edge >> 5), payload words, and byte weights indexed by global edge id.
  const uint2* chdr;
  const uint32_t* cpay;
  const uint8_t* w8;
  // Hot-source table (HOT launches): the values (PageRank: contributions)
  // of sources [0, hot_n) are copied into shared memory at the start of the
  // launch and gathered from there.
  int32_t hot_n;
  // 1: a shard the step does not sweep (host-driven selective steps of
  // streamed graphs): every unit only carries its vertices' values over, and
  // no edge is read (col then points nowhere valid).
  int32_t skip;
};

struct PushArgs {
  Ctl* ctl;
  const int64_t* ooff;      // out-edge offsets, V+1
  const int32_t* ocol;      // destinations
  const uint32_t* ow;       // weights aligned with ocol
  void* val[2];
  const int32_t* outdeg;
  const int4* frontier;     // (vertex, value bits, first out-edge of the entry, 0) from the previous step
  unsigned int* ctr;
  uint32_t* bm;
};

struct FinArgs {
  Ctl* ctl;
  StepStats* stats;
  uint32_t* bm;
  int32_t n_words;
  void* val[2];
  const int32_t* outdeg;
  int4* frontier;
  unsigned long long frontier_cap;  // entries; |frontier| + E / kPushChunk + 1 fit by construction
  unsigned int* work_ctr;
  int32_t n_work_ctr;
};

template <int APP> struct AppTraits;
template <> struct AppTraits<K_PR_REF> { typedef float T; };
template <> struct AppTraits<K_PR_STD> { typedef float T; };
template <> struct AppTraits<K_SSSP_UNIT> { typedef int32_t T; };
template <> struct AppTraits<K_SSSP_W> { typedef uint32_t T; };
template <> struct AppTraits<K_CC> { typedef int32_t T; };
template <> struct AppTraits<K_INDEG> { typedef int32_t T; };

template <int APP> constexpr bool is_pr() { return APP == K_PR_REF || APP == K_PR_STD; }

__device__ __forceinline__ uint32_t sat_add(uint32_t a, uint32_t b) {
  uint32_t s = a + b;
  return s < a ? kInfW : s;
}

// Candidate an in-edge (u -> v) offers v: PageRank contribution, or the
// min-plus / min-label candidate.
#ifndef GX_GATHER_CG
#define GX_GATHER_CG 0
#endif

// The value source u offers: from the shared-memory table when HOT and u is
// one of its hot_n sources, else from global memory.  Both loads are issued
// without a branch (the table read at a clamped index, the global read under
// a predicate), so a lane keeps all of its gathers in flight; cache hints on
// the global read (L1::no_allocate, L1::evict_first) measured 1.2-2x slower.
// ASYNC (Gauss-Seidel, min apps only): values are read and written in one
// buffer during the step, so gathers go through L2 (ld.cg), never the
// read-only path.
template <class T, bool ASYNC, bool HOT>
__device__ __forceinline__ T gather(const T* src, const T* hot, int32_t hot_n, int32_t u) {
  static_assert(sizeof(T) == 4, "4-byte values");
  if constexpr (HOT) {
    uint32_t r;
    memcpy(&r, hot + (u < hot_n ? u : hot_n - 1), 4);
    asm("{\n\t.reg .pred p;\n\tsetp.ge.s32 p, %1, %2;\n\t@p ld.global.nc.b32 %0, [%3];\n\t}"
        : "+r"(r) : "r"(u), "r"(hot_n), "l"(src + u));
    T x;
    memcpy(&x, &r, 4);
    return x;
  } else if constexpr (ASYNC) {
    return __ldcg(src + u);
  } else {
    return __ldg(src + u);
  }
}

template <int APP, bool ASYNC = false, bool HOT = false>
__device__ __forceinline__ typename AppTraits<APP>::T edge_value(const PullArgs& a, const void* src_val,
                                                                 const float* src_con, int32_t u, uint32_t wt,
                                                                 const void* hot = nullptr) {
  if constexpr (is_pr<APP>()) {
    if (GX_GATHER_CG && !HOT) return __ldcg(src_con + u);
    return gather<float, false, HOT>(src_con, static_cast<const float*>(hot), a.hot_n, u);
  } else if constexpr (APP == K_SSSP_UNIT) {
    return gather<int32_t, ASYNC, HOT>(static_cast<const int32_t*>(src_val), static_cast<const int32_t*>(hot),
                                       a.hot_n, u) + 1;  // sssp.cpp:43
  } else if constexpr (APP == K_SSSP_W) {
    return sat_add(gather<uint32_t, ASYNC, HOT>(static_cast<const uint32_t*>(src_val),
                                                static_cast<const uint32_t*>(hot), a.hot_n, u), wt);
  } else {
    return gather<int32_t, ASYNC, HOT>(static_cast<const int32_t*>(src_val), static_cast<const int32_t*>(hot),
                                       a.hot_n, u);  // cc.cpp:42
  }
}

template <int APP>
__device__ __forceinline__ typename AppTraits<APP>::T combine(typename AppTraits<APP>::T acc,
                                                              typename AppTraits<APP>::T x) {
  if constexpr (is_pr<APP>()) return acc + x;  // pagerank.cpp:46, ascending edge order
  else return x < acc ? x : acc;
}

// Per-step scalars the apply step needs.
struct ApplyCtx {
  int step;
  double damping, inv_n, fx_scale, base;
  const int32_t* outdeg;  // min apps that may push: sum the out-degree of changed vertices
};

struct LocalAcc {
  unsigned long long changed = 0, active = 0, edges = 0, resid = 0, dangl = 0, fedges = 0;
};

// Apply step for vertex v given its gathered value (end of comp_* + end_comp):
// writes MsgNew[v] (and the next contribution), counts changes.
template <int APP>
__device__ __forceinline__ bool apply_vertex(const ApplyCtx c, int v, typename AppTraits<APP>::T acc,
                                             typename AppTraits<APP>::T old, int32_t od, void* dst_val, float* dst_con,
                                             LocalAcc& la) {
  typedef typename AppTraits<APP>::T T;
  T nv;
  if constexpr (APP == K_PR_REF) {
    // rel = rel*0.85 + 1.0/VertexNum in double, stored as float (pagerank.cpp:48);
    // explicit _rn ops keep the compiler from contracting into an FMA.
    nv = static_cast<float>(__dadd_rn(__dmul_rn(static_cast<double>(acc), c.damping), c.inv_n));
  } else if constexpr (APP == K_PR_STD) {
    nv = static_cast<float>(__dadd_rn(c.base, __dmul_rn(c.damping, static_cast<double>(acc))));
  } else {
    nv = acc;
  }
  static_cast<T*>(dst_val)[v] = nv;
  if constexpr (is_pr<APP>()) {
    dst_con[v] = nv / static_cast<float>(od > 0 ? od : 1);  // Msg[u]/_VertexOut[u], clamp pagerank.cpp:77-80
    const double diff = fabs(static_cast<double>(nv) - static_cast<double>(old));
    la.resid += __double2ull_rn(diff * c.fx_scale);
    if (APP == K_PR_STD && od == 0) la.dangl += __double2ull_rn(static_cast<double>(nv) * c.fx_scale);
  }
  // _Changed_Vertex counts new != VertexValue; VertexValue is 0 before the
  // first step and equals Msg afterwards (pagerank.cpp:56-59, GraphPS.h:338-345).
  const T prev = c.step == 0 ? T(0) : old;
  la.changed += (nv != prev);
  const bool act = nv != old;
  la.active += act;  // not reported from here; finalize recounts from the bitmap
  if constexpr (!is_pr<APP>()) {
    if (act && c.outdeg) la.fedges += static_cast<unsigned long long>(__ldg(c.outdeg + v));
  }
  return act;
}

__device__ __forceinline__ void bitmap_set_tile(uint32_t* bm, int vb, unsigned mask) {
  // Lanes are consecutive vertices vb..vb+31: at most two bitmap words.
  if (mask == 0) return;
  const int sh = vb & 31;
  const int w0 = vb >> 5;
  const unsigned lo = mask << sh;
  const unsigned hi = sh ? (mask >> (32 - sh)) : 0u;
  if (lo) atomicOr(bm + w0, lo);
  if (hi) atomicOr(bm + w0 + 1, hi);
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// ---------------------------------------------------------------------------
// Pull.  The swept vertices are cut into warp work units of bounded size,
// which warps claim a few at a time from a per-launch counter:
//  * a tile of up to 32 consecutive vertices of in-degree <= heavy: lanes
//    with in-degree <= kLaneMaxDegree walk their own edge list (two 128-bit
//    index loads per step, next pair prefetched) and fold in edge order,
//    which is the reference's summation order (pagerank.cpp:44-47); lanes
//    with up to GX_MID_MAX edges are then swept four lists at a time by
//    groups of 8 lanes, and longer lists by the whole warp one by one
//    (coalesced index loads, fixed-shape tree sums);
//  * a heavy vertex (in-degree > heavy) is split into chunks of kHeavyChunk
//    edges; each chunk is reduced by one warp, and the warp that finishes a
//    vertex's last chunk folds the partials in chunk order and applies it.
// In exact-order mode (EXACT) every vertex is folded sequentially in edge
// order: tiles with a longer list stage their edge range through shared
// memory and each lane folds its own slice; no vertex is chunked.
// Results are deterministic run to run in both modes.
// ---------------------------------------------------------------------------
constexpr int kHeavyChunk = 2048;
#ifndef GX_LANE_MAX
#define GX_LANE_MAX 16
#endif
#ifndef GX_GRAB
#define GX_GRAB 4
#endif
#ifndef GX_TILE_PREFETCH
#define GX_TILE_PREFETCH 0
#endif
constexpr int kLaneMaxDegree = GX_LANE_MAX;  // longest list a lane walks alone
constexpr int kGrab = GX_GRAB;               // units a warp claims per atomic
constexpr int kQueues = 64;          // work-unit cursors per launch

// Queue q of nq splits U units evenly; its cursor counts units handed out.
// Returns the first queue after q (cyclically) whose cursor is below its
// size, reading every cursor in one round trip, or -1 when all are drained.
__device__ __forceinline__ int next_queue(const unsigned int* ctr, int q, int nq, int64_t U, int lane) {
  bool ok0 = false, ok1 = false;
  if (lane < nq) {
    const int64_t size = (U * (lane + 1)) / nq - (U * lane) / nq;
    ok0 = static_cast<int64_t>(*reinterpret_cast<const volatile unsigned int*>(ctr + lane)) < size;
  }
  if (lane + 32 < nq) {
    const int j = lane + 32;
    const int64_t size = (U * (j + 1)) / nq - (U * j) / nq;
    ok1 = static_cast<int64_t>(*reinterpret_cast<const volatile unsigned int*>(ctr + j)) < size;
  }
  const unsigned long long left = static_cast<unsigned long long>(__ballot_sync(0xffffffffu, ok0)) |
                                  (static_cast<unsigned long long>(__ballot_sync(0xffffffffu, ok1)) << 32);
  if (!left) return -1;
  const unsigned long long after = q + 1 < 64 ? (left >> (q + 1)) << (q + 1) : 0ull;
  return __ffsll(static_cast<long long>(after ? after : left)) - 1;
}

template <class T>
__device__ __forceinline__ void store4(T* dst, const T (&x)[4]) {
  uint4 u;
  memcpy(&u.x, &x[0], 4);
  memcpy(&u.y, &x[1], 4);
  memcpy(&u.z, &x[2], 4);
  memcpy(&u.w, &x[3], 4);
  *reinterpret_cast<uint4*>(dst) = u;
}

template <int APP>
__device__ __forceinline__ typename AppTraits<APP>::T identity() {
  typedef typename AppTraits<APP>::T T;
  if constexpr (is_pr<APP>()) return T(0);
  else if constexpr (APP == K_SSSP_W) return kInfW;
  else return T(0x7fffffff);
}

template <int NW = kWarps>
__device__ __forceinline__ void flush_block(Ctl* ctl, const LocalAcc& la) {
  __shared__ unsigned long long s_red[5][NW];
  unsigned long long ch = warp_sum(la.changed), ed = warp_sum(la.edges), rs = warp_sum(la.resid),
                     dg = warp_sum(la.dangl), fe = warp_sum(la.fedges);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    s_red[0][wid] = ch;
    s_red[1][wid] = ed;
    s_red[2][wid] = rs;
    s_red[3][wid] = dg;
    s_red[4][wid] = fe;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    unsigned long long t = 0;
    for (int i = 0; i < NW; ++i) t += s_red[threadIdx.x][i];
    unsigned long long* dst = threadIdx.x == 0 ? &ctl->changed
                            : threadIdx.x == 1 ? &ctl->edges
                            : threadIdx.x == 2 ? &ctl->resid_fx
                            : threadIdx.x == 3 ? &ctl->dangl_fx
                                               : &ctl->front_edges;
    if (t) atomicAdd(dst, t);
  }
}

// Compressed shard format: the source ids of global edges [32c, 32c+32) form
// chunk c, stored as hdr[c] = (min, w16 << 3 | nb) and 32 offsets id - min of
// nb bytes each (nb = 0..4, the fewest that hold the largest), at byte
// 16 * w16 of the payload.  Returns the ids of edges k..k+3 (k a multiple of
// 4: all four lie in one chunk, and their bytes start 4-byte aligned, 8-byte
// for nb = 2, 16-byte for nb = 4).
__device__ __forceinline__ int4 comp_idx4(const uint2* hdr, const uint32_t* pay, int64_t k) {
  const uint2 h = __ldg(hdr + (k >> 5));
  const uint32_t nb = h.y & 7u;
  const uint32_t j0 = static_cast<uint32_t>(k & 31);
  const unsigned char* p = reinterpret_cast<const unsigned char*>(pay) + static_cast<size_t>(h.y >> 3) * 16 + j0 * nb;
  uint32_t v0 = 0, v1 = 0, v2 = 0, v3 = 0;
  if (nb == 1) {
    const uint32_t x = __ldg(reinterpret_cast<const unsigned int*>(p));
    v0 = x & 255u, v1 = (x >> 8) & 255u, v2 = (x >> 16) & 255u, v3 = x >> 24;
  } else if (nb == 2) {
    const uint2 x = __ldg(reinterpret_cast<const uint2*>(p));
    v0 = x.x & 0xffffu, v1 = x.x >> 16, v2 = x.y & 0xffffu, v3 = x.y >> 16;
  } else if (nb == 3) {
    const unsigned int* q = reinterpret_cast<const unsigned int*>(p);
    const uint32_t w0 = __ldg(q), w1 = __ldg(q + 1), w2 = __ldg(q + 2);
    v0 = w0 & 0xffffffu;
    v1 = (w0 >> 24) | ((w1 & 0xffffu) << 8);
    v2 = (w1 >> 16) | ((w2 & 0xffu) << 16);
    v3 = w2 >> 8;
  } else if (nb == 4) {
    const uint4 x = __ldg(reinterpret_cast<const uint4*>(p));
    v0 = x.x, v1 = x.y, v2 = x.z, v3 = x.w;
  }
  const uint32_t m = h.x;
  return make_int4(static_cast<int>(m + v0), static_cast<int>(m + v1), static_cast<int>(m + v2),
                   static_cast<int>(m + v3));
}

// Source ids / weights of edges k..k+3 (k a multiple of 4): 128-bit loads of
// the plain arrays, or the compressed shard's chunk and byte weights.
template <bool COMP>
__device__ __forceinline__ int4 load_idx4(const PullArgs& a, int64_t k) {
  if constexpr (COMP) return comp_idx4(a.chdr, a.cpay, k);
  else return __ldcs(reinterpret_cast<const int4*>(a.col + k));
}
template <bool COMP>
__device__ __forceinline__ uint4 load_w4(const PullArgs& a, int64_t k) {
  if constexpr (COMP) {
    const uint32_t x = __ldcs(reinterpret_cast<const unsigned int*>(a.w8 + k));
    return make_uint4(x & 255u, (x >> 8) & 255u, (x >> 16) & 255u, x >> 24);
  } else {
    return __ldcs(reinterpret_cast<const uint4*>(a.w + k));
  }
}

// Warp-cooperative reduction of the edge range [b, e) (all lanes call it with
// the same range): lanes take 8 consecutive edges each per round, with
// 128-bit loads; the per-lane partials are combined by a fixed xor tree.
template <int APP, bool ASYNC = false, bool COMP = false, bool HOT = false>
__device__ __forceinline__ typename AppTraits<APP>::T warp_reduce_range(const PullArgs& a, const void* src_val,
                                                                        const float* src_con, int64_t b, int64_t e,
                                                                        int lane, const void* hot = nullptr) {
  typedef typename AppTraits<APP>::T T;
  T acc = identity<APP>();
  for (int64_t q = (b & ~3ll) + 4 * lane; q < e; q += 256) {
    const int64_t q2 = q + 128;
    const int4 c4 = load_idx4<COMP>(a, q);
    int4 d4 = make_int4(0, 0, 0, 0);
    if (q2 < e) d4 = load_idx4<COMP>(a, q2);
    uint4 w4 = make_uint4(0, 0, 0, 0), x4 = make_uint4(0, 0, 0, 0);
    if constexpr (APP == K_SSSP_W) {
      w4 = load_w4<COMP>(a, q);
      if (q2 < e) x4 = load_w4<COMP>(a, q2);
    }
    const int cs[8] = {c4.x, c4.y, c4.z, c4.w, d4.x, d4.y, d4.z, d4.w};
    const uint32_t ws[8] = {w4.x, w4.y, w4.z, w4.w, x4.x, x4.y, x4.z, x4.w};
    T vals[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int64_t k = (j < 4 ? q : q2) + (j & 3);
      vals[j] = (k >= b && k < e) ? edge_value<APP, ASYNC, HOT>(a, src_val, src_con, cs[j], ws[j], hot)
                                  : identity<APP>();
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) acc = combine<APP>(acc, vals[j]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc = combine<APP>(acc, __shfl_xor_sync(0xffffffffu, acc, o));
  return acc;
}

// Group-wise reduction of the edge range [b, e) by the GL lanes of group
// grp (lanes GL*grp .. GL*grp+GL-1, all calling with the same range): each
// lane takes 8 edges per round (two 128-bit index loads 4*GL edges apart),
// and the lanes' partials meet in a fixed xor tree within the group.
#ifndef GX_GROUP_SWEEP
#define GX_GROUP_SWEEP 1
#endif
#ifndef GX_MID_MAX
#define GX_MID_MAX 128
#endif
#ifndef GX_GROUP_LANES
#define GX_GROUP_LANES 8
#endif
constexpr int kGroupLanes = GX_GROUP_LANES;
template <int APP, bool ASYNC = false, bool COMP = false, bool HOT = false>
__device__ __forceinline__ typename AppTraits<APP>::T group_reduce_range(const PullArgs& a, const void* src_val,
                                                                         const float* src_con, int64_t b, int64_t e,
                                                                         int gl, int grp, const void* hot) {
  typedef typename AppTraits<APP>::T T;
  T acc = identity<APP>();
  for (int64_t q = (b & ~3ll) + 4 * gl; q < e; q += 8 * kGroupLanes) {
    const int64_t q2 = q + 4 * kGroupLanes;
    const int4 c4 = load_idx4<COMP>(a, q);
    int4 d4 = make_int4(0, 0, 0, 0);
    if (q2 < e) d4 = load_idx4<COMP>(a, q2);
    uint4 w4 = make_uint4(0, 0, 0, 0), x4 = make_uint4(0, 0, 0, 0);
    if constexpr (APP == K_SSSP_W) {
      w4 = load_w4<COMP>(a, q);
      if (q2 < e) x4 = load_w4<COMP>(a, q2);
    }
    const int cs[8] = {c4.x, c4.y, c4.z, c4.w, d4.x, d4.y, d4.z, d4.w};
    const uint32_t ws[8] = {w4.x, w4.y, w4.z, w4.w, x4.x, x4.y, x4.z, x4.w};
    T vals[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int64_t k = (j < 4 ? q : q2) + (j & 3);
      vals[j] = (k >= b && k < e) ? edge_value<APP, ASYNC, HOT>(a, src_val, src_con, cs[j], ws[j], hot)
                                  : identity<APP>();
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) acc = combine<APP>(acc, vals[j]);
  }
  const unsigned gmask = kGroupLanes == 32 ? 0xffffffffu : (((1u << kGroupLanes) - 1u) << (grp * kGroupLanes));
#pragma unroll
  for (int o = kGroupLanes / 2; o > 0; o >>= 1) acc = combine<APP>(acc, __shfl_xor_sync(gmask, acc, o));
  return acc;
}

#ifndef GX_PULL_MIN_BLOCKS
#define GX_PULL_MIN_BLOCKS 4
#endif

// HOT launches run one CTA of kHotThreads per SM, whose dynamic shared
// memory holds the hot-source table (a.hot_n values, a multiple of 4).
constexpr int kHotThreads = 1024;
template <bool HOT> constexpr int pull_threads() { return HOT ? kHotThreads : kThreads; }

template <int APP, bool EXACT, bool ASYNC = false, bool COMP = false, bool HOT = false>
__global__ void __launch_bounds__(pull_threads<HOT>(), HOT ? 1 : GX_PULL_MIN_BLOCKS) pull_kernel(PullArgs a) {
  typedef typename AppTraits<APP>::T T;
  static_assert(!(HOT && ASYNC), "a Gauss-Seidel step changes the values the table would hold");
  constexpr int NW = pull_threads<HOT>() / 32;
  __shared__ __align__(16) T s_buf[EXACT ? NW : 1][EXACT ? kChunk : 4];
  extern __shared__ __align__(16) unsigned char s_dyn[];
  Ctl* ctl = a.ctl;
  const int done = ctl->done, mode = ctl->mode;
  if (done || mode == MODE_PUSH) return;
  const void* hot = nullptr;
  if constexpr (HOT) {
    // The current step's values of sources [0, hot_n) (PageRank: their
    // contributions), read through L2 in 16-byte pieces.
    const int4* src = reinterpret_cast<const int4*>(
        is_pr<APP>() ? static_cast<const void*>(ctl->cur ? a.con[1] : a.con[0])
                     : static_cast<const void*>(ctl->cur ? a.val[1] : a.val[0]));
    int4* dst = reinterpret_cast<int4*>(s_dyn);
    for (int i = threadIdx.x; i < (a.hot_n >> 2); i += pull_threads<HOT>()) dst[i] = __ldcg(src + i);
    __syncthreads();
    hot = s_dyn;
  }
  ApplyCtx c;
  c.step = ctl->step;
  c.damping = ctl->damping;
  c.inv_n = ctl->inv_n;
  c.fx_scale = ctl->fx_scale;
  c.base = ctl->base;
  c.outdeg = ctl->push_ok ? a.outdeg : nullptr;
  const int cur = ctl->cur;
  // Selective steps skip the units of shards the last finalize left unmarked.
  const uint32_t* sbm = (mode == MODE_SELECTIVE && ctl->shard_valid)
                            ? ctl->shard_bm + static_cast<int64_t>(ctl->shard_cur) * ctl->shard_words
                            : nullptr;
  // Ternaries, not a[cur]: indexing a parameter array with a runtime value
  // would copy the whole parameter block to local memory.
  const void* src_val = cur ? a.val[1] : a.val[0];
  // Gauss-Seidel: new values overwrite the current ones in place.
  void* dst_val = ASYNC ? const_cast<void*>(src_val) : (cur ? a.val[0] : a.val[1]);
  const float* src_con = cur ? a.con[1] : a.con[0];
  float* dst_con = cur ? a.con[0] : a.con[1];
  const bool selective = sbm != nullptr;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T* buf = s_buf[EXACT ? wid : 0];
  LocalAcc la;

  // Units are split into up to kQueues contiguous ranges, each with its own
  // cursor; a warp starts on queue (warp id mod queues).  When its queue is
  // drained it reads every cursor at once (one round trip) and moves to the
  // next queue with units left, or stops when none has any.
  const int U = a.u_end - a.u_begin;
  const int nq = U / 256 < 1 ? 1 : (U / 256 < kQueues ? U / 256 : kQueues);
  const int gw = blockIdx.x * NW + wid;
  int q = gw % nq;
  for (;;) {
    const int qb = a.u_begin + static_cast<int>((static_cast<int64_t>(U) * q) / nq);
    const int qe = a.u_begin + static_cast<int>((static_cast<int64_t>(U) * (q + 1)) / nq);
    int u0 = 0;
    if (lane == 0) u0 = qb + static_cast<int>(atomicAdd(a.ctr + q, static_cast<unsigned>(kGrab)));
    u0 = __shfl_sync(0xffffffffu, u0, 0);
    if (u0 >= qe) {
      q = next_queue(a.ctr, q, nq, U, lane);
      if (q < 0) break;
      continue;
    }
    const int cnt = qe - u0 < kGrab ? qe - u0 : kGrab;
    // One coalesced load for the batch's descriptors.
    int2 myu = make_int2(0, 0);
    int mysh = 0;
    if (lane < cnt) {
      myu = a.units[u0 + lane];
      if (selective) mysh = a.unit_shard[u0 + lane];
    }
    // A tile's per-lane offsets, old value and out-degree are loaded one
    // unit ahead, so those loads overlap the previous unit's gathers.
    int64_t pbeg = 0, pend = 0;
    T pold = T(0);
    int32_t pod = 0;
    auto prefetch_tile = [&](int j) {
      const int px = __shfl_sync(0xffffffffu, myu.x, j), py = __shfl_sync(0xffffffffu, myu.y, j);
      if (px >= 0 && lane < py - px) {
        const int pv = px + lane;
        pbeg = a.off[pv];
        pend = a.off[pv + 1];
        pold = ASYNC ? __ldcg(static_cast<const T*>(src_val) + pv) : __ldcs(static_cast<const T*>(src_val) + pv);
        if constexpr (is_pr<APP>()) pod = __ldcs(a.outdeg + pv);
      }
    };
    if (GX_TILE_PREFETCH) prefetch_tile(0);
    for (int j = 0; j < cnt; ++j) {
      const int2 wu = make_int2(__shfl_sync(0xffffffffu, myu.x, j), __shfl_sync(0xffffffffu, myu.y, j));
      const int jsh = __shfl_sync(0xffffffffu, mysh, j);
      const bool on = !a.skip && (!selective || ((sbm[jsh >> 5] >> (jsh & 31)) & 1u));
      const int64_t cbeg = pbeg, cend = pend;
      const T cold = pold;
      const int32_t cod = pod;
      if (GX_TILE_PREFETCH && j + 1 < cnt) prefetch_tile(j + 1);
      if (wu.x < 0) {
        // ---- heavy chunk ----
        const int h = -wu.x - 1;
        const int4 H = a.heavy[h];
        const int v = H.x;
        if (!on) {
          if (wu.y == 0 && lane == 0) {
            static_cast<T*>(dst_val)[v] = static_cast<const T*>(src_val)[v];
            if constexpr (is_pr<APP>()) dst_con[v] = src_con[v];
          }
          continue;
        }
        const int64_t vb = a.off[v], ve = a.off[v + 1];
        const int64_t b = vb + static_cast<int64_t>(wu.y) * kHeavyChunk;
        const int64_t e = ve < b + kHeavyChunk ? ve : b + kHeavyChunk;
        T acc = identity<APP>();
        if constexpr (APP != K_INDEG) acc = warp_reduce_range<APP, ASYNC, COMP, HOT>(a, src_val, src_con, b, e, lane, hot);
        if (lane == 0) {
          la.edges += e - b;
          T* part = static_cast<T*>(a.partial);
          bool last = H.y == 1;
          if (!last) {
            part[H.z + wu.y] = acc;
            __threadfence();
            last = atomicAdd(a.hticket + h, 1u) == static_cast<unsigned>(H.y) - 1;
          }
          if (last) {
            __threadfence();
            const volatile T* vp = part;
            T tot = acc;
            if (H.y > 1) {
              tot = identity<APP>();
              for (int i = 0; i < H.y; ++i) tot = combine<APP>(tot, vp[H.z + i]);
              a.hticket[h] = 0;
            }
            const T old = static_cast<const T*>(src_val)[v];
            const int32_t od = is_pr<APP>() ? a.outdeg[v] : 0;
            T fin;
            if constexpr (is_pr<APP>()) fin = tot;
            else if constexpr (APP == K_INDEG) fin = static_cast<T>(ve - vb);
            else fin = combine<APP>(old, tot);
            if (apply_vertex<APP>(c, v, fin, old, od, dst_val, dst_con, la)) atomicOr(a.bm + (v >> 5), 1u << (v & 31));
          }
        }
        continue;
      }
      // ---- tile ----
      const int vb = wu.x, n = wu.y - wu.x;
      const int v = vb + lane;
      int64_t beg = 0, end = 0;
      T old = T(0);
      int32_t od = 0;
      if (GX_TILE_PREFETCH) {
        if (lane < n) {
          beg = cbeg;
          end = cend;
          old = cold;
          od = cod;
        }
      } else if (lane < n) {
        beg = a.off[v];
        end = a.off[v + 1];
        old = ASYNC ? __ldcg(static_cast<const T*>(src_val) + v) : __ldcs(static_cast<const T*>(src_val) + v);
        if constexpr (is_pr<APP>()) od = __ldcs(a.outdeg + v);
      }
      // Vertices above the heavy threshold are applied by their own units.
      const bool valid = lane < n && end - beg <= a.heavy_deg;
      if (!on) {
        if (valid) {
          static_cast<T*>(dst_val)[v] = old;
          if constexpr (is_pr<APP>()) dst_con[v] = src_con[v];
        }
        continue;
      }
      T acc;
      if constexpr (is_pr<APP>()) acc = 0.f;
      else acc = old;
      if constexpr (APP == K_INDEG) {
        acc = static_cast<T>(end - beg);
      } else {
        const bool longl = valid && end - beg > kLaneMaxDegree;
        const unsigned mlong = __ballot_sync(0xffffffffu, longl);
        if (EXACT && mlong) {
          // Stage the tile's edge range; each lane folds its own slice in order.
          const int64_t E0 = __shfl_sync(0xffffffffu, beg, 0);
          const int64_t E1 = __shfl_sync(0xffffffffu, end, n - 1);
          for (int64_t c0 = E0 & ~3ll; c0 < E1; c0 += kChunk) {
#pragma unroll
            for (int j = 0; j < kChunk / 128; ++j) {
              const int64_t q = c0 + 4 * (lane + 32 * j);
              if (q < E1) {
                const int4 c4 = load_idx4<COMP>(a, q);
                uint4 w4 = make_uint4(0, 0, 0, 0);
                if constexpr (APP == K_SSSP_W) w4 = load_w4<COMP>(a, q);
                const int cs[4] = {c4.x, c4.y, c4.z, c4.w};
                const uint32_t ws[4] = {w4.x, w4.y, w4.z, w4.w};
                T x[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                  const int64_t kk = q + e;
                  x[e] = (kk >= E0 && kk < E1) ? edge_value<APP, ASYNC, HOT>(a, src_val, src_con, cs[e], ws[e], hot)
                                                : identity<APP>();
                }
                store4(buf + 4 * (lane + 32 * j), x);
              }
            }
            __syncwarp();
            // Only a lane whose list meets the window folds: lo and hi then lie
            // in [0, kChunk] (a difference of 64-bit edge ids never reaches int).
            if (beg < c0 + kChunk && end > c0) {
              const int lo = static_cast<int>((beg > c0 ? beg : c0) - c0);
              const int hi = static_cast<int>((end < c0 + kChunk ? end : c0 + kChunk) - c0);
#pragma unroll 4
              for (int kk = lo; kk < hi; ++kk) acc = combine<APP>(acc, buf[kk]);
            }
            __syncwarp();
          }
        } else {
          // Short lists: lane per vertex, 8 edges per step, next step prefetched.
          const int64_t lend = longl ? beg : end;
          int64_t k = beg & ~3ll;
          const int steps = (valid && lend > beg) ? static_cast<int>((lend - k + 7) >> 3) : 0;
          const int smax = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(steps)));
          int4 c0v = make_int4(0, 0, 0, 0), c1v = make_int4(0, 0, 0, 0);
          uint4 w0v = make_uint4(0, 0, 0, 0), w1v = make_uint4(0, 0, 0, 0);
          if (steps > 0) {
            c0v = load_idx4<COMP>(a, k);
            if (k + 4 < lend) c1v = load_idx4<COMP>(a, k + 4);
            if constexpr (APP == K_SSSP_W) {
              w0v = load_w4<COMP>(a, k);
              if (k + 4 < lend) w1v = load_w4<COMP>(a, k + 4);
            }
          }
          for (int st = 0; st < smax; ++st) {
            if (st < steps) {
              const int cs[8] = {c0v.x, c0v.y, c0v.z, c0v.w, c1v.x, c1v.y, c1v.z, c1v.w};
              const uint32_t ws[8] = {w0v.x, w0v.y, w0v.z, w0v.w, w1v.x, w1v.y, w1v.z, w1v.w};
              const int64_t kn = k + 8;
              if (kn < lend) {
                c0v = load_idx4<COMP>(a, kn);
                if (kn + 4 < lend) c1v = load_idx4<COMP>(a, kn + 4);
                if constexpr (APP == K_SSSP_W) {
                  w0v = load_w4<COMP>(a, kn);
                  if (kn + 4 < lend) w1v = load_w4<COMP>(a, kn + 4);
                }
              }
              T vals[8];
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const int64_t kk = k + j;
                vals[j] = (kk >= beg && kk < lend) ? edge_value<APP, ASYNC, HOT>(a, src_val, src_con, cs[j], ws[j], hot)
                                                   : identity<APP>();
              }
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const int64_t kk = k + j;
                if (kk >= beg && kk < lend) acc = combine<APP>(acc, vals[j]);
              }
              k = kn;
            }
          }
          // Medium lists: several at a time, one per group of kGroupLanes lanes.
          unsigned mbig = mlong;
          if (GX_GROUP_SWEEP) {
            constexpr int NG = 32 / kGroupLanes;
            unsigned mmid = __ballot_sync(0xffffffffu, longl && end - beg <= GX_MID_MAX);
            mbig = mlong & ~mmid;
            const int grp = lane / kGroupLanes, gl = lane % kGroupLanes;
            while (mmid) {
              unsigned mm = mmid;  // group grp takes the grp-th lowest list left
              for (int i = 0; i < grp; ++i) mm &= mm - 1;
              const int l = mm ? __ffs(mm) - 1 : -1;
#pragma unroll
              for (int i = 0; i < NG; ++i) mmid &= mmid - 1;
              const int sl = l < 0 ? 0 : l;
              const int64_t bl = __shfl_sync(0xffffffffu, beg, sl);
              const int64_t el = __shfl_sync(0xffffffffu, end, sl);
              T r = identity<APP>();
              if (l >= 0) r = group_reduce_range<APP, ASYNC, COMP, HOT>(a, src_val, src_con, bl, el, gl, grp, hot);
#pragma unroll
              for (int g = 0; g < NG; ++g) {
                const int lg = __shfl_sync(0xffffffffu, l, kGroupLanes * g);
                const T rg = __shfl_sync(0xffffffffu, r, kGroupLanes * g);
                if (lane == lg) acc = combine<APP>(acc, rg);
              }
            }
          }
          // Longer lists: the whole warp sweeps each one in turn.
          for (unsigned m = mbig; m; m &= m - 1) {
            const int l = __ffs(m) - 1;
            const int64_t bl = __shfl_sync(0xffffffffu, beg, l);
            const int64_t el = __shfl_sync(0xffffffffu, end, l);
            const T r = warp_reduce_range<APP, ASYNC, COMP, HOT>(a, src_val, src_con, bl, el, lane, hot);
            if (lane == l) acc = combine<APP>(acc, r);
          }
        }
      }
      bool act = false;
      if (valid) {
        la.edges += end - beg;
        act = apply_vertex<APP>(c, v, acc, old, od, dst_val, dst_con, la);
      }
      const unsigned m = __ballot_sync(0xffffffffu, act);
      if (lane == 0) bitmap_set_tile(a.bm, vb, m);
    }
  }
  flush_block<NW>(ctl, la);
}

// ---------------------------------------------------------------------------
// Push (sparse steps of SSSP/CC): each frontier vertex u, with the value it
// held at the end of the previous step, relaxes its out-edges with atomicMin.
// For min-plus / min-label this equals the Jacobi pull of the reference:
// a vertex whose in-neighbours did not change cannot improve, so the values
// and the per-step change counts are those of a full pull.
// Frontier entries cover at most kPushChunk out-edges each (a hub is several
// entries).  A warp claims 32 entries and sweeps their concatenated edge
// ranges 32 edges at a time; each lane finds the entry that owns its edge by
// a binary search over the warp's exclusive prefix sums.
// ---------------------------------------------------------------------------
template <int APP>
__global__ void __launch_bounds__(kThreads) push_kernel(PushArgs a) {
  typedef typename AppTraits<APP>::T T;
  if (a.ctl->done || a.ctl->mode != MODE_PUSH) return;
  const int cur = a.ctl->cur;
  const int lane = threadIdx.x & 31;
  const int nf = a.ctl->n_frontier;
  LocalAcc la;
  if constexpr (!is_pr<APP>() && APP != K_INDEG) {
  T* val = static_cast<T*>(cur ? a.val[1] : a.val[0]);
  for (;;) {
    int base = 0;
    if (lane == 0) base = static_cast<int>(atomicAdd(a.ctr, 32u));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= nf) break;
    const int cnt = nf - base < 32 ? nf - base : 32;
    int d = 0;
    uint32_t su = 0;
    long long b = 0;
    if (lane < cnt) {
      const int4 f = a.frontier[base + lane];
      su = static_cast<uint32_t>(f.y);
      b = a.ooff[f.x] + f.z;
      const long long left = a.ooff[f.x + 1] - b;
      d = static_cast<int>(left < kPushChunk ? left : kPushChunk);
    }
    int incl = d;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int excl = incl - d;
    la.edges += static_cast<unsigned long long>(d);
    // 128 edges per round, four per lane, each stage's loads in flight
    // together (index and weight, then the destination's value); the value
    // read is only a filter before the atomicMin, so a stale one is harmless.
    for (int k0 = 0; k0 < total; k0 += 128) {
      long long edge[4];
      uint32_t sv[4];
      bool ok[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = k0 + 32 * u + lane;
        // Largest j with excl[j] <= k; that entry has d[j] > 0 when k < total.
        // (every lane takes part in every shuffle)
        int j = 0;
#pragma unroll
        for (int sp = 16; sp > 0; sp >>= 1) {
          const int ex = __shfl_sync(0xffffffffu, excl, j + sp);
          if (ex <= k) j += sp;
        }
        const int exj = __shfl_sync(0xffffffffu, excl, j);
        const long long bj = __shfl_sync(0xffffffffu, b, j);
        sv[u] = __shfl_sync(0xffffffffu, su, j);
        ok[u] = k < total;
        edge[u] = bj + (k - exj);
      }
      int vtx[4];
      T cand[4], now[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        vtx[u] = ok[u] ? __ldcs(a.ocol + edge[u]) : 0;
        if constexpr (APP == K_SSSP_UNIT) cand[u] = static_cast<T>(sv[u]) + 1;
        else if constexpr (APP == K_SSSP_W) cand[u] = sat_add(sv[u], ok[u] ? __ldcs(a.ow + edge[u]) : 0u);
        else cand[u] = static_cast<T>(sv[u]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) now[u] = ok[u] ? val[vtx[u]] : cand[u];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (ok[u] && cand[u] < now[u]) {
          const T prev = atomicMin(val + vtx[u], cand[u]);
          if (cand[u] < prev) {
            const uint32_t bit = 1u << (vtx[u] & 31);
            const uint32_t was = atomicOr(a.bm + (vtx[u] >> 5), bit);
            if (!(was & bit)) {
              la.changed += 1;
              la.fedges += static_cast<unsigned long long>(__ldg(a.outdeg + vtx[u]));
            }
          }
        }
      }
    }
  }
  }
  flush_block(a.ctl, la);
}

// ---------------------------------------------------------------------------
// Finalize: the host-side tail of GraphPS::run's step (GraphPS.h:291-385) on
// the device.  All CTAs sweep the next-frontier bitmap: count it, clear it,
// and — when the next step is selective — either compact it into the push
// frontier or OR the shard-group masks of its vertices into the next shard
// mask (the bloom-filter partition test of GraphPS.h:349-368, made exact per
// shard group).  The last CTA to finish records the step and advances.
// ---------------------------------------------------------------------------
template <int APP>
__global__ void __launch_bounds__(kThreads) finalize_kernel(FinArgs a) {
  typedef typename AppTraits<APP>::T T;
  __shared__ unsigned long long s_act[kWarps];
  __shared__ bool s_last;
  Ctl* ctl = a.ctl;
  const Ctl c = *ctl;
  if (c.done) return;
  // A step-0 push from the SSSP source alone stands for the reference's
  // full first pull, whose _Changed_Vertex compares against VertexValue = 0:
  // every vertex but the source ends with a non-zero distance.
  const unsigned long long changed =
      (c.step == 0 && c.step0_push) ? static_cast<unsigned long long>(c.n_vertices - 1) : c.changed;
  // updated_ratio is a float in the reference (GraphPS.h:203,297).
  const float ratio = static_cast<float>(static_cast<double>(changed) / c.n_vertices);
  const bool sel_next = static_cast<double>(ratio) < c.sel_threshold;
  // Push is exact for min apps whatever the frontier size; beyond the
  // reference's selective steps it is chosen when the frontier's out-edges
  // are few enough to beat a full pull.
  const bool push_next = c.push_ok && (sel_next || c.front_edges <= c.push_edge_limit);
  // A selective pull step sweeps only the shards its changed in-neighbours
  // reach: marked here from the out-edges (MARK_OUT), or by the host from
  // the list of changed vertices (MARK_LIST).  Without either, every shard.
  const bool mark = sel_next && !push_next &&
                    (c.mark_mode == MARK_LIST || (c.mark_mode == MARK_OUT && c.shard_bm != nullptr));
  uint32_t* next_bm = c.shard_bm ? c.shard_bm + static_cast<int64_t>(c.shard_cur ^ 1) * c.shard_words : nullptr;
  const int nb = (c.mode == MODE_PUSH || c.async_mode) ? c.cur : (c.cur ^ 1);
  const T* newv = static_cast<const T*>(nb ? a.val[1] : a.val[0]);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long act = 0;
  // Warp-uniform sweep: lane i takes word w0 + i, so the frontier compaction
  // can reserve its slots with one atomic per warp.
  for (int w0 = blockIdx.x * kThreads + (wid << 5); w0 < a.n_words; w0 += gridDim.x * kThreads) {
    const int w = w0 + lane;
    const uint32_t word = w < a.n_words ? a.bm[w] : 0u;
    if (word) {
      a.bm[w] = 0;
      act += __popc(word);
      if (mark) {
        for (uint32_t x = word; x; x &= x - 1) {
          const int u = (w << 5) + __ffs(x) - 1;
          if (c.mark_mode == MARK_OUT) {
            for (int64_t k = c.ooff[u]; k < c.ooff[u + 1]; ++k) {
              const int v = c.ocol[k];
              int lo = 0, hi = c.n_shards;  // bounds[lo] <= v < bounds[lo + 1]
              while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (__ldg(c.bounds + mid) <= v) lo = mid;
                else hi = mid;
              }
              const uint32_t bit = 1u << (lo & 31);
              if (!(next_bm[lo >> 5] & bit)) atomicOr(next_bm + (lo >> 5), bit);
            }
          } else {
            const unsigned pos = atomicAdd(&ctl->n_changed_list, 1u);
            if (pos < c.changed_cap) c.changed_list[pos] = u;
            else ctl->list_overflow = 1;
          }
        }
      }
    }
    if (push_next) {
      unsigned n_ent = 0;
      for (uint32_t x = word; x; x &= x - 1) {
        const int od = __ldg(a.outdeg + (w << 5) + __ffs(x) - 1);
        n_ent += static_cast<unsigned>((od + kPushChunk - 1) / kPushChunk);  // sinks need no entry
      }
      unsigned incl = n_ent;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      const unsigned tot = __shfl_sync(0xffffffffu, incl, 31);
      if (tot) {
        unsigned wbase = 0;
        if (lane == 31) wbase = atomicAdd(&ctl->next_frontier, tot);
        wbase = __shfl_sync(0xffffffffu, wbase, 31);
        unsigned long long pos = static_cast<unsigned long long>(wbase) + (incl - n_ent);
        for (uint32_t x = word; x; x &= x - 1) {
          const int u = (w << 5) + __ffs(x) - 1;
          const int od = __ldg(a.outdeg + u);
          T vu = newv[u];
          const int bits = *reinterpret_cast<int*>(&vu);
          for (int k = 0; k < od; k += kPushChunk, ++pos) {
            if (pos < a.frontier_cap) a.frontier[pos] = make_int4(u, bits, k, 0);
            else ctl->error = 2;
          }
        }
      }
    }
  }
  act = warp_sum(act);
  if (lane == 0) s_act[wid] = act;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long ta = 0;
    for (int i = 0; i < kWarps; ++i) ta += s_act[i];
    if (ta) atomicAdd(&ctl->active, ta);
    __threadfence();
    const unsigned ticket = atomicAdd(&ctl->fin_ticket, 1u);
    s_last = ticket == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (threadIdx.x == 0) {
    volatile Ctl* vc = ctl;
    StepStats s;
    s.changed = changed;
    s.active = vc->active;
    s.edges = vc->edges;
    s.resid_fx = vc->resid_fx;
    s.dangl_fx = vc->dangl_fx;
    s.mode = c.mode;
    s.shards_active = -1;  // every shard (the host counts MARK_LIST steps)
    if (c.mode == MODE_SELECTIVE && c.shard_valid) {
      const uint32_t* cur_bm = c.shard_bm + static_cast<int64_t>(c.shard_cur) * c.shard_words;
      int n = 0;
      for (int i = 0; i < c.shard_words; ++i) n += __popc(cur_bm[i]);
      s.shards_active = n;
    }
    a.stats[c.step] = s;
    const double resid = static_cast<double>(s.resid_fx) / c.fx_scale;
    int done = (s.changed == 0 && c.step > 1) || (c.step + 1 >= c.max_iter);  // GraphPS.h:256,383
    if (is_pr<APP>() && c.tolerance > 0 && resid < c.tolerance) done = 1;
    ctl->cur = nb;  // Msg <- MsgNew as a swap (in place: push steps, async mode)
    ctl->mode = push_next ? MODE_PUSH : (sel_next ? MODE_SELECTIVE : MODE_DENSE);
    if (c.mark_mode == MARK_OUT) {
      ctl->shard_valid = mark;
      if (mark) ctl->shard_cur = c.shard_cur ^ 1;
    }
    ctl->n_frontier = static_cast<int>(vc->next_frontier);
    ctl->next_frontier = 0;
    ctl->front_edges = 0;
    if (APP == K_PR_STD) {
      const double D = static_cast<double>(s.dangl_fx) / c.fx_scale;
      ctl->base = (1.0 - c.damping) * c.inv_n + c.damping * D * c.inv_n;
    }
    ctl->changed = 0;
    ctl->active = 0;
    ctl->edges = 0;
    ctl->resid_fx = 0;
    ctl->dangl_fx = 0;
    ctl->fin_ticket = 0;
    ctl->step = c.step + 1;
    __threadfence();
    ctl->done = done;
  }
  for (int i = threadIdx.x; i < a.n_work_ctr; i += kThreads) a.work_ctr[i] = 0;
  // The bitmap the next finalize marks into starts empty.
  if (c.mark_mode == MARK_OUT && mark) {
    uint32_t* old_bm = c.shard_bm + static_cast<int64_t>(c.shard_cur) * c.shard_words;
    for (int i = threadIdx.x; i < c.shard_words; i += kThreads) old_bm[i] = 0;
  }
}

// Initial values (init_vertex of each app) and PageRank contributions.
// label (nullable): CC's start label of each vertex, its id as the caller
// numbered it (a relabelled engine), else the vertex's own index.
template <int APP>
__global__ void init_kernel(Ctl* ctl, void* val, float* con, const int32_t* outdeg, int n, int source, int use_init,
                            const int32_t* label = nullptr) {
  typedef typename AppTraits<APP>::T T;
  T* v = static_cast<T*>(val);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!use_init) {
      if constexpr (is_pr<APP>()) v[i] = static_cast<float>(ctl->inv_n);  // assign(V, 1.0/V), pagerank.cpp:81
      else if constexpr (APP == K_SSSP_UNIT) v[i] = i == source ? 0 : kGpsInf;  // sssp.cpp:70-72
      else if constexpr (APP == K_SSSP_W) v[i] = i == source ? 0u : kInfW;
      else if constexpr (APP == K_CC) v[i] = label ? label[i] : i;  // cc.cpp:70-73
      else v[i] = 0;  // cal.cpp:77
    }
    if constexpr (is_pr<APP>()) {
      const int32_t od = outdeg[i];
      con[i] = v[i] / static_cast<float>(od > 0 ? od : 1);
    }
  }
}

// Load-time checks before any kernel indexes with the data: bit 0 set when
// off decreases somewhere, bit 1 when a source id lies outside [0, V).
static __global__ void validate_csc_kernel(const int64_t* off, int32_t V, const int32_t* col, int64_t E,
                                           unsigned int* flag) {
  const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t nt = static_cast<int64_t>(gridDim.x) * blockDim.x;
  unsigned int f = 0;
  for (int64_t v = tid; v < V; v += nt) f |= off[v] > off[v + 1] ? 1u : 0u;
  if (col)
    for (int64_t k = tid; k < E; k += nt) f |= (col[k] < 0 || col[k] >= V) ? 2u : 0u;
  if (f) atomicOr(flag, f);
}

// Relabelling, on the device at load.  The order: within each shard, the
// vertices by descending in-degree (capped at 4095), ties by ascending id.
// relabel_keys_kernel writes the sort key of every vertex, its shard and
// degree rank above `vb` bits of vertex id; a stable sort of those upper
// bits leaves the keys in the new order.  A length is taken as 0 where off
// decreases (the load reports that separately).
static __global__ void relabel_keys_kernel(const int64_t* off, const int32_t* bounds, int32_t P, int32_t V, int vb,
                                           unsigned long long* keys) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    int32_t lo = 0, hi = P;  // the shard p with bounds[p] <= v < bounds[p + 1]
    while (hi - lo > 1) {
      const int32_t mid = (lo + hi) >> 1;
      if (bounds[mid] <= v) lo = mid;
      else hi = mid;
    }
    const int64_t d = off[v + 1] - off[v];
    const unsigned long long rank = 4095u - static_cast<unsigned>(d < 0 ? 0 : d > 4095 ? 4095 : d);
    keys[v] = ((static_cast<unsigned long long>(lo) << 12 | rank) << vb) | static_cast<unsigned long long>(v);
  }
}

// From the sorted keys: inv[i] (the old id of new vertex i), perm (its
// inverse), the out-degree and the in-list length of every new vertex.
static __global__ void relabel_order_kernel(const unsigned long long* sorted, unsigned long long vmask, int32_t V,
                                            const int64_t* off_old, const int32_t* outdeg_old, int32_t* inv,
                                            int32_t* perm, int32_t* outdeg_new, uint32_t* len_new) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x) {
    const int32_t v = static_cast<int32_t>(sorted[i] & vmask);
    inv[i] = v;
    perm[v] = i;
    outdeg_new[i] = outdeg_old[v];
    const int64_t d = off_old[v + 1] - off_old[v];
    len_new[i] = static_cast<uint32_t>(d < 0 ? 0 : d);
  }
}

// Moves per-edge data from the caller's layout to the engine's: new vertex
// i (old vertex inv[i]) gets the old list src[off_old[v], off_old[v+1]) at
// off_new[i], in order, with every entry renamed through `rename` (source
// ids) or copied (rename null: weights).  A warp takes 32 consecutive new
// vertices, whose lists lie end to end in the new layout, and moves their
// entries 128 at a time, four per lane with the loads in flight together;
// each lane finds the list of its entry by a binary search over the lanes'
// running entry counts.  Lists longer than max_len go to `longs` for
// relabel_scatter_long_kernel, so that no warp is left with a shard's
// heaviest lists (the relabelling puts them side by side).  A warp whose
// lists have offsets that leave [0, E] or decrease writes nothing (flag bit
// 0), and out-of-range ids are written as 0 (flag bit 1), so a malformed CSC
// neither reads nor writes out of bounds.
__device__ __forceinline__ int32_t relabel_rename(int32_t x, const int32_t* rename, int32_t V, unsigned int& f) {
  if (!rename) return x;
  if (x < 0 || x >= V) {
    f |= 2u;
    return 0;
  }
  return rename[x];
}
static __global__ void relabel_scatter_kernel(const int64_t* off_old, const int32_t* src, const int64_t* off_new,
                                              const int32_t* inv, const int32_t* rename, int32_t V, int64_t E,
                                              int64_t max_len, int32_t* dst, int32_t* longs,
                                              unsigned int longs_cap, unsigned int* n_longs, unsigned int* flag) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  unsigned int f = 0;
  for (int64_t i0 = ((static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) * 32; i0 < V;
       i0 += warps * 32) {
    const int64_t i = i0 + lane;
    int64_t b0 = 0, n = 0, b1 = 0;
    bool ok = true;
    if (i < V) {
      const int32_t v = inv[i];
      b0 = off_old[v];
      const int64_t e0 = off_old[v + 1];
      b1 = off_new[i];
      n = e0 - b0;
      ok = b0 >= 0 && e0 >= b0 && e0 <= E && b1 >= 0 && b1 + n <= E;
    }
    if (__any_sync(0xffffffffu, !ok)) {
      f |= 1u;
      continue;
    }
    if (n > max_len) {
      const unsigned int at = atomicAdd(n_longs, 1u);
      if (at < longs_cap) longs[at] = static_cast<int32_t>(i);
      else f |= 1u;  // more long lists than E allows: overlapping lists
    }
    const int64_t eff = n > max_len ? 0 : n;
    int64_t pre = eff;  // inclusive scan over the lanes, then exclusive
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, pre, o);
      if (lane >= o) pre += t;
    }
    const int64_t tot = __shfl_sync(0xffffffffu, pre, 31);
    pre -= eff;
    for (int64_t q0 = 0; q0 < tot; q0 += 128) {
      int64_t sk[4], dk[4];
      int32_t x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t q = q0 + 32 * u + lane;
        int l = 0;  // the last lane whose entries start at or before q
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          const int64_t b = __shfl_sync(0xffffffffu, pre, l + step);
          if (b <= q) l += step;
        }
        // (every lane takes part in every shuffle)
        const int64_t lp = __shfl_sync(0xffffffffu, pre, l);
        const int64_t lb0 = __shfl_sync(0xffffffffu, b0, l);
        const int64_t lb1 = __shfl_sync(0xffffffffu, b1, l);
        sk[u] = lb0 + (q - lp);
        dk[u] = q < tot ? lb1 + (q - lp) : -1;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = dk[u] >= 0 ? src[sk[u]] : 0;
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = dk[u] >= 0 ? relabel_rename(x[u], rename, V, f) : 0;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (dk[u] >= 0) dst[dk[u]] = x[u];
    }
  }
  if (f) atomicOr(flag, f);
}
// A CTA per long list, four entries per thread in flight.
static __global__ void relabel_scatter_long_kernel(const int64_t* off_old, const int32_t* src, const int64_t* off_new,
                                                   const int32_t* inv, const int32_t* rename, int32_t V,
                                                   int32_t* dst, const int32_t* longs, unsigned int longs_cap,
                                                   const unsigned int* n_longs, unsigned int* flag) {
  unsigned int f = 0;
  const unsigned int n_l = *n_longs < longs_cap ? *n_longs : longs_cap;
  for (unsigned int l = blockIdx.x; l < n_l; l += gridDim.x) {
    const int32_t i = longs[l];  // offsets checked by relabel_scatter_kernel
    const int32_t v = inv[i];
    const int64_t b0 = off_old[v], n = off_old[v + 1] - b0, b1 = off_new[i];
    const int64_t span = 4 * static_cast<int64_t>(blockDim.x);
    for (int64_t j0 = 0; j0 < n; j0 += span) {
      int32_t x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t j = j0 + u * blockDim.x + threadIdx.x;
        x[u] = j < n ? src[b0 + j] : 0;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t j = j0 + u * blockDim.x + threadIdx.x;
        if (j < n) x[u] = relabel_rename(x[u], rename, V, f);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t j = j0 + u * blockDim.x + threadIdx.x;
        if (j < n) dst[b1 + j] = x[u];
      }
    }
  }
  if (f) atomicOr(flag, f);
}

// out[v] = in[perm[v]] (values to the caller's numbering), and the inverse.
static __global__ void gather_values_kernel(const uint32_t* in, const int32_t* perm, int32_t V, uint32_t* out) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) out[v] = in[perm[v]];
}
static __global__ void scatter_values_kernel(const uint32_t* in, const int32_t* perm, int32_t V, uint32_t* out) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) out[perm[v]] = in[v];
}

// Out-edge CSR from the CSC (counting sort by source; order within a source
// is unspecified, which min-plus / min-label do not observe).
static __global__ void transpose_kernel(const int64_t* off, const int32_t* col, const uint32_t* w, int n,
                                 unsigned long long* cursor, int32_t* ocol, uint32_t* ow) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
    for (int64_t k = off[v] + lane; k < off[v + 1]; k += 32) {
      const int u = col[k];
      const unsigned long long p = atomicAdd(cursor + u, 1ull);
      ocol[p] = v;
      if (w) ow[p] = w[k];
    }
  }
}

}  // namespace gx

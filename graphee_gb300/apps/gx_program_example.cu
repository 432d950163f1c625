// Vertex programs plugged into the engine from outside the library, through
// include/gx_program.cuh: three of the reference's apps re-expressed as
// plug-ins, and one program the engine does not ship.  An application adds
// its own program the same way the reference's apps hand GraphPS<T> a _comp
// function (GraphMP/system/GraphPS.h:25-34): one struct of device functions,
// compiled in its own .cu file against the installed headers and libgx.so.
#include <climits>
#include <cstdint>

#include "gx_program.cuh"

namespace {

// comp_cc (GraphMP/app/cc.cpp:40-45): min label over in-neighbours, l[v] = v at start.
struct MinLabel {
  typedef int32_t T;
  __device__ static T init(int32_t v, int32_t) { return v; }
  __device__ static T identity() { return INT_MAX; }
  __device__ static T gather(T s, int32_t, uint32_t) { return s; }
  __device__ static T combine(T a, T b) { return b < a ? b : a; }
  __device__ static T apply(int32_t, T acc, T old, int32_t, int32_t) { return acc < old ? acc : old; }
};

// comp_sssp (GraphMP/app/sssp.cpp:40-47) from vertex 0: unit weights, INF = GPS_INF.
struct HopsFromZero {
  typedef int32_t T;
  __device__ static T init(int32_t v, int32_t) { return v == 0 ? 0 : 10000; }
  __device__ static T identity() { return INT_MAX; }
  __device__ static T gather(T s, int32_t, uint32_t) { return s + 1; }
  __device__ static T combine(T a, T b) { return b < a ? b : a; }
  __device__ static T apply(int32_t, T acc, T old, int32_t, int32_t) { return acc < old ? acc : old; }
};

// comp_pagerank (GraphMP/app/pagerank.cpp:42-48): out-degree clamped to 1,
// new = (float)((double)acc * 0.85 + 1.0 / N).
struct PageRank {
  typedef float T;
  __device__ static T init(int32_t, int32_t V) { return static_cast<float>(1.0 / V); }
  __device__ static T identity() { return 0.f; }
  __device__ static T gather(T s, int32_t od, uint32_t) { return s / static_cast<float>(od > 0 ? od : 1); }
  __device__ static T combine(T a, T b) { return a + b; }
  __device__ static T apply(int32_t, T acc, T, int32_t, int32_t V) {
    return static_cast<float>(__dadd_rn(__dmul_rn(static_cast<double>(acc), 0.85), 1.0 / V));
  }
};

// Not in the engine: the widest (maximum-bottleneck) path from vertex 0 over
// the edge weights, 0 where vertex 0 cannot reach.
struct WidestFromZero {
  typedef uint32_t T;
  __device__ static T init(int32_t v, int32_t) { return v == 0 ? 0xFFFFFFFFu : 0u; }
  __device__ static T identity() { return 0u; }
  __device__ static T gather(T s, int32_t, uint32_t w) { return s < w ? s : w; }
  __device__ static T combine(T a, T b) { return b > a ? b : a; }
  __device__ static T apply(int32_t, T acc, T old, int32_t, int32_t) { return acc > old ? acc : old; }
};

}  // namespace

// which: 0 MinLabel, 1 HopsFromZero, 2 PageRank, 3 WidestFromZero.
extern "C" gx_status gx_example_program(gx_engine* e, int32_t which, int32_t max_iter, void* host_out,
                                        int64_t* changed_out, int32_t* steps_out) {
  switch (which) {
    case 0: return gx::run_program<MinLabel>(e, max_iter, static_cast<int32_t*>(host_out), changed_out, steps_out);
    case 1: return gx::run_program<HopsFromZero>(e, max_iter, static_cast<int32_t*>(host_out), changed_out, steps_out);
    case 2: return gx::run_program<PageRank>(e, max_iter, static_cast<float*>(host_out), changed_out, steps_out);
    case 3: return gx::run_program<WidestFromZero>(e, max_iter, static_cast<uint32_t*>(host_out), changed_out,
                                                   steps_out);
  }
  return GX_ERR_INVALID;
}

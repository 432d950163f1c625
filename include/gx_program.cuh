/*
 * gx_program.cuh — user vertex programs on the engine's graph.
 *
 * The reference lets an app plug any vertex program into its engine:
 * GraphPS<T> calls the function pointer _comp once per partition with the
 * vertex arrays (GraphMP/system/GraphPS.h:25-34), after the app's
 * init_vertex() override set the start values (GraphPS.h:60).  This header
 * is that plug-in point for CUDA code: a program is a struct of device
 * functions, compiled into the caller's own .cu file, and
 * gx::run_program<Program>() runs the reference's superstep loop
 * (GraphPS.h:256-386: Jacobi pull supersteps, `changed == 0 && step > 1`
 * or max_iter to stop) over the graph a gx_engine holds in device memory
 * (gx_get_device_graph).  The engine's own apps (PageRank, SSSP, CC) keep
 * their tuned kernels; a user program runs this generic one.
 *
 *   struct MyProgram {
 *     typedef float T;                                     // any 4-byte type
 *     __device__ static T init(int32_t v, int32_t V);      // init_vertex()
 *     __device__ static T identity();                      // neutral element of combine
 *     __device__ static T gather(T src_value, int32_t src_outdeg, uint32_t weight);
 *                                                          // what in-edge (src -> v) offers v
 *     __device__ static T combine(T a, T b);               // associative and commutative
 *     __device__ static T apply(int32_t v, T acc, T old, int32_t step, int32_t V);
 *                                                          // v's new value from the combined
 *                                                          // in-edges and its old value
 *   };
 *
 * Each superstep computes new[v] = apply(v, combine over in-edges (u -> v)
 * of gather(old[u], outdeg[u], w(u, v)), old[v], step, V) for every v and
 * counts the reference's _Changed_Vertex: new[v] != VertexValue[v], where
 * VertexValue is 0 before the first step and the previous value after
 * (GraphMP/app/pagerank.cpp:56-59).  The combine order within a vertex is a
 * fixed tree over the warp's lanes, so results are deterministic; a sum in
 * floating point therefore rounds differently from the reference's
 * sequential loop (within the engine's PageRank tolerance on R-MAT graphs).
 * Weights are 0 when the engine has none.
 */
#ifndef GX_PROGRAM_CUH_
#define GX_PROGRAM_CUH_

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "gx.h"

namespace gx {
namespace program {

constexpr int kThreads = 256;
constexpr int kVertsPerClaim = 32;  // vertices a warp claims per counter atomic

template <class P>
__global__ void init_kernel(typename P::T* val, int32_t V) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) val[v] = P::init(v, V);
}

// One superstep: warps claim batches of vertices; a warp folds one vertex's
// in-edges at a time, each lane four edges per round with the loads in flight
// together, then a fixed xor tree.
template <class P>
__global__ void __launch_bounds__(kThreads) step_kernel(gx_device_graph g, const typename P::T* src,
                                                        typename P::T* dst, int32_t step,
                                                        unsigned int* claim, unsigned long long* changed) {
  typedef typename P::T T;
  const int lane = threadIdx.x & 31;
  unsigned long long mine = 0;
  for (;;) {
    int32_t v0 = 0;
    if (lane == 0) v0 = static_cast<int32_t>(atomicAdd(claim, static_cast<unsigned>(kVertsPerClaim)));
    v0 = __shfl_sync(0xffffffffu, v0, 0);
    if (v0 >= g.V) break;
    const int32_t v1 = v0 + kVertsPerClaim < g.V ? v0 + kVertsPerClaim : g.V;
    for (int32_t v = v0; v < v1; ++v) {
      const int64_t b = g.off[v], e = g.off[v + 1];
      T acc = P::identity();
      for (int64_t k = b + lane; k < e; k += 128) {
        T x[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int64_t kk = k + 32 * j;
          if (kk < e) {
            const int32_t u = g.col[kk];
            x[j] = P::gather(src[u], g.outdeg[u], g.w ? g.w[kk] : 0u);
          } else {
            x[j] = P::identity();
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) acc = P::combine(acc, x[j]);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        T y = acc;
        uint32_t bits;
        memcpy(&bits, &y, 4);
        bits = __shfl_xor_sync(0xffffffffu, bits, o);
        memcpy(&y, &bits, 4);
        acc = P::combine(acc, y);
      }
      if (lane == 0) {
        const T old = src[v];
        const T nv = P::apply(v, acc, old, step, g.V);
        dst[v] = nv;
        const T prev = step == 0 ? T(0) : old;
        mine += nv != prev;
      }
    }
  }
  if (lane == 0 && mine) atomicAdd(changed, mine);
}

}  // namespace program

// Runs program P over the engine's resident graph for up to max_iter
// supersteps with GraphPS::run's stop rule.  host_out (nullable) receives
// the final values (T[V]); changed_out (nullable, max_iter entries) the
// per-step _Changed_Vertex; *steps_out (nullable) the supersteps run.
// Device memory: two value buffers and a few counters, allocated here.
template <class P>
gx_status run_program(gx_engine* e, int32_t max_iter, typename P::T* host_out, int64_t* changed_out,
                      int32_t* steps_out) {
  typedef typename P::T T;
  static_assert(sizeof(T) == 4, "vertex values are 4 bytes");
  gx_device_graph g;
  gx_status st = gx_get_device_graph(e, &g);
  if (st != GX_OK) return st;
  if (max_iter < 0) return GX_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(g.stream);
  T* val[2] = {nullptr, nullptr};
  unsigned int* claim = nullptr;
  unsigned long long* changed = nullptr;
  auto cleanup = [&]() {
    cudaFree(val[0]);
    cudaFree(val[1]);
    cudaFree(claim);
    cudaFree(changed);
  };
  if (cudaMalloc(&val[0], sizeof(T) * g.V) != cudaSuccess || cudaMalloc(&val[1], sizeof(T) * g.V) != cudaSuccess ||
      cudaMalloc(&claim, sizeof(unsigned int) * (max_iter > 0 ? max_iter : 1)) != cudaSuccess ||
      cudaMalloc(&changed, sizeof(unsigned long long) * (max_iter > 0 ? max_iter : 1)) != cudaSuccess) {
    cleanup();
    return GX_ERR_OOM;
  }
  int dev = 0, n_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const int grid = n_sm * 8;
  program::init_kernel<P><<<grid, program::kThreads, 0, s>>>(val[0], g.V);
  cudaMemsetAsync(claim, 0, sizeof(unsigned int) * (max_iter > 0 ? max_iter : 1), s);
  cudaMemsetAsync(changed, 0, sizeof(unsigned long long) * (max_iter > 0 ? max_iter : 1), s);
  int cur = 0, step = 0;
  for (; step < max_iter; ++step) {
    program::step_kernel<P><<<grid, program::kThreads, 0, s>>>(g, val[cur], val[cur ^ 1], step, claim + step,
                                                                changed + step);
    unsigned long long c = 0;
    cudaMemcpyAsync(&c, changed + step, sizeof(c), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      cleanup();
      return GX_ERR_CUDA;
    }
    cur ^= 1;  // Msg <- MsgNew (GraphPS.h:338-345)
    if (changed_out) changed_out[step] = static_cast<int64_t>(c);
    if (c == 0 && step > 1) {  // GraphPS.h:383
      ++step;
      break;
    }
  }
  cudaError_t err = cudaSuccess;
  if (host_out) err = cudaMemcpyAsync(host_out, val[cur], sizeof(T) * g.V, cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  cleanup();
  if (err != cudaSuccess) return GX_ERR_CUDA;
  if (steps_out) *steps_out = step;
  return GX_OK;
}

}  // namespace gx

#endif  // GX_PROGRAM_CUH_

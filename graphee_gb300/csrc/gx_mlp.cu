// Learned PageRank warm start: a 6 -> 64 -> 64 -> 1 MLP (GELU, tanh form, hidden
// layers, softplus output normalised to sum 1) predicts initial ranks from
// per-vertex degree features; standard PageRank (GX_APP_PAGERANK_STD) then
// runs from that start to the L1 residual tolerance, and falls back to the
// uniform start when the warm start's first-step residual is worse than the
// uniform start's.  No reference counterpart.
//
// Features of v (one pull pass over in-edges, 8-byte gather per edge):
//   log1p(indeg v), log1p(outdeg v), mean and max over in-neighbours u of
//   log1p(outdeg u), log1p(sum over in-neighbours of indeg u), [outdeg v == 0].
// The same pass accumulates sum 1/outdeg(u), which gives the uniform start's
// first-step residual for free.
//
// Training target: t_v = log(N * r_v) of converged standard PageRank; the
// network's per-vertex output y_v = log softplus(z_v) is fitted to t_v in
// squared error weighted by min(N * r_v, 100), so the normalised softplus
// output approximates r where the L1 error lives.
// Weights: FP32 master copy updated by Adam; every forward pass (training
// and inference) uses the weights rounded to BF16, with FP32 accumulation.
// Inference runs on the tensor cores (mma.sync m16n8k16 in f16, in which a
// BF16-rounded weight is exact when its magnitude lies in [2^-17, 65504];
// smaller ones land on f16's subnormal grid, an error below 2^-25, and larger
// ones are clamped to 65504; each layer's accumulators re-packed in
// registers as the next layer's A fragments, GELUs on packed f16 pairs,
// layer 3 as an MMA against the w3 column); training runs
// hand-written FP32 forward/backward kernels whose per-CTA weight gradients
// are summed in CTA order, so training is deterministic.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <vector>

#include "gx_engine.h"
#include "gx_nvtx.h"

using namespace gx;

namespace {

constexpr int kH = 64;
constexpr int kF = 6;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kH * kF, kOffW2 = kOffB1 + kH, kOffB2 = kOffW2 + kH * kH,
              kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kH, kNumParams = kOffB3 + 1;  // 4673
constexpr int kFeatStride = 8;
constexpr int kTrainSamples = 128;   // samples per training CTA
constexpr int kTrainThreads = 256;
constexpr int kPartStride = kNumParams + 3;  // gradient partial + loss
constexpr float kLossWeightCap = 100.f;

// GELU in its tanh form, 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))):
// training uses tanhf in FP32, inference the hardware tanh.approx.f16x2 on
// packed pairs (gelu_h2).
constexpr float kGeluC = 0.7978845608028654f;  // sqrt(2/pi)
constexpr float kGeluA = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.f + tanhf(kGeluC * (x + kGeluA * x * x * x)));
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float t = tanhf(kGeluC * (x + kGeluA * x * x * x));
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * kGeluC * (1.f + 3.f * kGeluA * x * x);
}
__device__ __forceinline__ float softplus(float z) { return z > 20.f ? z : log1pf(expf(z)); }
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Per-vertex data gathered once per in-edge by the feature pass (8 bytes):
// log1p(outdeg) and 1/max(outdeg,1) as halves (finer than the BF16 the
// network sees), in-degree as a float (exact below 2^24).
struct __align__(8) NbrInfo {
  __half2 lo_inv;
  float indeg;
};

__global__ void mlp_nbr_kernel(const int64_t* off, const int32_t* outdeg, int32_t V, NbrInfo* nb) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int32_t od = outdeg[v];
    NbrInfo x;
    x.lo_inv = __floats2half2_rn(log1pf(static_cast<float>(od)), 1.f / static_cast<float>(od > 0 ? od : 1));
    x.indeg = static_cast<float>(off[v + 1] - off[v]);
    nb[v] = x;
  }
}

// Accumulators of one vertex's feature pass.
struct FeatAcc {
  float sum_g = 0.f, max_g = 0.f, sum_inv = 0.f, sum_in = 0.f;
  __device__ __forceinline__ void add(const NbrInfo& x) {
    const float2 li = __half22float2(x.lo_inv);
    sum_g += li.x;
    max_g = fmaxf(max_g, li.x);
    sum_in += x.indeg;
    sum_inv += li.y;
  }
};

// Features, plus each CTA's share of the uniform start's first-step L1
// residual sum |r1 - 1/N| (standard PageRank).  Tiles of 32 consecutive
// vertices: a lane walks a list of up to 32 edges with 128-bit index loads
// (the next one prefetched) and 4 gathers in flight; longer lists are swept
// by the whole warp.
__global__ void __launch_bounds__(256, 3) mlp_features_kernel(const int64_t* off, const int32_t* col,
                                                           const int32_t* outdeg, const NbrInfo* nb, int32_t V,
                                                           const int2* units, int32_t n_units, unsigned int* cursor,
                                                           int64_t heavy_deg, double damping, double dangling0,
                                                           float* feat, double* part_resid) {
  __shared__ double s_red[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // Per-vertex arithmetic is FP32 (FP64 is slow on this part): the uniform
  // start's first-step residual term |r1 - 1/N| = d/N |sum_inv + D - 1| is
  // summed per thread in FP32 (a few hundred terms) and across threads in FP64.
  const float invn_f = static_cast<float>(1.0 / V), d_f = static_cast<float>(damping);
  const float dang_f = static_cast<float>(dangling0);
  float resid_f = 0.f;
  // The engine's work units (edge-capped tiles of consecutive vertices),
  // claimed dynamically; heavy chunks belong to mlp_heavy_features_kernel.
  for (int u = 0;; ++u) {
    if ((u & 3) == 0) {  // claim four units per atomic
      int c = 0;
      if (lane == 0) c = static_cast<int>(atomicAdd(cursor, 4u));
      u = __shfl_sync(0xffffffffu, c, 0);
    }
    if (u >= n_units) break;
    const int2 wu = units[u];
    if (wu.x < 0) continue;
    const int v = wu.x + lane;
    const bool valid = v < wu.y;
    int64_t beg = 0, end = 0;
    if (valid) {
      beg = off[v];
      end = off[v + 1];
    }
    // Lists above heavy_deg belong to mlp_heavy_features_kernel.
    const bool mine = valid && end - beg <= heavy_deg;
    FeatAcc f;
    const bool longl = mine && end - beg > 32;
    if (mine && !longl) {
      int64_t k = beg & ~3ll;
      int4 c0 = make_int4(0, 0, 0, 0);
      if (k < end) c0 = *reinterpret_cast<const int4*>(col + k);
      for (; k < end; k += 4) {
        const int cs[4] = {c0.x, c0.y, c0.z, c0.w};
        if (k + 4 < end) c0 = *reinterpret_cast<const int4*>(col + k + 4);  // next step's indices
        NbrInfo x[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (k + j >= beg && k + j < end) x[j] = nb[cs[j]];
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (k + j >= beg && k + j < end) f.add(x[j]);
      }
    }
    for (unsigned m = __ballot_sync(0xffffffffu, longl); m; m &= m - 1) {
      const int l = __ffs(m) - 1;
      const int64_t bl = __shfl_sync(0xffffffffu, beg, l), el = __shfl_sync(0xffffffffu, end, l);
      FeatAcc g;
      for (int64_t k0 = bl + lane; k0 < el; k0 += 128) {
        NbrInfo x[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (k0 + 32 * j < el) x[j] = nb[col[k0 + 32 * j]];
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (k0 + 32 * j < el) g.add(x[j]);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        g.sum_g += __shfl_xor_sync(0xffffffffu, g.sum_g, o);
        g.max_g = fmaxf(g.max_g, __shfl_xor_sync(0xffffffffu, g.max_g, o));
        g.sum_in += __shfl_xor_sync(0xffffffffu, g.sum_in, o);
        g.sum_inv += __shfl_xor_sync(0xffffffffu, g.sum_inv, o);
      }
      if (lane == l) f = g;
    }
    if (mine) {
      const float deg = static_cast<float>(end - beg);
      const int32_t od = outdeg[v];
      float4* fo = reinterpret_cast<float4*>(feat + static_cast<size_t>(v) * kFeatStride);
      fo[0] = make_float4(log1pf(deg), log1pf(static_cast<float>(od)), deg > 0 ? f.sum_g / deg : 0.f, f.max_g);
      fo[1] = make_float4(log1pf(f.sum_in), od == 0 ? 1.f : 0.f, 0.f, 0.f);
      resid_f += d_f * invn_f * fabsf(f.sum_inv + dang_f - 1.f);
    }
  }
  double resid = resid_f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) resid += __shfl_xor_sync(0xffffffffu, resid, o);
  if (lane == 0) s_red[wid] = resid;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int i = 0; i < (blockDim.x >> 5); ++i) t += s_red[i];
    part_resid[blockIdx.x] = t;
  }
}

// Features of the vertices above the heavy threshold: a CTA per vertex,
// per-thread partials combined in a fixed order; writes the vertex's share
// of the uniform first-step residual to part_resid[i].
__global__ void __launch_bounds__(256) mlp_heavy_features_kernel(const int64_t* off, const int32_t* col,
                                                                 const int32_t* outdeg, const NbrInfo* nb,
                                                                 const int4* heavy, int32_t n_heavy, int32_t V,
                                                                 double damping, double dangling0, float* feat,
                                                                 double* part_resid) {
  __shared__ float s_g[8], s_m[8], s_i[8], s_n[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = blockIdx.x; i < n_heavy; i += gridDim.x) {
    const int v = heavy[i].x;
    const int64_t beg = off[v], end = off[v + 1];
    FeatAcc g;
    for (int64_t k0 = beg + threadIdx.x; k0 < end; k0 += 4 * 256) {
      NbrInfo x[4];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (k0 + 256 * j < end) x[j] = nb[col[k0 + 256 * j]];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (k0 + 256 * j < end) g.add(x[j]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      g.sum_g += __shfl_xor_sync(0xffffffffu, g.sum_g, o);
      g.max_g = fmaxf(g.max_g, __shfl_xor_sync(0xffffffffu, g.max_g, o));
      g.sum_in += __shfl_xor_sync(0xffffffffu, g.sum_in, o);
      g.sum_inv += __shfl_xor_sync(0xffffffffu, g.sum_inv, o);
    }
    if (lane == 0) {
      s_g[wid] = g.sum_g;
      s_m[wid] = g.max_g;
      s_i[wid] = g.sum_inv;
      s_n[wid] = g.sum_in;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      FeatAcc f;
      for (int w = 0; w < 8; ++w) {
        f.sum_g += s_g[w];
        f.max_g = fmaxf(f.max_g, s_m[w]);
        f.sum_inv += s_i[w];
        f.sum_in += s_n[w];
      }
      const float deg = static_cast<float>(end - beg);
      const int32_t od = outdeg[v];
      float4* fo = reinterpret_cast<float4*>(feat + static_cast<size_t>(v) * kFeatStride);
      fo[0] = make_float4(log1pf(deg), log1pf(static_cast<float>(od)), deg > 0 ? f.sum_g / deg : 0.f, f.max_g);
      fo[1] = make_float4(log1pf(f.sum_in), od == 0 ? 1.f : 0.f, 0.f, 0.f);
      const double invn = 1.0 / V;
      part_resid[i] = damping * invn * fabs(static_cast<double>(f.sum_inv) + dangling0 - 1.0);
    }
    __syncthreads();
  }
}

// A BF16-rounded weight as an f16 operand: exact for magnitudes in
// [2^-17, 65504] (BF16's 8 significant bits fit f16's subnormal grid down to
// 2^-17), rounded below that, clamped above it.
__device__ __forceinline__ __half half_weight(float w) {
  return __float2half_rn(fminf(fmaxf(bf16r(w), -65504.f), 65504.f));
}

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
  const __half2 h = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ void mma_f16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// GELU (tanh form) of two f16 values at once: 0.5 x + 0.5 x tanh(c x (1 +
// a x^2)), written c x + (c a) x^3 inside.  Six packed instructions for two
// values; for |x| > 255 the square overflows to inf and the result tends to
// x or 0, the function's own limits.
__device__ __forceinline__ uint32_t gelu_h2(uint32_t xr) {
  const __half2 x = *reinterpret_cast<const __half2*>(&xr);
  const __half2 c = __float2half2_rn(kGeluC), ca = __float2half2_rn(kGeluC * kGeluA), half = __float2half2_rn(0.5f);
  const __half2 u = __hmul2(x, __hfma2(__hmul2(x, x), ca, c));
  uint32_t ur = *reinterpret_cast<const uint32_t*>(&u), tr;
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(tr) : "r"(ur));
  const __half2 hx = __hmul2(x, half);
  const __half2 y = __hfma2(hx, *reinterpret_cast<const __half2*>(&tr), hx);
  return *reinterpret_cast<const uint32_t*>(&y);
}

// Inference: 16 vertices per warp step on the tensor cores, all three layers
// as f16 mma.sync m16n8k16 with FP32 accumulation, on the BF16-rounded
// weights converted by half_weight.  Each layer's accumulators plus bias are
// packed to f16x2 in registers, where they already sit as the next layer's A
// fragments; the GELUs run on the packed pairs.  Layer 3 is an MMA against w3 as column 0
// of an otherwise zero B, so lanes with t == 0 receive z of rows g and g+8.
// Writes s_v = softplus(z_v) and each CTA's partial sums of s and of s over
// dangling vertices.
__global__ void __launch_bounds__(128) mlp_infer_kernel(const float* feat, const float* norm, const float* params,
                                                        int32_t V, float* s_out, double* part_sum,
                                                        double* part_dang) {
  __shared__ __align__(16) __half sW1[kH][24];
  __shared__ __align__(16) __half sW2[kH][72];
  __shared__ float sb1[kH], sb2[kH], sb3, smean[kF], sinv[kF];
  __shared__ __align__(16) __half sw3[kH];
  __shared__ double s_red[2][4];
  for (int i = threadIdx.x; i < kH * 24; i += blockDim.x) {
    const int n = i / 24, k = i % 24;
    sW1[n][k] = half_weight(k < kF ? params[kOffW1 + n * kF + k] : 0.f);
  }
  for (int i = threadIdx.x; i < kH * 72; i += blockDim.x) {
    const int n = i / 72, k = i % 72;
    sW2[n][k] = half_weight(k < kH ? params[kOffW2 + n * kH + k] : 0.f);
  }
  for (int i = threadIdx.x; i < kH; i += blockDim.x) {
    sb1[i] = params[kOffB1 + i];
    sb2[i] = params[kOffB2 + i];
    sw3[i] = half_weight(params[kOffW3 + i]);
  }
  if (threadIdx.x == 0) sb3 = params[kOffB3];
  if (threadIdx.x < kF) {
    smean[threadIdx.x] = norm[threadIdx.x];
    sinv[threadIdx.x] = norm[kF + threadIdx.x];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int warps = gridDim.x * (blockDim.x >> 5);
  // Per-lane constants: layer biases of this lane's output columns and the
  // layer-3 B fragments (w3 in column 0: lanes with g == 0).
  float bl1[8][2], bl2[8][2];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    bl1[j][0] = sb1[8 * j + 2 * t];
    bl1[j][1] = sb1[8 * j + 2 * t + 1];
    bl2[j][0] = sb2[8 * j + 2 * t];
    bl2[j][1] = sb2[8 * j + 2 * t + 1];
  }
  uint32_t b3[4][2];
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    b3[kk][0] = g == 0 ? *reinterpret_cast<const uint32_t*>(&sw3[16 * kk + 2 * t]) : 0u;
    b3[kk][1] = g == 0 ? *reinterpret_cast<const uint32_t*>(&sw3[16 * kk + 8 + 2 * t]) : 0u;
  }
  const float b3s = sb3;
  double sum = 0, dang = 0;
  for (int grp = blockIdx.x * (blockDim.x >> 5) + wid; grp * 16 < V; grp += warps) {
    const int r0 = grp * 16 + g, r1 = r0 + 8;
    float x[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    if (2 * t < kF) {
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const int v = r ? r1 : r0;
        if (v < V) {
          const float2 f = *reinterpret_cast<const float2*>(feat + static_cast<size_t>(v) * kFeatStride + 2 * t);
          x[r][0] = (f.x - smean[2 * t]) * sinv[2 * t];
          x[r][1] = (f.y - smean[2 * t + 1]) * sinv[2 * t + 1];
        }
      }
    }
    const uint32_t a1[4] = {pack_h2(x[0][0], x[0][1]), pack_h2(x[1][0], x[1][1]), 0u, 0u};
    // Layer 1 -> GELU -> layer-2 A fragments (k-step kk takes n-tiles 2kk, 2kk+1).
    uint32_t a2[4][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float h[4] = {0.f, 0.f, 0.f, 0.f};
      const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&sW1[8 * j + g][2 * t]);
      const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&sW1[8 * j + g][2 * t + 8]);
      mma_f16(h, a1, b0, b1);
      a2[j >> 1][(j & 1) * 2] = gelu_h2(pack_h2(h[0] + bl1[j][0], h[1] + bl1[j][1]));
      a2[j >> 1][(j & 1) * 2 + 1] = gelu_h2(pack_h2(h[2] + bl1[j][0], h[3] + bl1[j][1]));
    }
    // Layer 2 -> GELU -> layer-3 A fragments.
    uint32_t a3[4][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&sW2[8 * j + g][16 * kk + 2 * t]);
        const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&sW2[8 * j + g][16 * kk + 8 + 2 * t]);
        mma_f16(c, a2[kk], b0, b1);
      }
      a3[j >> 1][(j & 1) * 2] = gelu_h2(pack_h2(c[0] + bl2[j][0], c[1] + bl2[j][1]));
      a3[j >> 1][(j & 1) * 2 + 1] = gelu_h2(pack_h2(c[2] + bl2[j][0], c[3] + bl2[j][1]));
    }
    float z[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) mma_f16(z, a3[kk], b3[kk][0], b3[kk][1]);
    if (t == 0) {
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const int v = r ? r1 : r0;
        if (v < V) {
          const float sv = softplus((r ? z[2] : z[0]) + b3s);
          s_out[v] = sv;
          sum += sv;
          if (feat[static_cast<size_t>(v) * kFeatStride + 5] != 0.f) dang += sv;
        }
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
    dang += __shfl_xor_sync(0xffffffffu, dang, o);
  }
  if (lane == 0) {
    s_red[0][wid] = sum;
    s_red[1][wid] = dang;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int i = 0; i < (blockDim.x >> 5); ++i) {
      a += s_red[0][i];
      b += s_red[1][i];
    }
    part_sum[blockIdx.x] = a;
    part_dang[blockIdx.x] = b;
  }
}

__global__ void mlp_normalize_kernel(const float* s, int32_t V, double inv_sum, float* out) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    out[v] = static_cast<float>(s[v] * inv_sum);
}

// Training: one CTA = kTrainSamples samples; forward in FP32 with BF16-rounded
// weights, backward in FP32; writes the CTA's gradient and loss partial.
__global__ void __launch_bounds__(kTrainThreads) mlp_train_kernel(const float* x_all, const float* t_all,
                                                                  int64_t n_all, int64_t first, int64_t count,
                                                                  const float* norm, const float* params,
                                                                  double inv_batch, float* part) {
  extern __shared__ float sm[];
  float* W1 = sm;                       // 64*6
  float* b1 = W1 + kH * kF;             // 64
  float* W2 = b1 + kH;                  // 64*65 (padded rows)
  float* b2 = W2 + kH * 65;             // 64
  float* w3 = b2 + kH;                  // 64
  float* X = w3 + kH;                   // 128*6
  float* Tg = X + kTrainSamples * kF;   // 128
  float* dz = Tg + kTrainSamples;       // 128
  float* A1 = dz + kTrainSamples;       // 128*64
  float* H1 = A1 + kTrainSamples * kH;  // 128*64 (later D1)
  float* A2 = H1 + kTrainSamples * kH;  // 128*64
  float* D2 = A2 + kTrainSamples * kH;  // 128*64
  __shared__ float s_loss[kTrainThreads / 32];
  const int tid = threadIdx.x;
  for (int i = tid; i < kH * kF; i += kTrainThreads) W1[i] = bf16r(params[kOffW1 + i]);
  for (int i = tid; i < kH * kH; i += kTrainThreads) W2[(i / kH) * 65 + (i % kH)] = bf16r(params[kOffW2 + i]);
  for (int i = tid; i < kH; i += kTrainThreads) {
    b1[i] = params[kOffB1 + i];
    b2[i] = params[kOffB2 + i];
    w3[i] = bf16r(params[kOffW3 + i]);
  }
  const float b3 = params[kOffB3];
  const int64_t base = first + static_cast<int64_t>(blockIdx.x) * kTrainSamples;
  for (int i = tid; i < kTrainSamples * kF; i += kTrainThreads) {
    const int s = i / kF, f = i % kF;
    const int64_t gidx = base + s;
    float v = 0.f;
    if (gidx < first + count) {
      const int64_t r = gidx % n_all;
      v = (x_all[r * kFeatStride + f] - norm[f]) * norm[kF + f];
    }
    X[i] = v;
  }
  for (int s = tid; s < kTrainSamples; s += kTrainThreads) {
    const int64_t gidx = base + s;
    Tg[s] = gidx < first + count ? t_all[gidx % n_all] : 0.f;
  }
  __syncthreads();
  // layer 1
  for (int i = tid; i < kTrainSamples * kH; i += kTrainThreads) {
    const int s = i / kH, n = i % kH;
    float a = b1[n];
#pragma unroll
    for (int f = 0; f < kF; ++f) a += X[s * kF + f] * W1[n * kF + f];
    A1[i] = a;
    H1[i] = gelu(a);
  }
  __syncthreads();
  // layer 2
  for (int i = tid; i < kTrainSamples * kH; i += kTrainThreads) {
    const int s = i / kH, n = i % kH;
    float a = b2[n];
    const float* h = H1 + s * kH;
    const float* w = W2 + n * 65;
#pragma unroll 16
    for (int k = 0; k < kH; ++k) a += h[k] * w[k];
    A2[i] = a;
  }
  __syncthreads();
  // layer 3, loss, dL/dz
  float loss = 0.f;
  for (int s = tid; s < kTrainSamples; s += kTrainThreads) {
    const bool live = base + s < first + count;
    float z = b3;
    for (int n = 0; n < kH; ++n) z += gelu(A2[s * kH + n]) * w3[n];
    const float sp = softplus(z);
    const float y = logf(sp);
    const float e = live ? y - Tg[s] : 0.f;
    // Weight N*r_v = exp(t): the L1 error of the start vector is carried by
    // the high-rank vertices (capped so single hubs do not dominate).
    const float wt = fminf(expf(Tg[s]), kLossWeightCap);
    loss += wt * e * e;
    const float sig = 1.f / (1.f + expf(-z));
    dz[s] = static_cast<float>(2.0 * inv_batch) * wt * e * sig / sp;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
  if ((tid & 31) == 0) s_loss[tid >> 5] = loss;
  __syncthreads();
  // D2 = dz * w3 * gelu'(A2)
  for (int i = tid; i < kTrainSamples * kH; i += kTrainThreads) {
    const int s = i / kH, n = i % kH;
    D2[i] = dz[s] * w3[n] * gelu_grad(A2[i]);
  }
  __syncthreads();
  float* g = part + static_cast<size_t>(blockIdx.x) * kPartStride;
  // dW3, db3, db2, dW2
  for (int n = tid; n < kH; n += kTrainThreads) {
    float gw = 0.f, gb = 0.f;
    for (int s = 0; s < kTrainSamples; ++s) {
      gw += dz[s] * gelu(A2[s * kH + n]);
      gb += D2[s * kH + n];
    }
    g[kOffW3 + n] = gw;
    g[kOffB2 + n] = gb;
  }
  if (tid == 0) {
    float gb = 0.f, l = 0.f;
    for (int s = 0; s < kTrainSamples; ++s) gb += dz[s];
    for (int w = 0; w < kTrainThreads / 32; ++w) l += s_loss[w];
    g[kOffB3] = gb;
    g[kNumParams] = l;
  }
  for (int i = tid; i < kH * kH; i += kTrainThreads) {
    const int n = i / kH, k = i % kH;
    float acc = 0.f;
    for (int s = 0; s < kTrainSamples; ++s) acc += D2[s * kH + n] * H1[s * kH + k];
    g[kOffW2 + i] = acc;
  }
  __syncthreads();
  // D1 = (D2 W2) * gelu'(A1), stored over H1
  for (int i = tid; i < kTrainSamples * kH; i += kTrainThreads) {
    const int s = i / kH, k = i % kH;
    float acc = 0.f;
    for (int n = 0; n < kH; ++n) acc += D2[s * kH + n] * W2[n * 65 + k];
    H1[i] = acc * gelu_grad(A1[i]);
  }
  __syncthreads();
  for (int i = tid; i < kH * kF; i += kTrainThreads) {
    const int n = i / kF, f = i % kF;
    float acc = 0.f;
    for (int s = 0; s < kTrainSamples; ++s) acc += H1[s * kH + n] * X[s * kF + f];
    g[kOffW1 + i] = acc;
  }
  for (int n = tid; n < kH; n += kTrainThreads) {
    float acc = 0.f;
    for (int s = 0; s < kTrainSamples; ++s) acc += H1[s * kH + n];
    g[kOffB1 + n] = acc;
  }
}

// Sums the CTA partials in CTA order; applies Adam when lr > 0.
__global__ void mlp_reduce_adam_kernel(const float* part, int n_part, float* grad, float* params, float* m, float* v,
                                       float lr, float b1, float b2, float c1, float c2, float eps) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kNumParams + 1; p += gridDim.x * blockDim.x) {
    double gsum = 0;
    for (int b = 0; b < n_part; ++b) gsum += part[static_cast<size_t>(b) * kPartStride + p];
    const float gp = static_cast<float>(gsum);
    grad[p] = gp;
    if (lr > 0.f && p < kNumParams) {
      const float mm = b1 * m[p] + (1.f - b1) * gp;
      const float vv = b2 * v[p] + (1.f - b2) * gp * gp;
      m[p] = mm;
      v[p] = vv;
      params[p] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    }
  }
}

__global__ void mlp_norm_stats_kernel(const float* x, int64_t n, double* part) {
  __shared__ double s[2 * kF][8];
  double acc[2 * kF] = {};
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
#pragma unroll
    for (int f = 0; f < kF; ++f) {
      const double v = x[i * kFeatStride + f];
      acc[f] += v;
      acc[kF + f] += v * v;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int f = 0; f < 2 * kF; ++f) {
    double a = acc[f];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) s[f][wid] = a;
  }
  __syncthreads();
  if (threadIdx.x < 2 * kF) {
    double a = 0;
    for (int w = 0; w < (blockDim.x >> 5); ++w) a += s[threadIdx.x][w];
    part[blockIdx.x * 2 * kF + threadIdx.x] = a;
  }
}

// Picks up to `max_samples` vertices (a seeded stride sample) and appends
// (features, log(N * r_v)) to the training set.
__global__ void mlp_gather_samples_kernel(const float* feat, const float* rank, int32_t V, int64_t stride,
                                          int64_t n_take, uint64_t seed, float* x_dst, float* t_dst) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n_take;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    uint64_t h = seed ^ (static_cast<uint64_t>(i) * 0x9e3779b97f4a7c15ull);
    h ^= h >> 31;
    h *= 0xbf58476d1ce4e5b9ull;
    h ^= h >> 29;
    int64_t v = i * stride + static_cast<int64_t>(h % static_cast<uint64_t>(stride));
    if (v >= V) v = V - 1;
#pragma unroll
    for (int f = 0; f < kFeatStride; ++f) x_dst[i * kFeatStride + f] = feat[v * kFeatStride + f];
    const float r = rank[v];
    t_dst[i] = logf(fmaxf(r, 1e-30f) * static_cast<float>(V));
  }
}

}  // namespace

struct gx_mlp {
  int dev = 0;
  int n_sm = 0;
  cudaStream_t s = nullptr;
  float* params = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  float* grad = nullptr;
  float* part = nullptr;
  int part_cap = 0;
  float* norm = nullptr;  // mean[6], 1/std[6]
  bool norm_set = false;
  float* x = nullptr;     // training features [n][8]
  float* t = nullptr;     // targets [n]
  int64_t n = 0, cap = 0;
  int64_t adam_t = 0;
  uint64_t seed = 0;
  ~gx_mlp() {
    cudaSetDevice(dev);
    dev_free(&params);
    dev_free(&m);
    dev_free(&v);
    dev_free(&grad);
    dev_free(&part);
    dev_free(&norm);
    dev_free(&x);
    dev_free(&t);
    if (s) cudaStreamDestroy(s);
  }
};

namespace {

gx_status ensure_part(gx_mlp* m, int blocks) {
  if (blocks <= m->part_cap) return GX_OK;
  GX_TRY(dev_alloc(&m->part, static_cast<size_t>(blocks) * kPartStride));
  m->part_cap = blocks;
  return GX_OK;
}

gx_status compute_norm(gx_mlp* m) {
  const int grid = std::min<int64_t>(m->n_sm * 4, std::max<int64_t>(1, (m->n + 255) / 256));
  double* part = nullptr;
  GX_TRY(dev_alloc(&part, static_cast<size_t>(grid) * 2 * kF));
  mlp_norm_stats_kernel<<<grid, 256, 0, m->s>>>(m->x, m->n, part);
  std::vector<double> h(static_cast<size_t>(grid) * 2 * kF);
  cudaError_t err = cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, m->s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(m->s);
  gx::pool_free(part);
  if (err != cudaSuccess) return fail(GX_ERR_CUDA, "mlp norm: %s", cudaGetErrorString(err));
  float nrm[2 * kF];
  for (int f = 0; f < kF; ++f) {
    double s1 = 0, s2 = 0;
    for (int b = 0; b < grid; ++b) {
      s1 += h[static_cast<size_t>(b) * 2 * kF + f];
      s2 += h[static_cast<size_t>(b) * 2 * kF + kF + f];
    }
    const double mean = s1 / m->n, var = std::max(s2 / m->n - mean * mean, 1e-12);
    nrm[f] = static_cast<float>(mean);
    nrm[kF + f] = static_cast<float>(1.0 / std::sqrt(var));
  }
  GX_CUDA(cudaMemcpy(m->norm, nrm, sizeof(nrm), cudaMemcpyHostToDevice));
  m->norm_set = true;
  return GX_OK;
}

// Scratch of one feature pass, allocated before any timed region.
struct FeatScratch {
  NbrInfo* nb = nullptr;
  double* part = nullptr;
  unsigned int* cursor = nullptr;
  int grid = 0;
  cudaEvent_t ready = nullptr, heavy_done = nullptr;  // fork / join of the heavy lists' side stream
  ~FeatScratch() {
    dev_free(&nb);
    dev_free(&part);
    dev_free(&cursor);
    if (ready) cudaEventDestroy(ready);
    if (heavy_done) cudaEventDestroy(heavy_done);
  }
  gx_status alloc(const gx_engine* e) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mlp_features_kernel, 256, 0);
    grid = std::max(1, per_sm) * e->n_sm;
    GX_TRY(dev_alloc(&nb, static_cast<size_t>(e->V)));
    GX_TRY(dev_alloc(&part, static_cast<size_t>(grid) + e->heavy.size()));
    GX_TRY(dev_alloc(&cursor, 1));
    GX_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    GX_CUDA(cudaEventCreateWithFlags(&heavy_done, cudaEventDisableTiming));
    return GX_OK;
  }
};

// Features of the engine's graph into feat[V][8]; returns the uniform
// start's first-step L1 residual.
gx_status engine_features(gx_engine* e, double damping, float* feat, double* uniform_resid, cudaStream_t s,
                          FeatScratch& fs) {
  const int32_t V = e->V;
  const double dangling0 = static_cast<double>(e->n_dangling) / V;
  // The engine's heavy-vertex table (in-degree above heavy_degree) marks
  // the lists the tile kernel leaves to a CTA each.
  const int32_t n_heavy = static_cast<int32_t>(e->heavy.size());
  const int64_t heavy_deg = e->cfg.exact_order ? INT64_MAX : std::max(e->cfg.heavy_degree, 32);
  mlp_nbr_kernel<<<fs.grid, 256, 0, s>>>(e->d_off, e->d_outdeg, V, fs.nb);
  GX_CUDA(cudaMemsetAsync(fs.cursor, 0, sizeof(unsigned int), s));
  GX_CUDA(cudaMemsetAsync(fs.part, 0, sizeof(double) * fs.grid, s));
  // The heavy lists (a CTA each) run on the engine's side stream beside the
  // tile kernel; both write disjoint vertices' features and partials.  (With
  // one CTA per SM instead, the hub lists became the critical path: 2.07 ->
  // 2.63 ms at R-MAT scale 24.)
  if (n_heavy) {
    GX_CUDA(cudaEventRecord(fs.ready, s));
    GX_CUDA(cudaStreamWaitEvent(e->s_copy, fs.ready, 0));
    mlp_heavy_features_kernel<<<std::min(n_heavy, e->n_sm * 8), 256, 0, e->s_copy>>>(
        e->d_off, e->d_col, e->d_outdeg, fs.nb, e->d_heavy, n_heavy, V, damping, dangling0, feat, fs.part + fs.grid);
    GX_CUDA(cudaEventRecord(fs.heavy_done, e->s_copy));
  }
  mlp_features_kernel<<<fs.grid, 256, 0, s>>>(e->d_off, e->d_col, e->d_outdeg, fs.nb, V, e->d_units,
                                               static_cast<int32_t>(e->units.size()), fs.cursor,
                                               n_heavy ? heavy_deg : INT64_MAX, damping, dangling0, feat, fs.part);
  if (n_heavy) GX_CUDA(cudaStreamWaitEvent(s, fs.heavy_done, 0));
  GX_CUDA(cudaGetLastError());
  std::vector<double> h(static_cast<size_t>(fs.grid) + n_heavy);
  GX_CUDA(cudaMemcpyAsync(h.data(), fs.part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s));
  GX_CUDA(cudaStreamSynchronize(s));
  double r = 0;
  for (double x : h) r += x;
  if (uniform_resid) *uniform_resid = r;
  return GX_OK;
}

void host_init_params(uint64_t seed, std::vector<float>& p) {
  p.assign(kNumParams, 0.f);
  auto uni = [&](uint64_t i) {
    const uint64_t h = mix64(seed ^ mix64(i + 1));
    return static_cast<float>((h >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
  };
  for (int i = 0; i < kH * kF; ++i) p[kOffW1 + i] = uni(i) * std::sqrt(6.f / (kF + kH));
  for (int i = 0; i < kH * kH; ++i) p[kOffW2 + i] = uni(100000 + i) * std::sqrt(6.f / (2 * kH));
  for (int i = 0; i < kH; ++i) p[kOffW3 + i] = uni(200000 + i) * std::sqrt(6.f / (kH + 1));
  p[kOffB3] = 0.5413f;  // softplus(b3) = 1: the mean of N * r
}

}  // namespace

extern "C" {

int32_t gx_mlp_num_params(void) { return kNumParams; }

gx_status gx_mlp_create(int32_t device, uint64_t seed, gx_mlp** out) {
  if (!out) return fail(GX_ERR_INVALID, "gx_mlp_create: out is NULL");
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(GX_ERR_NODEVICE, "gx_mlp_create: no CUDA device");
  }
  std::unique_ptr<gx_mlp> m(new gx_mlp());
  m->dev = device;
  m->seed = seed;
  GX_CUDA(cudaSetDevice(device));
  GX_CUDA(cudaDeviceGetAttribute(&m->n_sm, cudaDevAttrMultiProcessorCount, device));
  GX_CUDA(cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking));
  GX_TRY(dev_alloc(&m->params, kNumParams + 1));
  GX_TRY(dev_alloc(&m->m, kNumParams + 1));
  GX_TRY(dev_alloc(&m->v, kNumParams + 1));
  GX_TRY(dev_alloc(&m->grad, kNumParams + 1));
  GX_TRY(dev_alloc(&m->norm, 2 * kF));
  std::vector<float> p;
  host_init_params(seed, p);
  p.push_back(0.f);
  GX_CUDA(cudaMemcpy(m->params, p.data(), sizeof(float) * p.size(), cudaMemcpyHostToDevice));
  GX_CUDA(cudaMemset(m->m, 0, sizeof(float) * (kNumParams + 1)));
  GX_CUDA(cudaMemset(m->v, 0, sizeof(float) * (kNumParams + 1)));
  float nrm[2 * kF];
  for (int f = 0; f < kF; ++f) {
    nrm[f] = 0.f;
    nrm[kF + f] = 1.f;
  }
  GX_CUDA(cudaMemcpy(m->norm, nrm, sizeof(nrm), cudaMemcpyHostToDevice));
  *out = m.release();
  return GX_OK;
}

gx_status gx_mlp_destroy(gx_mlp* m) {
  delete m;
  return GX_OK;
}

gx_status gx_mlp_get_params(gx_mlp* m, float* params, float* norm) {
  if (!m) return fail(GX_ERR_INVALID, "gx_mlp_get_params: NULL");
  GX_CUDA(cudaSetDevice(m->dev));
  if (params) GX_CUDA(cudaMemcpy(params, m->params, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost));
  if (norm) GX_CUDA(cudaMemcpy(norm, m->norm, sizeof(float) * 2 * kF, cudaMemcpyDeviceToHost));
  return GX_OK;
}

gx_status gx_mlp_set_params(gx_mlp* m, const float* params, const float* norm) {
  if (!m) return fail(GX_ERR_INVALID, "gx_mlp_set_params: NULL");
  GX_CUDA(cudaSetDevice(m->dev));
  if (params) GX_CUDA(cudaMemcpy(m->params, params, sizeof(float) * kNumParams, cudaMemcpyHostToDevice));
  if (norm) {
    GX_CUDA(cudaMemcpy(m->norm, norm, sizeof(float) * 2 * kF, cudaMemcpyHostToDevice));
    m->norm_set = true;
  }
  return GX_OK;
}

gx_status gx_mlp_add_graph(gx_mlp* m, gx_engine* e, int32_t max_samples, int32_t max_iter, double tolerance) {
  gx::NvtxRange nvtx_range("gx_mlp_add_graph");
  if (!m || !e || max_samples < 1) return fail(GX_ERR_INVALID, "gx_mlp_add_graph: bad arguments");
  if (!e->loaded || !e->all_resident) return fail(GX_ERR_STATE, "gx_mlp_add_graph: load a resident graph first");
  if (e->dev != m->dev) return fail(GX_ERR_INVALID, "gx_mlp_add_graph: engine and MLP on different devices");
  GX_CUDA(cudaSetDevice(m->dev));
  const int32_t V = e->V;
  // Converged standard PageRank: the training target.
  gx_run_params p;
  gx_run_params_default(&p, GX_APP_PAGERANK_STD);
  p.max_iter = max_iter;
  p.tolerance = tolerance;
  GX_TRY(gx_run(e, &p, nullptr));
  GX_CUDA(cudaMemcpy(e->h_ctl, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  const float* rank = static_cast<const float*>(e->d_val[e->h_ctl->cur & 1]);
  float* feat = nullptr;
  GX_TRY(dev_alloc(&feat, static_cast<size_t>(V) * kFeatStride));
  std::unique_ptr<float, void (*)(float*)> fg(feat, [](float* q) { gx::pool_free(q); });
  FeatScratch fs;
  GX_TRY(fs.alloc(e));
  GX_TRY(engine_features(e, p.damping, feat, nullptr, m->s, fs));
  const int64_t take = std::min<int64_t>(max_samples, V);
  const int64_t stride = V / take;
  if (m->n + take > m->cap) {
    const int64_t ncap = std::max<int64_t>(m->n + take, m->cap * 2);
    float *nx = nullptr, *nt = nullptr;
    GX_TRY(dev_alloc(&nx, static_cast<size_t>(ncap) * kFeatStride));
    GX_TRY(dev_alloc(&nt, static_cast<size_t>(ncap)));
    if (m->n) {
      GX_CUDA(cudaMemcpy(nx, m->x, sizeof(float) * m->n * kFeatStride, cudaMemcpyDeviceToDevice));
      GX_CUDA(cudaMemcpy(nt, m->t, sizeof(float) * m->n, cudaMemcpyDeviceToDevice));
    }
    dev_free(&m->x);
    dev_free(&m->t);
    m->x = nx;
    m->t = nt;
    m->cap = ncap;
  }
  mlp_gather_samples_kernel<<<m->n_sm * 4, 256, 0, m->s>>>(feat, rank, V, stride, take, m->seed ^ (m->n * 7919),
                                                           m->x + m->n * kFeatStride, m->t + m->n);
  GX_CUDA(cudaGetLastError());
  GX_CUDA(cudaStreamSynchronize(m->s));
  m->n += take;
  return GX_OK;
}

gx_status gx_mlp_train(gx_mlp* m, int32_t epochs, int32_t batch, double lr, double* final_loss) {
  gx::NvtxRange nvtx_range("gx_mlp_train");
  if (!m || epochs < 0 || batch < kTrainSamples) return fail(GX_ERR_INVALID, "gx_mlp_train: bad arguments");
  if (m->n == 0) return fail(GX_ERR_STATE, "gx_mlp_train: no training samples (gx_mlp_add_graph)");
  GX_CUDA(cudaSetDevice(m->dev));
  if (!m->norm_set) GX_TRY(compute_norm(m));
  const int blocks = (batch + kTrainSamples - 1) / kTrainSamples;
  GX_TRY(ensure_part(m, blocks));
  const size_t smem = sizeof(float) * (kH * kF + kH + kH * 65 + kH + kH + kTrainSamples * kF + 2 * kTrainSamples +
                                       4 * kTrainSamples * kH);
  GX_CUDA(cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  const int64_t per_epoch = (m->n + batch - 1) / batch;
  double loss_sum = 0;
  int64_t loss_n = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    loss_sum = 0;
    loss_n = 0;
    const int64_t shift = static_cast<int64_t>(mix64(m->seed + ep) % static_cast<uint64_t>(m->n));
    for (int64_t b = 0; b < per_epoch; ++b) {
      const int64_t first = shift + b * batch;
      const int64_t count = std::min<int64_t>(batch, m->n - b * batch);
      ++m->adam_t;
      const float c1 = static_cast<float>(1.0 - std::pow(0.9, static_cast<double>(m->adam_t)));
      const float c2 = static_cast<float>(1.0 - std::pow(0.999, static_cast<double>(m->adam_t)));
      const int nb = static_cast<int>((count + kTrainSamples - 1) / kTrainSamples);
      mlp_train_kernel<<<nb, kTrainThreads, smem, m->s>>>(m->x, m->t, m->n, first, count, m->norm, m->params,
                                                           1.0 / count, m->part);
      mlp_reduce_adam_kernel<<<(kNumParams + 256) / 256, 256, 0, m->s>>>(m->part, nb, m->grad, m->params, m->m, m->v,
                                                                        static_cast<float>(lr), 0.9f, 0.999f, c1, c2,
                                                                        1e-8f);
      if (ep + 1 == epochs || (b % 64) == 0) {
        float l = 0;
        GX_CUDA(cudaMemcpyAsync(&l, m->grad + kNumParams, sizeof(float), cudaMemcpyDeviceToHost, m->s));
        GX_CUDA(cudaStreamSynchronize(m->s));
        loss_sum += l;
        loss_n += count;
      }
    }
  }
  GX_CUDA(cudaGetLastError());
  GX_CUDA(cudaStreamSynchronize(m->s));
  if (final_loss) *final_loss = loss_n ? loss_sum / loss_n : 0;
  return GX_OK;
}

gx_status gx_mlp_grad(gx_mlp* m, const float* host_x, const float* host_t, int32_t n, float* host_grad,
                      double* loss) {
  if (!m || !host_x || !host_t || n < 1 || !host_grad) return fail(GX_ERR_INVALID, "gx_mlp_grad: bad arguments");
  GX_CUDA(cudaSetDevice(m->dev));
  float *x = nullptr, *t = nullptr;
  GX_TRY(dev_alloc(&x, static_cast<size_t>(n) * kFeatStride));
  std::unique_ptr<float, void (*)(float*)> gx_(x, [](float* q) { gx::pool_free(q); });
  GX_TRY(dev_alloc(&t, static_cast<size_t>(n)));
  std::unique_ptr<float, void (*)(float*)> gt_(t, [](float* q) { gx::pool_free(q); });
  std::vector<float> hx(static_cast<size_t>(n) * kFeatStride, 0.f);
  for (int32_t i = 0; i < n; ++i)
    for (int f = 0; f < kF; ++f) hx[static_cast<size_t>(i) * kFeatStride + f] = host_x[static_cast<size_t>(i) * kF + f];
  GX_CUDA(cudaMemcpy(x, hx.data(), sizeof(float) * hx.size(), cudaMemcpyHostToDevice));
  GX_CUDA(cudaMemcpy(t, host_t, sizeof(float) * n, cudaMemcpyHostToDevice));
  const int nb = (n + kTrainSamples - 1) / kTrainSamples;
  GX_TRY(ensure_part(m, nb));
  const size_t smem = sizeof(float) * (kH * kF + kH + kH * 65 + kH + kH + kTrainSamples * kF + 2 * kTrainSamples +
                                       4 * kTrainSamples * kH);
  GX_CUDA(cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  mlp_train_kernel<<<nb, kTrainThreads, smem, m->s>>>(x, t, n, 0, n, m->norm, m->params, 1.0 / n, m->part);
  mlp_reduce_adam_kernel<<<(kNumParams + 256) / 256, 256, 0, m->s>>>(m->part, nb, m->grad, m->params, m->m, m->v, 0.f,
                                                                    0.9f, 0.999f, 1.f, 1.f, 1e-8f);
  GX_CUDA(cudaGetLastError());
  std::vector<float> g(kNumParams + 1);
  GX_CUDA(cudaMemcpyAsync(g.data(), m->grad, sizeof(float) * (kNumParams + 1), cudaMemcpyDeviceToHost, m->s));
  GX_CUDA(cudaStreamSynchronize(m->s));
  memcpy(host_grad, g.data(), sizeof(float) * kNumParams);
  if (loss) *loss = g[kNumParams] / n;
  return GX_OK;
}

gx_status gx_mlp_predict(gx_mlp* m, gx_engine* e, double damping, float* host_out, double* ms_features,
                         double* ms_mlp) {
  gx::NvtxRange nvtx_range("gx_mlp_predict");
  if (!m || !e) return fail(GX_ERR_INVALID, "gx_mlp_predict: bad arguments");
  if (!e->loaded || !e->all_resident) return fail(GX_ERR_STATE, "gx_mlp_predict: load a resident graph first");
  GX_CUDA(cudaSetDevice(e->dev));
  const int32_t V = e->V;
  cudaStream_t s = e->s_comp;
  float *feat = nullptr, *sv = nullptr;
  GX_TRY(dev_alloc(&feat, static_cast<size_t>(V) * kFeatStride));
  std::unique_ptr<float, void (*)(float*)> fg(feat, [](float* q) { gx::pool_free(q); });
  GX_TRY(dev_alloc(&sv, static_cast<size_t>(V)));
  std::unique_ptr<float, void (*)(float*)> sg(sv, [](float* q) { gx::pool_free(q); });
  FeatScratch fs;
  GX_TRY(fs.alloc(e));
  const int grid = e->n_sm * 8;
  double *ps = nullptr, *pd = nullptr;
  GX_TRY(dev_alloc(&ps, static_cast<size_t>(grid)));
  std::unique_ptr<double, void (*)(double*)> psg(ps, [](double* q) { gx::pool_free(q); });
  GX_TRY(dev_alloc(&pd, static_cast<size_t>(grid)));
  std::unique_ptr<double, void (*)(double*)> pdg(pd, [](double* q) { gx::pool_free(q); });
  cudaEvent_t ev[3];
  for (auto& x : ev) GX_CUDA(cudaEventCreate(&x));
  GX_CUDA(cudaEventRecord(ev[0], s));
  double ures = 0;
  GX_TRY(engine_features(e, damping, feat, &ures, s, fs));
  GX_CUDA(cudaEventRecord(ev[1], s));
  mlp_infer_kernel<<<grid, 128, 0, s>>>(feat, m->norm, m->params, V, sv, ps, pd);
  std::vector<double> hs(grid), hd(grid);
  GX_CUDA(cudaMemcpyAsync(hs.data(), ps, sizeof(double) * grid, cudaMemcpyDeviceToHost, s));
  GX_CUDA(cudaMemcpyAsync(hd.data(), pd, sizeof(double) * grid, cudaMemcpyDeviceToHost, s));
  GX_CUDA(cudaStreamSynchronize(s));
  double S = 0, D = 0;
  for (int i = 0; i < grid; ++i) {
    S += hs[i];
    D += hd[i];
  }
  float* dst = static_cast<float*>(e->d_val[0]);
  mlp_normalize_kernel<<<grid, 256, 0, s>>>(sv, V, 1.0 / S, dst);
  GX_CUDA(cudaEventRecord(ev[2], s));
  GX_CUDA(cudaEventSynchronize(ev[2]));
  float t0 = 0, t1 = 0;
  cudaEventElapsedTime(&t0, ev[0], ev[1]);
  cudaEventElapsedTime(&t1, ev[1], ev[2]);
  for (auto& x : ev) cudaEventDestroy(x);
  if (ms_features) *ms_features = t0;
  if (ms_mlp) *ms_mlp = t1;
  e->device_init_dangling = D / S;
  e->last_uniform_resid = ures;
  if (host_out) {
    const void* src = dst;
    if (e->relabeled) {  // back to the caller's numbering
      gather_values_kernel<<<grid, 256, 0, s>>>(reinterpret_cast<const uint32_t*>(dst), e->d_perm, V, e->d_stage);
      GX_CUDA(cudaGetLastError());
      src = e->d_stage;
    }
    GX_CUDA(cudaMemcpyAsync(host_out, src, sizeof(float) * V, cudaMemcpyDeviceToHost, s));
    GX_CUDA(cudaStreamSynchronize(s));
  }
  return GX_OK;
}

gx_status gx_pagerank_warm(gx_engine* e, gx_mlp* m, int32_t max_iter, double tolerance, double damping,
                           gx_warm_stats* out) {
  gx::NvtxRange nvtx_range("gx_pagerank_warm");
  if (!e || !m || max_iter < 1) return fail(GX_ERR_INVALID, "gx_pagerank_warm: bad arguments");
  const auto t0 = std::chrono::steady_clock::now();
  gx_warm_stats ws{};
  GX_TRY(gx_mlp_predict(m, e, damping, nullptr, &ws.ms_features, &ws.ms_mlp));
  ws.resid_uniform_first = e->last_uniform_resid;
  gx_run_params p;
  gx_run_params_default(&p, GX_APP_PAGERANK_STD);
  p.damping = damping;
  p.tolerance = tolerance;
  p.use_init = 1;
  // First step from the predicted start.
  p.max_iter = 1;
  e->device_init = true;
  gx_run_stats st{};
  GX_TRY(gx_run(e, &p, &st));
  ws.resid_warm_first = st.residual_l1_last;
  double ms = st.ms_total;
  int32_t iters = st.iterations;
  if (ws.resid_warm_first <= ws.resid_uniform_first) {
    ws.used_warm = 1;
    // Continue from the current vector: move it into buffer 0 and restart the
    // loop from there (the dangling mass of that vector seeds the base).
    GX_CUDA(cudaMemcpy(e->h_ctl, e->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    const int cur = e->h_ctl->cur & 1;
    if (cur == 1) GX_CUDA(cudaMemcpy(e->d_val[0], e->d_val[1], sizeof(float) * e->V, cudaMemcpyDeviceToDevice));
    e->device_init_dangling = static_cast<double>(e->last_stats[0].dangl_fx) / (static_cast<double>(e->V) * 1073741824.0);
    if (ws.resid_warm_first >= tolerance || tolerance <= 0) {
      p.max_iter = max_iter - 1;
      e->device_init = true;
      if (p.max_iter > 0) {
        GX_TRY(gx_run(e, &p, &st));
        ms += st.ms_total;
        iters += st.iterations;
        ws.resid_last = st.residual_l1_last;
      } else {
        ws.resid_last = ws.resid_warm_first;
      }
    } else {
      ws.resid_last = ws.resid_warm_first;
    }
  } else {
    ws.used_warm = 0;
    p.use_init = 0;
    p.max_iter = max_iter;
    GX_TRY(gx_run(e, &p, &st));
    ms += st.ms_total;
    iters += st.iterations;
    ws.resid_last = st.residual_l1_last;
  }
  ws.iterations = iters;
  ws.ms_pagerank = ms;
  ws.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (out) *out = ws;
  return GX_OK;
}

}  // extern "C"

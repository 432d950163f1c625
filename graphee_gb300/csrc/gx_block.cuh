// Pull kernel over the block layout, selected by gx_config.layout = 1 (the
// engine then re-lays each shard's edges at load time; see build_blocks in
// gx_engine.cu).  The default layout is the warp work units of
// gx_kernels.cuh, which measured faster on R-MAT inputs.
//
// A block is one of
//   light  : up to 32 vertices of in-degree <= kLightDegree, consecutive in
//            id order within the shard, and their in-edges (<= kBlockEdges)
//   medium : vertices of in-degree in (kLightDegree, kBlockEdges], packed
//            up to kBlockEdges edges
//   heavy  : one kBlockEdges-edge chunk of a longer list
// with its edges (and weights), vertex ids and block-relative list starts
// stored contiguously and 16-byte aligned.  Every warp of a persistent grid
// walks its own blocks (static stride) through its own two shared-memory
// stages: lane 0 issues the 1-D TMA bulk copies (cp.async.bulk + mbarrier
// complete_tx) of the next block while the warp gathers for the current
// one, and no warp ever waits for another, so only the data-dependent
// gathers remain on the critical path.
// Each block is then two phases: all lanes issue every gather of the block at
// once (up to 16 per lane) into a per-warp shared-memory value buffer; then
//   light/medium : a lane per vertex folds its slice of the buffer in edge
//                  order (the reference's summation order, so light and
//                  medium vertices match the reference bit for bit);
//   heavy        : a fixed-shape tree over the chunk; the warp that finishes
//                  a vertex's last chunk folds the chunk partials in order.
// Every mbarrier wait is bounded: on timeout the kernel records an error in
// the control block and stops.
#pragma once
#include "gx_kernels.cuh"

namespace gx {

constexpr int kBlockEdges = 512;
constexpr int kBlockVerts = 32;
constexpr int kLightDegree = 32;
constexpr int kBlockThreads = 256;
constexpr int kBlockWarps = kBlockThreads / 32;
constexpr uint32_t kWaitSpins = 1u << 26;

struct BlockDesc {
  long long e_begin;  // first edge of the block in the block layout (multiple of 4)
  int n_copy;         // edges copied (multiple of 4)
  int n_real;         // edges in use
  int first;          // light/medium: first index into vlist/loff (multiple of 4); heavy: heavy id
  int count;          // light/medium: vertices; heavy: chunks of the vertex
  int type;           // 0 light, 1 medium, 2 heavy chunk
  int aux;            // heavy: chunk index
  int shard;
  int pad;
};

struct BlockArgs {
  Ctl* ctl;
  const BlockDesc* blocks;
  int n_blocks;
  const int32_t* colp;   // edges in block layout
  const uint32_t* wp;    // weights in block layout (weighted SSSP)
  const int32_t* vlist;  // vertex ids of light/medium blocks
  const int32_t* loff;   // block-relative list starts
  const int4* heavy;     // (v, n_chunks, partial base, shard)
  const int32_t* outdeg;
  void* val[2];
  float* con[2];
  void* partial;
  unsigned int* hticket;
  uint32_t* bm;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// 1-D bulk copy global -> shared, completing on `bar`; 16-byte aligned, size % 16 == 0.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

template <int APP>
constexpr int block_stage_bytes() {
  return kBlockEdges * 4 * (APP == K_SSSP_W ? 2 : 1) + kBlockVerts * 4 * 2 + 64;
}

template <int APP>
__device__ __forceinline__ void issue_block(const BlockArgs& a, int blk, unsigned char* stage, uint64_t* bar) {
  const BlockDesc d = a.blocks[blk];
  *reinterpret_cast<BlockDesc*>(stage) = d;
  int32_t* col_s = reinterpret_cast<int32_t*>(stage + 64);
  uint32_t* w_s = reinterpret_cast<uint32_t*>(stage + 64 + kBlockEdges * 4);
  int32_t* vl_s = reinterpret_cast<int32_t*>(stage + 64 + kBlockEdges * 4 * (APP == K_SSSP_W ? 2 : 1));
  int32_t* lo_s = vl_s + kBlockVerts;
  uint32_t bytes = static_cast<uint32_t>(d.n_copy) * 4u * (APP == K_SSSP_W ? 2u : 1u);
  const int nv = d.type < 2 ? ((d.count + 3) & ~3) : 0;
  bytes += static_cast<uint32_t>(nv) * 8u;
  mbar_expect_tx(bar, bytes);
  if (d.n_copy > 0) {
    tma_load_1d(col_s, a.colp + d.e_begin, static_cast<uint32_t>(d.n_copy) * 4u, bar);
    if constexpr (APP == K_SSSP_W) tma_load_1d(w_s, a.wp + d.e_begin, static_cast<uint32_t>(d.n_copy) * 4u, bar);
  }
  if (nv > 0) {
    tma_load_1d(vl_s, a.vlist + d.first, static_cast<uint32_t>(nv) * 4u, bar);
    tma_load_1d(lo_s, a.loff + d.first, static_cast<uint32_t>(nv) * 4u, bar);
  }
}

template <int APP>
__device__ __forceinline__ typename AppTraits<APP>::T stage_value(const void* src_val, const float* src_con,
                                                                  const int32_t* col_s, const uint32_t* w_s, int k) {
  uint32_t wt = 0;
  if constexpr (APP == K_SSSP_W) wt = w_s[k];
  const int32_t u = col_s[k];
  if constexpr (is_pr<APP>()) return __ldg(src_con + u);
  else if constexpr (APP == K_SSSP_UNIT) return __ldg(static_cast<const int32_t*>(src_val) + u) + 1;
  else if constexpr (APP == K_SSSP_W) return sat_add(__ldg(static_cast<const uint32_t*>(src_val) + u), wt);
  else return __ldg(static_cast<const int32_t*>(src_val) + u);
}

// Lanes whose vertices share a bitmap word combine their bits; the lowest
// such lane issues one atomicOr.
__device__ __forceinline__ void set_active_bit(uint32_t* bm, int v, bool act) {
  if (!__ballot_sync(0xffffffffu, act)) return;
  const unsigned grp = __match_any_sync(0xffffffffu, v >> 5);
  const unsigned bits = __reduce_or_sync(grp, act ? (1u << (v & 31)) : 0u);
  if ((threadIdx.x & 31) == __ffs(grp) - 1 && bits) atomicOr(bm + (v >> 5), bits);
}

#ifndef GX_BLOCK_MIN_BLOCKS
#define GX_BLOCK_MIN_BLOCKS 3
#endif

template <int APP>
__global__ void __launch_bounds__(kBlockThreads, GX_BLOCK_MIN_BLOCKS) pull_block_kernel(BlockArgs a) {
  typedef typename AppTraits<APP>::T T;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ uint64_t bar[kBlockWarps][2];
  Ctl* ctl = a.ctl;
  const int done = ctl->done, mode = ctl->mode;
  if (done || mode == MODE_PUSH) return;
  ApplyCtx c;
  c.step = ctl->step;
  c.damping = ctl->damping;
  c.inv_n = ctl->inv_n;
  c.fx_scale = ctl->fx_scale;
  c.base = ctl->base;
  c.outdeg = ctl->push_ok ? a.outdeg : nullptr;
  const int cur = ctl->cur;
  const int group = ctl->shard_group;
  const unsigned long long smask = ctl->shard_mask;
  const bool selective = mode == MODE_SELECTIVE;
  const void* src_val = cur ? a.val[1] : a.val[0];
  void* dst_val = cur ? a.val[0] : a.val[1];
  const float* src_con = cur ? a.con[1] : a.con[0];
  float* dst_con = cur ? a.con[0] : a.con[1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int kStage = block_stage_bytes<APP>();
  // Per warp: two copy stages, then one buffer of gathered values.
  unsigned char* wsm = smem_raw + static_cast<size_t>(wid) * (2 * kStage + kBlockEdges * 4);
  T* vbuf = reinterpret_cast<T*>(wsm + 2 * kStage);
  uint64_t* wbar = bar[wid];
  if (lane == 0) {
    mbar_init(&wbar[0], 1);
    mbar_init(&wbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  LocalAcc la;
  uint32_t parity[2] = {0, 0};
  int st = 0;
  bool err = false;
  const int gw = blockIdx.x * kBlockWarps + wid;
  const int nw = gridDim.x * kBlockWarps;
  int b = gw;
  if (lane == 0 && b < a.n_blocks) issue_block<APP>(a, b, wsm, &wbar[0]);
  for (; b < a.n_blocks; b += nw) {
    const int nb = b + nw;
    if (lane == 0 && nb < a.n_blocks) {
      fence_proxy_async();
      issue_block<APP>(a, nb, wsm + (st ^ 1) * kStage, &wbar[st ^ 1]);
    }
    // Bounded wait for this block's copies.
    uint32_t spins = 0;
    bool ready = mbar_try_wait(&wbar[st], parity[st]);
    while (!ready && ++spins < kWaitSpins) ready = mbar_try_wait(&wbar[st], parity[st]);
    if (!__all_sync(0xffffffffu, ready)) {
      err = true;
      break;
    }
    parity[st] ^= 1u;
    const unsigned char* sp = wsm + st * kStage;
    const BlockDesc d = *reinterpret_cast<const BlockDesc*>(sp);
    const int32_t* col_s = reinterpret_cast<const int32_t*>(sp + 64);
    const uint32_t* w_s = reinterpret_cast<const uint32_t*>(sp + 64 + kBlockEdges * 4);
    const int32_t* vl_s = reinterpret_cast<const int32_t*>(sp + 64 + kBlockEdges * 4 * (APP == K_SSSP_W ? 2 : 1));
    const int32_t* lo_s = vl_s + kBlockVerts;
    const bool on = !selective || ((smask >> (d.shard / group)) & 1ull);
    // Per-lane vertex of a light/medium block, loaded before the gathers.
    const bool valid = d.type < 2 && lane < d.count;
    int v = 0, beg = 0, end = 0;
    T old = T(0);
    int32_t od = 0;
    if (valid) {
      v = vl_s[lane];
      beg = lo_s[lane];
      end = lane + 1 < d.count ? lo_s[lane + 1] : d.n_real;
      old = static_cast<const T*>(src_val)[v];
      if constexpr (is_pr<APP>()) od = a.outdeg[v];
    }
    if (!on) {
      if (valid) {
        static_cast<T*>(dst_val)[v] = old;
        if constexpr (is_pr<APP>()) dst_con[v] = src_con[v];
      }
      if (d.type == 2 && d.aux == 0 && lane == 0) {
        const int hv = a.heavy[d.first].x;
        static_cast<T*>(dst_val)[hv] = static_cast<const T*>(src_val)[hv];
        if constexpr (is_pr<APP>()) dst_con[hv] = src_con[hv];
      }
      __syncwarp();
      st ^= 1;
      continue;
    }
    // Phase 1: every gather of the block in flight at once (16 per lane).
    {
      T vals[kBlockEdges / 32];
#pragma unroll
      for (int j = 0; j < kBlockEdges / 32; ++j) {
        const int k = lane + 32 * j;
        vals[j] = k < d.n_real ? stage_value<APP>(src_val, src_con, col_s, w_s, k) : identity<APP>();
      }
#pragma unroll
      for (int j = 0; j < kBlockEdges / 32; ++j) vbuf[lane + 32 * j] = vals[j];
    }
    __syncwarp();
    // Phase 2: fold.
    if (d.type < 2) {
      // Lane per vertex, in edge order (the reference's summation order).
      bool act = false;
      if (valid) {
        T acc;
        if constexpr (is_pr<APP>()) acc = 0.f;
        else acc = old;
#pragma unroll 4
        for (int k = beg; k < end; ++k) acc = combine<APP>(acc, vbuf[k]);
        la.edges += end - beg;
        act = apply_vertex<APP>(c, v, acc, old, od, dst_val, dst_con, la);
      }
      set_active_bit(a.bm, v, act);
    } else {
      // Heavy chunk: fixed-shape tree over the chunk, then chunk partials in order.
      T acc = identity<APP>();
#pragma unroll
      for (int j = 0; j < kBlockEdges / 32; ++j) acc = combine<APP>(acc, vbuf[lane + 32 * j]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc = combine<APP>(acc, __shfl_xor_sync(0xffffffffu, acc, o));
      if (lane == 0) {
        const int4 H = a.heavy[d.first];
        const int hv = H.x;
        T tot = acc;
        la.edges += d.n_real;
        T* part = static_cast<T*>(a.partial);
        bool last = H.y == 1;
        if (!last) {
          part[H.z + d.aux] = tot;
          __threadfence();
          last = atomicAdd(a.hticket + d.first, 1u) == static_cast<unsigned>(H.y) - 1;
        }
        if (last) {
          __threadfence();
          if (H.y > 1) {
            const volatile T* vp = part;
            tot = identity<APP>();
            for (int i = 0; i < H.y; ++i) tot = combine<APP>(tot, vp[H.z + i]);
            a.hticket[d.first] = 0;
          }
          const T hold = static_cast<const T*>(src_val)[hv];
          const int32_t hod = is_pr<APP>() ? a.outdeg[hv] : 0;
          T fin;
          if constexpr (is_pr<APP>()) fin = tot;
          else fin = combine<APP>(hold, tot);
          if (apply_vertex<APP>(c, hv, fin, hold, hod, dst_val, dst_con, la))
            atomicOr(a.bm + (hv >> 5), 1u << (hv & 31));
        }
      }
    }
    __syncwarp();  // stage and value buffer free for the next block
    st ^= 1;
  }
  if (err && lane == 0) {
    atomicExch(&ctl->error, 1);
    // Let this warp's issued copies land before it exits (bounded).
    for (int s2 = 0; s2 < 2; ++s2) {
      uint32_t spins = 0;
      while (!mbar_try_wait(&wbar[s2], parity[s2]) && ++spins < kWaitSpins) {
      }
    }
  }
  __syncthreads();
  flush_block(ctl, la);
}

}  // namespace gx

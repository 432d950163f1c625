// Internal helpers shared by the host and device translation units.
#pragma once
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/gx.h"

#ifdef __CUDACC__
#define GX_HD __host__ __device__
#else
#define GX_HD
#endif

namespace gx {

// Records `msg` as the thread's last error and returns `st`.
gx_status fail(gx_status st, const char* fmt, ...);

// 1-D little-endian .npy files of 4-byte elements (descr "<i4", "<u4" or
// "<f4").  open_npy_4 leaves `*out` at the first element and sets `*kind` to
// 'i', 'u' or 'f'.
bool write_npy_4(const std::string& path, const void* data, int64_t n, const char* descr);
gx_status open_npy_4(const std::string& path, FILE** out, int64_t* n, char* kind);

// splitmix64 finaliser (Steele, Lea, Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014): a bijective 64-bit mixer used as a
// counter-based generator, so any element can be produced independently.
GX_HD inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// SSSP weight of edge u->v in [1,255]: a pure function of (seed, u, v).
GX_HD inline uint32_t edge_weight(uint64_t seed, int32_t u, int32_t v) {
  uint64_t h = mix64(seed ^ mix64((static_cast<uint64_t>(static_cast<uint32_t>(u)) << 32) |
                                  static_cast<uint32_t>(v)));
  return 1u + static_cast<uint32_t>(h % 255u);
}

}  // namespace gx

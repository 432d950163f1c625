// Host-side graph construction and the reference's on-disk shard format.
//
// The reference prepares graphs offline with a Spark job
// (GraphMP/tools/format_spark.py): in-degree count (:51-57), edge-balanced
// destination-range partitioner (:91-108), per-partition CSR-by-destination
// written as one int32 array [E, len(indices), len(indptr), start, end,
// indices..., indptr...] (:137-157).  The engine reads those as
// `{p}.edge.npy` (GraphMP/system/Comp.h:33-42) plus `vertexout.npy`
// (GraphMP/system/GraphPS.h:162-169).  This file produces and reads the same
// layout from C++ with OpenMP, with no Spark/HDFS.
#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gx_internal.h"

namespace gx {

static thread_local std::string g_last_error;

gx_status fail(gx_status st, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return st;
}

namespace {

std::string shard_dir(const char* dir) {
  std::string d(dir);
  if (!d.empty() && d.back() != '/') d.push_back('/');
  return d;
}

// Parallel exclusive prefix sum over int64 counts: out[0] = 0,
// out[i+1] = out[i] + cnt[i].  `cnt` and `out` may not alias.
void exclusive_scan(const int64_t* cnt, int64_t n, int64_t* out) {
  int nt = omp_get_max_threads();
  std::vector<int64_t> part(nt + 1, 0);
#pragma omp parallel num_threads(nt)
  {
    int t = omp_get_thread_num();
    int64_t lo = n * t / nt, hi = n * (t + 1) / nt, s = 0;
    for (int64_t i = lo; i < hi; ++i) s += cnt[i];
    part[t + 1] = s;
#pragma omp barrier
#pragma omp single
    for (int i = 0; i < nt; ++i) part[i + 1] += part[i];
    int64_t run = part[t];
    for (int64_t i = lo; i < hi; ++i) {
      out[i] = run;
      run += cnt[i];
    }
  }
  out[n] = part[nt];
}

// ---- .npy (format version 1.0, 1-D little-endian 4-byte elements) ----

bool write_npy_i32(const std::string& path, const int32_t* data, int64_t n) {
  return write_npy_4(path, data, n, "<i4");
}

// Opens a 1-D int32 .npy and leaves `f` positioned at the first element.
gx_status open_npy_i32(const std::string& path, FILE** out, int64_t* n) {
  char descr = 0;
  gx_status st = open_npy_4(path, out, n, &descr);
  if (st != GX_OK) return st;
  if (descr != 'i') {
    fclose(*out);
    *out = nullptr;
    return fail(GX_ERR_FORMAT, "%s: expected a 1-D little-endian int32 array", path.c_str());
  }
  return GX_OK;
}

gx_status read_npy_i32(const std::string& path, std::vector<int32_t>* v) {
  FILE* f;
  int64_t n;
  gx_status st = open_npy_i32(path, &f, &n);
  if (st != GX_OK) return st;
  v->resize(static_cast<size_t>(n));
  size_t got = n ? fread(v->data(), sizeof(int32_t), static_cast<size_t>(n), f) : 0;
  fclose(f);
  if (got != static_cast<size_t>(n)) return fail(GX_ERR_IO, "%s: short read", path.c_str());
  return GX_OK;
}

}  // namespace

bool write_npy_4(const std::string& path, const void* data, int64_t n, const char* descr) {
  char dict[160];
  int dl = snprintf(dict, sizeof(dict), "{'descr': '%s', 'fortran_order': False, 'shape': (%lld,), }", descr,
                    static_cast<long long>(n));
  int total = 10 + dl + 1;
  int pad = (64 - total % 64) % 64;
  int hlen = dl + pad + 1;
  std::string hdr("\x93NUMPY\x01\x00", 8);
  hdr.push_back(static_cast<char>(hlen & 0xff));
  hdr.push_back(static_cast<char>((hlen >> 8) & 0xff));
  hdr.append(dict, dl);
  hdr.append(pad, ' ');
  hdr.push_back('\n');
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = fwrite(hdr.data(), 1, hdr.size(), f) == hdr.size();
  if (ok && n > 0) ok = fwrite(data, 4, static_cast<size_t>(n), f) == static_cast<size_t>(n);
  ok = (fclose(f) == 0) && ok;
  return ok;
}

// Opens a 1-D little-endian .npy of 4-byte elements (int32, uint32 or
// float32; `kind` gets 'i', 'u' or 'f') positioned at the first element.
gx_status open_npy_4(const std::string& path, FILE** out, int64_t* n, char* kind) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return fail(GX_ERR_IO, "cannot open %s: %s", path.c_str(), strerror(errno));
  unsigned char pre[10];
  if (fread(pre, 1, 10, f) != 10 || memcmp(pre, "\x93NUMPY", 6) != 0) {
    fclose(f);
    return fail(GX_ERR_FORMAT, "%s: not a .npy file", path.c_str());
  }
  uint32_t hlen;
  if (pre[6] == 1) {
    hlen = pre[8] | (pre[9] << 8);
  } else {
    unsigned char ext[2];
    if (fread(ext, 1, 2, f) != 2) {
      fclose(f);
      return fail(GX_ERR_FORMAT, "%s: short header", path.c_str());
    }
    hlen = pre[8] | (pre[9] << 8) | (ext[0] << 16) | (ext[1] << 24);
  }
  std::string h(hlen, '\0');
  if (hlen > (1u << 20) || fread(&h[0], 1, hlen, f) != hlen) {
    fclose(f);
    return fail(GX_ERR_FORMAT, "%s: short header", path.c_str());
  }
  char k = 0;
  if (h.find("'<i4'") != std::string::npos || h.find("'|i4'") != std::string::npos) k = 'i';
  else if (h.find("'<u4'") != std::string::npos || h.find("'|u4'") != std::string::npos) k = 'u';
  else if (h.find("'<f4'") != std::string::npos) k = 'f';
  bool fortran = h.find("'fortran_order': True") != std::string::npos;
  size_t lp = h.find('('), rp = h.find(')');
  if (!k || fortran || lp == std::string::npos || rp == std::string::npos) {
    fclose(f);
    return fail(GX_ERR_FORMAT, "%s: expected a 1-D little-endian array of 4-byte elements", path.c_str());
  }
  *kind = k;
  std::string shape = h.substr(lp + 1, rp - lp - 1);
  if (std::count(shape.begin(), shape.end(), ',') > 1 ||
      (shape.find(',') != std::string::npos && shape.find_first_not_of(" ", shape.find(',') + 1) != std::string::npos)) {
    fclose(f);
    return fail(GX_ERR_FORMAT, "%s: expected a 1-D array, shape (%s)", path.c_str(), shape.c_str());
  }
  *n = atoll(shape.c_str());
  *out = f;
  return GX_OK;
}

}  // namespace gx

using namespace gx;

extern "C" {

gx_status gx_read_values_npy(const char* path, int64_t n, void* out) {
  if (!path || n < 0 || (n > 0 && !out)) return fail(GX_ERR_INVALID, "gx_read_values_npy: bad arguments");
  FILE* f = nullptr;
  int64_t m = 0;
  char kind = 0;
  gx_status st = open_npy_4(path, &f, &m, &kind);
  if (st != GX_OK) return st;
  if (m != n) {
    fclose(f);
    return fail(GX_ERR_FORMAT, "%s: %lld elements, expected %lld", path, static_cast<long long>(m),
                static_cast<long long>(n));
  }
  const bool ok = n == 0 || fread(out, 4, static_cast<size_t>(n), f) == static_cast<size_t>(n);
  fclose(f);
  if (!ok) return fail(GX_ERR_FORMAT, "%s: short data", path);
  return GX_OK;
}


const char* gx_last_error(void) { return g_last_error.c_str(); }

gx_status gx_rmat_edges(int32_t scale, int64_t n, double a, double b, double c, uint64_t seed,
                        int64_t first, int32_t* src, int32_t* dst) {
  if (scale < 1 || scale > 30 || n < 0 || first < 0 || (n > 0 && (!src || !dst)))
    return fail(GX_ERR_INVALID, "gx_rmat_edges: bad arguments (scale %d, n %lld)", scale,
                static_cast<long long>(n));
  if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0 + 1e-12)
    return fail(GX_ERR_INVALID, "gx_rmat_edges: bad quadrant probabilities");
  // Quadrant thresholds on a 16-bit uniform draw per level: a = (row 0,
  // col 0), b = (0,1), c = (1,0), d = (1,1), row = source, col = destination.
  const uint32_t ta = static_cast<uint32_t>(std::llround(a * 65536.0));
  const uint32_t tb = ta + static_cast<uint32_t>(std::llround(b * 65536.0));
  const uint32_t tc = tb + static_cast<uint32_t>(std::llround(c * 65536.0));
  const uint64_t key0 = mix64(seed ^ 0x5ca1ab1e0ddba11ull);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < n; ++k) {
    const uint64_t i = static_cast<uint64_t>(first + k);
    const uint64_t key = key0 ^ (i * 0xd1b54a32d192ed03ull);
    uint32_t s = 0, d = 0;
    for (int lv = 0; lv < scale; lv += 4) {
      const uint64_t h = mix64(key + static_cast<uint64_t>(lv / 4 + 1) * 0x9e3779b97f4a7c15ull);
      for (int j = 0; j < 4 && lv + j < scale; ++j) {
        const uint32_t u = static_cast<uint32_t>(h >> (16 * j)) & 0xffffu;
        const uint32_t bit = 1u << (scale - 1 - (lv + j));
        if (u < ta) {
        } else if (u < tb) {
          d |= bit;
        } else if (u < tc) {
          s |= bit;
        } else {
          s |= bit;
          d |= bit;
        }
      }
    }
    src[k] = static_cast<int32_t>(s);
    dst[k] = static_cast<int32_t>(d);
  }
  return GX_OK;
}

gx_status gx_build_csc(int32_t V, int64_t n, const int32_t* src, const int32_t* dst, int32_t flags,
                       int64_t* off, int32_t* col, int64_t* n_out) {
  if (V < 0 || n < 0 || !off || (n > 0 && (!src || !dst || !col)) || !n_out)
    return fail(GX_ERR_INVALID, "gx_build_csc: bad arguments");
  const bool drop_self = flags & GX_BUILD_DROP_SELF;
  const bool dedup = flags & GX_BUILD_DEDUP;
  const bool sym = flags & GX_BUILD_SYMMETRIZE;
  std::vector<int64_t> cnt(static_cast<size_t>(V) + 1, 0);
  std::atomic<int> bad{0};
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    int32_t s = src[i], d = dst[i];
    if (s < 0 || s >= V || d < 0 || d >= V) {
      bad.store(1, std::memory_order_relaxed);
      continue;
    }
    if (drop_self && s == d) continue;
    __atomic_fetch_add(&cnt[d], 1, __ATOMIC_RELAXED);
    if (sym) __atomic_fetch_add(&cnt[s], 1, __ATOMIC_RELAXED);
  }
  if (bad.load()) return fail(GX_ERR_INVALID, "gx_build_csc: vertex id outside [0, %d)", V);
  exclusive_scan(cnt.data(), V, off);
  // cnt becomes the per-destination write cursor.
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < V; ++v) cnt[v] = off[v];
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    int32_t s = src[i], d = dst[i];
    if (drop_self && s == d) continue;
    col[__atomic_fetch_add(&cnt[d], 1, __ATOMIC_RELAXED)] = s;
    if (sym) col[__atomic_fetch_add(&cnt[s], 1, __ATOMIC_RELAXED)] = d;
  }
  // Sources ascending within each destination (scipy's canonical CSR order,
  // which format_spark.py's csr_matrix produces), then optional dedup.
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t v = 0; v < V; ++v) {
    int32_t* b = col + off[v];
    int32_t* e = col + off[v + 1];
    std::sort(b, e);
    cnt[v] = dedup ? (std::unique(b, e) - b) : (e - b);
  }
  if (dedup) {
    std::vector<int64_t> noff(static_cast<size_t>(V) + 1);
    exclusive_scan(cnt.data(), V, noff.data());
    // new offsets never exceed old ones, so an in-order forward move is safe.
    for (int64_t v = 0; v < V; ++v)
      if (noff[v] != off[v] && cnt[v] > 0)
        memmove(col + noff[v], col + off[v], static_cast<size_t>(cnt[v]) * sizeof(int32_t));
    memcpy(off, noff.data(), (static_cast<size_t>(V) + 1) * sizeof(int64_t));
  }
  *n_out = off[V];
  return GX_OK;
}

gx_status gx_partition_bounds(int32_t V, const int64_t* off, int32_t P, int32_t* bounds) {
  if (V < 0 || P < 1 || !off || !bounds) return fail(GX_ERR_INVALID, "gx_partition_bounds: bad arguments");
  const int64_t E = off[V];
  const int64_t per = (E + P - 1) / P;  // math.ceil(edge_num/partition_num), format_spark.py:91
  bounds[0] = 0;
  for (int32_t i = 1; i < P; ++i) {
    // np.argmax(cumsum >= per*i) (format_spark.py:100-101); when no vertex
    // reaches the target the Spark job would get 0, here the range closes at V.
    const int64_t target = per * i;
    int32_t j = static_cast<int32_t>(std::lower_bound(off, off + V + 1, target) - off);
    bounds[i] = std::max(bounds[i - 1], std::min(j, V));
  }
  bounds[P] = V;
  return GX_OK;
}

gx_status gx_out_degree(int32_t V, const int64_t* off, const int32_t* col, int32_t* outdeg) {
  if (V < 0 || !off || !outdeg) return fail(GX_ERR_INVALID, "gx_out_degree: bad arguments");
  memset(outdeg, 0, sizeof(int32_t) * static_cast<size_t>(V));
  const int64_t E = off[V];
  std::atomic<int> bad{0};
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < E; ++k) {
    int32_t u = col[k];
    if (u < 0 || u >= V) {
      bad.store(1, std::memory_order_relaxed);
      continue;
    }
    __atomic_fetch_add(&outdeg[u], 1, __ATOMIC_RELAXED);
  }
  if (bad.load()) return fail(GX_ERR_INVALID, "gx_out_degree: source id outside [0, %d)", V);
  return GX_OK;
}

gx_status gx_write_shards(const char* dir, int32_t V, int32_t P, const int32_t* bounds, const int64_t* off,
                          const int32_t* col, const int32_t* outdeg) {
  if (!dir || V < 0 || P < 1 || !bounds || !off || (off[V] > 0 && !col) || !outdeg)
    return fail(GX_ERR_INVALID, "gx_write_shards: bad arguments");
  const std::string d = shard_dir(dir);
  std::atomic<int> err{0};
  std::string err_path;
#pragma omp parallel for schedule(dynamic, 1)
  for (int32_t p = 0; p < P; ++p) {
    const int32_t s = bounds[p], e = bounds[p + 1];
    const int64_t lo = off[s], ne = off[e] - lo, nv = e - s;
    if (s < 0 || e < s || e > V || ne + nv + 6 > INT32_MAX) {
      err.store(1);
      continue;
    }
    std::vector<int32_t> blob(static_cast<size_t>(5 + ne + nv + 1));
    blob[0] = static_cast<int32_t>(ne);
    blob[1] = static_cast<int32_t>(ne);
    blob[2] = static_cast<int32_t>(nv + 1);
    blob[3] = s;
    blob[4] = e;
    if (ne) memcpy(&blob[5], col + lo, static_cast<size_t>(ne) * sizeof(int32_t));
    int32_t* ip = &blob[static_cast<size_t>(5 + ne)];
    for (int64_t i = 0; i <= nv; ++i) ip[i] = static_cast<int32_t>(off[s + i] - lo);
    if (!write_npy_i32(d + std::to_string(p) + ".edge.npy", blob.data(), static_cast<int64_t>(blob.size()))) {
#pragma omp critical
      err_path = d + std::to_string(p) + ".edge.npy";
      err.store(2);
    }
  }
  if (err.load() == 1) return fail(GX_ERR_INVALID, "gx_write_shards: a shard exceeds the int32 layout");
  if (err.load() == 2) return fail(GX_ERR_IO, "gx_write_shards: cannot write %s", err_path.c_str());
  std::vector<int32_t> indeg(static_cast<size_t>(V));
  for (int64_t v = 0; v < V; ++v) indeg[v] = static_cast<int32_t>(off[v + 1] - off[v]);
  if (!write_npy_i32(d + "vertexout.npy", outdeg, V) || !write_npy_i32(d + "vertexin.npy", indeg.data(), V))
    return fail(GX_ERR_IO, "gx_write_shards: cannot write vertex files in %s", d.c_str());
  return GX_OK;
}

gx_status gx_read_shards(const char* dir, int32_t V, int32_t P, int32_t* bounds, int64_t* off, int32_t* col,
                         int32_t* outdeg, int64_t* E_out) {
  if (!dir || V < 0 || P < 1 || !E_out) return fail(GX_ERR_INVALID, "gx_read_shards: bad arguments");
  const std::string d = shard_dir(dir);
  // Pass 1: headers only -> sizes and ranges.
  std::vector<int32_t> hdr(static_cast<size_t>(P) * 5);
  for (int32_t p = 0; p < P; ++p) {
    const std::string path = d + std::to_string(p) + ".edge.npy";
    FILE* f;
    int64_t n;
    gx_status st = open_npy_i32(path, &f, &n);
    if (st != GX_OK) return st;
    size_t got = fread(&hdr[static_cast<size_t>(p) * 5], sizeof(int32_t), 5, f);
    fclose(f);
    const int32_t* h = &hdr[static_cast<size_t>(p) * 5];
    if (got != 5 || h[1] < 0 || h[2] < 1 || n != 5ll + h[1] + h[2] || h[2] != h[4] - h[3] + 1)
      return fail(GX_ERR_FORMAT, "%s: header [%d %d %d %d %d] does not match %lld elements", path.c_str(),
                  got > 0 ? h[0] : -1, h[1], h[2], h[3], h[4], static_cast<long long>(n));
    const int32_t expect_start = p == 0 ? 0 : hdr[static_cast<size_t>(p - 1) * 5 + 4];
    if (h[3] != expect_start || h[4] < h[3] || h[4] > V || (p == P - 1 && h[4] != V))
      return fail(GX_ERR_FORMAT, "%s: destination range [%d,%d) does not continue [.., %d) over V=%d", path.c_str(),
                  h[3], h[4], expect_start, V);
  }
  int64_t E = 0;
  for (int32_t p = 0; p < P; ++p) E += hdr[static_cast<size_t>(p) * 5 + 1];
  *E_out = E;
  if (!off && !col) return GX_OK;
  if (!off || !col || !bounds) return fail(GX_ERR_INVALID, "gx_read_shards: bounds/off/col required");
  std::vector<int64_t> base(static_cast<size_t>(P) + 1, 0);
  for (int32_t p = 0; p < P; ++p) base[p + 1] = base[p] + hdr[static_cast<size_t>(p) * 5 + 1];
  for (int32_t p = 0; p < P; ++p) bounds[p] = hdr[static_cast<size_t>(p) * 5 + 3];
  bounds[P] = V;
  std::atomic<int> err{0};
  std::string err_msg;
#pragma omp parallel for schedule(dynamic, 1)
  for (int32_t p = 0; p < P; ++p) {
    std::vector<int32_t> blob;
    const std::string path = d + std::to_string(p) + ".edge.npy";
    gx_status st = read_npy_i32(path, &blob);
    const int32_t* h = blob.data();
    bool ok = st == GX_OK;
    if (ok) {
      const int32_t ni = h[1], np1 = h[2], s = h[3];
      const int32_t* idx = h + 5;
      const int32_t* ip = h + 5 + ni;
      ok = ip[0] == 0 && ip[np1 - 1] == ni;
      for (int32_t i = 0; ok && i + 1 < np1; ++i) ok = ip[i] <= ip[i + 1];
      for (int32_t k = 0; ok && k < ni; ++k) ok = idx[k] >= 0 && idx[k] < V;
      if (ok) {
        memcpy(col + base[p], idx, static_cast<size_t>(ni) * sizeof(int32_t));
        for (int32_t i = 0; i + 1 < np1; ++i) off[s + i] = base[p] + ip[i];
      }
    }
    if (!ok) {
#pragma omp critical
      err_msg = st == GX_OK ? path + ": indptr/indices out of range" : std::string(gx_last_error());
      err.store(1);
    }
  }
  if (err.load()) return fail(GX_ERR_FORMAT, "%s", err_msg.c_str());
  off[V] = E;
  if (outdeg) {
    std::vector<int32_t> od;
    gx_status st = read_npy_i32(d + "vertexout.npy", &od);
    if (st != GX_OK) return st;
    if (od.size() < static_cast<size_t>(V))
      return fail(GX_ERR_FORMAT, "%svertexout.npy: %zu entries for V=%d", d.c_str(), od.size(), V);
    memcpy(outdeg, od.data(), sizeof(int32_t) * static_cast<size_t>(V));
  }
  return GX_OK;
}

gx_status gx_convert_edge_list(const char* path, int32_t V, int32_t P, int32_t flags, const char* out_dir,
                               int64_t* n_edges_out) {
  if (!path || !out_dir || V < 1 || P < 1) return fail(GX_ERR_INVALID, "gx_convert_edge_list: bad arguments");
  FILE* f = fopen(path, "rb");
  if (!f) return fail(GX_ERR_IO, "cannot open %s: %s", path, strerror(errno));
  fseek(f, 0, SEEK_END);
  const long size = ftell(f);
  fseek(f, 0, SEEK_SET);
  std::string text(static_cast<size_t>(size > 0 ? size : 0), '\0');
  if (size > 0 && fread(&text[0], 1, static_cast<size_t>(size), f) != static_cast<size_t>(size)) {
    fclose(f);
    return fail(GX_ERR_IO, "%s: short read", path);
  }
  fclose(f);
  // Split at line starts so threads parse independent ranges; '#' and '%'
  // lines are comments.  Each line holds "src dst" (whitespace separated),
  // the input format of GraphMP/tools/format_spark.py:51-53,111-113.
  const int nt = omp_get_max_threads();
  std::vector<size_t> cut(nt + 1, text.size());
  cut[0] = 0;
  for (int t = 1; t < nt; ++t) {
    size_t c = text.size() * t / nt;
    while (c < text.size() && text[c - 1] != '\n') ++c;
    cut[t] = c;
  }
  std::vector<std::vector<int32_t>> srcs(nt), dsts(nt);
  std::atomic<int> bad{0};
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    const char* p = text.data() + cut[t];
    const char* end = text.data() + cut[t + 1];
    while (p < end) {
      const char* eol = static_cast<const char*>(memchr(p, '\n', end - p));
      if (!eol) eol = end;
      const char* q = p;
      while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
      if (q < eol && *q != '#' && *q != '%') {
        char* e1 = nullptr;
        const long long a = strtoll(q, &e1, 10);
        char* e2 = nullptr;
        const long long b = strtoll(e1, &e2, 10);
        if (e1 == q || e2 == e1 || a < 0 || b < 0 || a >= V || b >= V) {
          bad.store(1);
        } else {
          srcs[t].push_back(static_cast<int32_t>(a));
          dsts[t].push_back(static_cast<int32_t>(b));
        }
      }
      p = eol + 1;
    }
  }
  if (bad.load()) return fail(GX_ERR_FORMAT, "%s: a line is not \"src dst\" with ids in [0, %d)", path, V);
  std::vector<int32_t> src, dst;
  for (int t = 0; t < nt; ++t) {
    src.insert(src.end(), srcs[t].begin(), srcs[t].end());
    dst.insert(dst.end(), dsts[t].begin(), dsts[t].end());
  }
  const int64_t n = static_cast<int64_t>(src.size());
  std::vector<int64_t> off(static_cast<size_t>(V) + 1);
  std::vector<int32_t> col(static_cast<size_t>(flags & GX_BUILD_SYMMETRIZE ? 2 * n : n) + 1);
  int64_t E = 0;
  gx_status st = gx_build_csc(V, n, src.data(), dst.data(), flags, off.data(), col.data(), &E);
  if (st != GX_OK) return st;
  std::vector<int32_t> outdeg(static_cast<size_t>(V)), bounds(static_cast<size_t>(P) + 1);
  if ((st = gx_out_degree(V, off.data(), col.data(), outdeg.data())) != GX_OK) return st;
  if ((st = gx_partition_bounds(V, off.data(), P, bounds.data())) != GX_OK) return st;
  if ((st = gx_write_shards(out_dir, V, P, bounds.data(), off.data(), col.data(), outdeg.data())) != GX_OK) return st;
  if (n_edges_out) *n_edges_out = E;
  return GX_OK;
}

gx_status gx_edge_weights(uint64_t seed, int32_t V, const int64_t* off, const int32_t* col, uint32_t* w) {
  if (V < 0 || !off || (off[V] > 0 && (!col || !w))) return fail(GX_ERR_INVALID, "gx_edge_weights: bad arguments");
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t v = 0; v < V; ++v)
    for (int64_t k = off[v]; k < off[v + 1]; ++k) w[k] = edge_weight(seed, col[k], static_cast<int32_t>(v));
  return GX_OK;
}

}  // extern "C"

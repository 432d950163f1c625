/* snappy is only reached at edge-cache compression level 1
 * (GraphMP/system/Global.h:133-147,176-187); the oracle recipe builds with
 * the cache off or uncompressed, so these abort if ever reached.  Test
 * infrastructure only. */
#ifndef GX_STUB_SNAPPY_H
#define GX_STUB_SNAPPY_H
#include <cstdlib>
#include <cstddef>
namespace snappy {
static inline size_t MaxCompressedLength(size_t n) { abort(); return n; }
static inline void RawCompress(const char*, size_t, char*, size_t*) { abort(); }
static inline bool RawUncompress(const char*, size_t, char*) { abort(); return false; }
}
#endif

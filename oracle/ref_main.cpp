// Harness that runs the reference's own GraphMP app (compiled from the
// reference sources by oracle/Makefile) on a shard directory and dumps the
// final vertex messages.  Test infrastructure only: it produces the golden
// vectors under tests/golden/ that pin the oracle; nothing in the product
// links or calls it.
//
// Build: see oracle/Makefile (GX_REF_APP names the app source, GX_REF_T its
// value type).  Usage:
//   ref_<app> <shard_dir/> <V> <P> <max_iter> <out.bin> [threads] [source]
// The reference driver is GraphPS<T>::init + run (GraphMP/system/GraphPS.h:77,171);
// the app classes are GraphMP/app/{pagerank,sssp,cc}.cpp.
#include <cstdio>
#include <cstdlib>
#include <string>
#define main gx_reference_app_main
#include GX_REF_APP
#undef main

typedef GX_REF_T ValueT;

#ifdef GX_REF_SSSP
// The reference hard-codes source vertex 1 (GraphMP/app/sssp.cpp:72); this
// subclass only moves the source, as the reference's own commented-out line
// (sssp.cpp:73) does by hand.
struct SourcedApp : public PagerankPS<ValueT> {
  int32_t source = 1;
  void init_vertex() {
    PagerankPS<ValueT>::init_vertex();
    if (this->_VertexNum > 1) this->_VertexMsg[1] = GPS_INF;
    this->_VertexMsg[source] = 0;
  }
};
#else
struct SourcedApp : public PagerankPS<ValueT> { int32_t source = 0; };
#endif

int main(int argc, char** argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: %s dir/ V P max_iter out.bin [threads] [source]\n", argv[0]);
    return 2;
  }
  std::string dir = argv[1];
  int32_t V = atoi(argv[2]), P = atoi(argv[3]), iters = atoi(argv[4]);
  const char* out = argv[5];
  int threads = argc > 6 ? atoi(argv[6]) : 0;
  init_workers();
  SourcedApp pg;
  if (argc > 7) pg.source = atoi(argv[7]);
  auto t0 = std::chrono::steady_clock::now();
  pg.init(dir, V, P, iters);
  if (threads > 0 && threads <= CMPNUM) pg._ThreadNum = threads;
  pg.run();
  auto t1 = std::chrono::steady_clock::now();
  FILE* f = fopen(out, "wb");
  if (!f) { perror(out); return 1; }
  fwrite(pg._VertexMsg.data(), sizeof(ValueT), (size_t)V, f);
  fclose(f);
  fprintf(stderr, "GX_REF_DONE wall_ms=%.3f threads=%d\n",
          std::chrono::duration<double, std::milli>(t1 - t0).count(), pg._ThreadNum);
  return 0;
}

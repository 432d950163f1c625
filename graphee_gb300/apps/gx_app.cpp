// Command-line drivers with the shape of the reference's app mains
// (GraphMP/app/pagerank.cpp:86-104, sssp.cpp:77-94, cc.cpp:77-94), which
// hard-code init(path, V, P, maxIter) and run(); here those four come from
// the command line, and the result is written as raw values.
//
//   gx_app pagerank <shard_dir/> <V> <P> <max_iter> [out.bin]
//   gx_app sssp     <shard_dir/> <V> <P> <max_iter> [out.bin] [source]
//   gx_app cc       <shard_dir/> <V> <P> <max_iter> [out.bin]
//   gx_app tc       <shard_dir/> <V> <P> 0          (symmetric shards)
//   gx_app convert  <edges.tsv> <V> <P> <out_dir/>  (edge list -> shards)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "gx_graphps.hpp"

template <class App>
static int run_app(App& app, int argc, char** argv, const char* name) {
  app.init(argv[2], atoi(argv[3]), atoi(argv[4]), atoi(argv[5]));
  app.run();
  fprintf(stderr, "%s: %d supersteps, %.3f ms, %lld edges read\n", name, app._Stats.iterations,
          app._Stats.ms_total, static_cast<long long>(app._Stats.edges_scanned));
  if (argc > 6) {
    FILE* f = fopen(argv[6], "wb");
    if (!f) {
      perror(argv[6]);
      return 1;
    }
    fwrite(app._VertexMsg.data(), sizeof(app._VertexMsg[0]), app._VertexMsg.size(), f);
    fclose(f);
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 6) {
    fprintf(stderr,
            "usage: %s pagerank|sssp|cc|tc <shard_dir/> <V> <P> <max_iter> [out.bin] [source]\n"
            "       %s convert <edges.tsv> <V> <P> <out_dir/>\n",
            argv[0], argv[0]);
    return 2;
  }
  const std::string app = argv[1];
  try {
    if (app == "pagerank") {
      gx::PagerankPS<float> pg;
      return run_app(pg, argc, argv, "pagerank");
    }
    if (app == "sssp") {
      gx::SsspPS<int32_t> pg;
      if (argc > 7) pg._Source = atoi(argv[7]);
      return run_app(pg, argc, argv, "sssp");
    }
    if (app == "cc") {
      gx::CcPS<int32_t> pg;
      return run_app(pg, argc, argv, "cc");
    }
    if (app == "convert") {
      int64_t kept = 0;
      gx::check(gx_convert_edge_list(argv[2], atoi(argv[3]), atoi(argv[4]), GX_BUILD_DROP_SELF | GX_BUILD_DEDUP,
                                     argv[5], &kept),
                "gx_convert_edge_list");
      printf("%lld\n", static_cast<long long>(kept));
      return 0;
    }
    if (app == "tc") {
      gx_engine* e = nullptr;
      gx::check(gx_create(nullptr, &e), "gx_create");
      gx::check(gx_load_shards(e, argv[2], atoi(argv[3]), atoi(argv[4])), "gx_load_shards");
      uint64_t t = 0;
      gx_run_stats st;
      gx::check(gx_triangle_count(e, &t, &st), "gx_triangle_count");
      printf("%llu\n", static_cast<unsigned long long>(t));
      gx_destroy(e);
      return 0;
    }
  } catch (const gx::Error& err) {
    fprintf(stderr, "%s\n", err.what());
    return 1;
  }
  fprintf(stderr, "unknown app %s\n", app.c_str());
  return 2;
}

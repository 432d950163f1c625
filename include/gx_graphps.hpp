// gx_graphps.hpp — C++ mirror of GraphMP's operator interface over the gx C ABI.
//
// The reference's apps subclass GraphPS<T> (GraphMP/system/GraphPS.h:22-63),
// set the vertex program through the _comp function pointer, override
// init_vertex(), then call init(path, V, P, maxIter) and run().  This header
// keeps that shape so an app ports by changing its base class: the vertex
// program is chosen by the app class (PagerankPS / SsspPS / CcPS below,
// mirroring GraphMP/app/{pagerank,sssp,cc}.cpp), init_vertex() may fill
// _VertexMsg to replace the program's own initialisation, and after run()
// _VertexMsg holds the result.  Errors throw gx::Error (the reference
// asserts or aborts instead, e.g. cnpy.h:131-134).
#ifndef GX_GRAPHPS_HPP_
#define GX_GRAPHPS_HPP_

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "gx.h"

namespace gx {

struct Error : std::runtime_error {
  gx_status status;
  Error(gx_status s, const std::string& where)
      : std::runtime_error(where + ": " + gx_last_error()), status(s) {}
};

inline void check(gx_status s, const char* where) {
  if (s != GX_OK) throw Error(s, where);
}

template <class T>
class GraphPS {
 public:
  std::string _DataPath;
  int32_t _VertexNum = 0;
  int32_t _PartitionNum = 0;
  int32_t _MaxIteration = 0;
  std::vector<T> _VertexMsg;  // after run(): the final messages (GraphPS.h:49)
  gx_run_stats _Stats{};

  explicit GraphPS(gx_app app, const gx_config* cfg = nullptr) : app_(app) {
    check(gx_create(cfg, &engine_), "gx_create");
  }
  virtual ~GraphPS() { gx_destroy(engine_); }
  GraphPS(const GraphPS&) = delete;
  GraphPS& operator=(const GraphPS&) = delete;

  // GraphPS<T>::init (GraphPS.h:77): shard directory ending in '/', |V|, #shards, max iterations.
  void init(std::string DataPath, const int32_t VertexNum, const int32_t PartitionNum,
            const int32_t MaxIteration = 10) {
    _DataPath = DataPath;
    _VertexNum = VertexNum;
    _PartitionNum = PartitionNum;
    _MaxIteration = MaxIteration;
    check(gx_load_shards(engine_, DataPath.c_str(), VertexNum, PartitionNum), "gx_load_shards");
  }

  // GraphPS.h:60.  Leave _VertexMsg empty to keep the vertex program's own
  // initialisation; fill it with V values to start from them.
  virtual void init_vertex() {}

  // GraphPS<T>::run (GraphPS.h:171).
  void run() {
    _VertexMsg.clear();
    init_vertex();
    gx_run_params p;
    gx_run_params_default(&p, app_);
    p.max_iter = _MaxIteration;
    configure(&p);
    if (!_VertexMsg.empty()) {
      if (static_cast<int32_t>(_VertexMsg.size()) != _VertexNum)
        throw std::invalid_argument("init_vertex: _VertexMsg must hold _VertexNum values");
      check(gx_set_init(engine_, _VertexMsg.data()), "gx_set_init");
      p.use_init = 1;
    }
    check(gx_run(engine_, &p, &_Stats), "gx_run");
    _VertexMsg.assign(_VertexNum, T());
    check(gx_get_values(engine_, _VertexMsg.data()), "gx_get_values");
  }

  gx_engine* engine() { return engine_; }

 protected:
  virtual void configure(gx_run_params*) {}

 private:
  gx_app app_;
  gx_engine* engine_ = nullptr;
};

// GraphMP/app/pagerank.cpp: PagerankPS<float>.
template <class T = float>
class PagerankPS : public GraphPS<T> {
 public:
  explicit PagerankPS(const gx_config* cfg = nullptr) : GraphPS<T>(GX_APP_PAGERANK_REF, cfg) {}
};

// GraphMP/app/sssp.cpp: unit-weight SSSP from vertex 1 (set _Source to move it).
template <class T = int32_t>
class SsspPS : public GraphPS<T> {
 public:
  int32_t _Source = 1;
  explicit SsspPS(const gx_config* cfg = nullptr) : GraphPS<T>(GX_APP_SSSP, cfg) {}

 protected:
  void configure(gx_run_params* p) override { p->source = _Source; }
};

// GraphMP/app/cc.cpp: min-label connected components.
template <class T = int32_t>
class CcPS : public GraphPS<T> {
 public:
  explicit CcPS(const gx_config* cfg = nullptr) : GraphPS<T>(GX_APP_CC, cfg) {}
};

}  // namespace gx

#endif  // GX_GRAPHPS_HPP_

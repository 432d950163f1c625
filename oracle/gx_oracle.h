/*
 * gx_oracle.h — CPU restatement of GraphMP's engine and vertex programs.
 *
 * TEST INFRASTRUCTURE ONLY.  The correctness reference for the CUDA path and the timed CPU
 * baseline ("port"); the product never links, loads or calls it.  Pinned
 * against outputs of the reference's own apps (oracle/_ref, built by
 * oracle/Makefile) stored under tests/golden/.
 *
 * The graph is passed as the reference's shards laid end to end: bounds[P+1]
 * destination ranges (Comp.h:36-37 start/end), off[V+1] global in-edge
 * offsets (the shards' indptr, rebased), col[] source ids (the shards'
 * indices).
 */
#ifndef GX_ORACLE_H_
#define GX_ORACLE_H_
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum {
  GXO_PAGERANK_REF = 0,   /* float, GraphMP/app/pagerank.cpp */
  GXO_PAGERANK_STD = 1,   /* double, dangling redistributed */
  GXO_SSSP = 2,           /* int32 unit weight (GPS_INF) or uint32 weighted */
  GXO_CC = 3,             /* int32 min label */
  GXO_INDEGREE = 4,       /* int32, GraphMP/app/cal.cpp */
  GXO_PAGERANK_REF64 = 5  /* the pagerank.cpp formula evaluated in double */
};

/* Runs GraphPS<T>::run (GraphMP/system/GraphPS.h:171-387) with the chosen
 * vertex program.  out_vals: float[V] (REF), double[V] (STD, REF64),
 * int32/uint32[V] (SSSP, CC, INDEGREE).  init_vals (nullable) replaces
 * init_vertex().  changed (nullable, max_iter entries) receives
 * _Changed_Vertex per step, ms (nullable) the per-step time.  Returns 0 on
 * success. */
int gxo_run(int app, int32_t V, int32_t P, const int32_t* bounds, const int64_t* off,
            const int32_t* col, const int32_t* outdeg, const uint32_t* w, int32_t max_iter,
            double damping, int32_t source, double tolerance, int threads,
            const void* init_vals, void* out_vals, int64_t* changed, double* ms,
            int32_t* iters_out);

/* Triangles of an undirected simple graph given as a symmetric CSR. */
uint64_t gxo_triangles(int32_t V, const int64_t* off, const int32_t* col, int threads);

/* Personalized PageRank, k sources, R <- restart*S + (1-restart)*A^T D^-1 R,
 * R0 = S, in double.  out: double[V*k] row-major (vertex, source). */
int gxo_ppr(int32_t V, const int64_t* off, const int32_t* col, const int32_t* outdeg, int32_t k,
            const int32_t* sources, int32_t iters, double restart, int threads, double* out);

/* Seeded R-MAT graph as a CSC (the library's generator restated): n edges
 * over 2^scale vertices, quadrant probabilities a, b, c; self-loops dropped
 * when drop_self, duplicates when dedup, both directions kept when
 * symmetric.  col holds n entries (2n when symmetric); *n_out = off[V]. */
int gxo_rmat_csc(int32_t scale, int64_t n, double a, double b, double c, uint64_t seed, int32_t drop_self,
                 int32_t dedup, int32_t symmetric, int threads, int64_t* off, int32_t* col, int64_t* n_out);
/* Edge-balanced destination-range shards (GraphMP/tools/format_spark.py:91-108). */
int gxo_partition_bounds(int32_t V, const int64_t* off, int32_t P, int32_t* bounds);
int gxo_out_degree(int32_t V, const int64_t* off, const int32_t* col, int threads, int32_t* outdeg);
/* Seeded SSSP weights in [1, 255] per CSC entry, a pure function of (seed, source, destination). */
int gxo_edge_weights(uint64_t seed, int32_t V, const int64_t* off, const int32_t* col, int threads, uint32_t* w);

#ifdef __cplusplus
}
#endif
#endif

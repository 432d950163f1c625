/* The three ZeroMQ calls GraphMP's single-process path touches
 * (GraphMP/system/Global.h:284,352).  Test infrastructure only. */
#ifndef GX_STUB_ZMQ_H
#define GX_STUB_ZMQ_H
static inline void* zmq_ctx_new() { static int ctx; return &ctx; }
static inline int zmq_ctx_destroy(void*) { return 0; }
static inline int zmq_close(void*) { return 0; }
#endif

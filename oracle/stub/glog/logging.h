/* Minimal stand-in for glog's LOG(INFO) as used by GraphMP
 * (GraphMP/system/GraphPS.h:375-382): lines go to stderr.  Test
 * infrastructure only. */
#ifndef GX_STUB_GLOG_H
#define GX_STUB_GLOG_H
#include <iostream>
namespace google { static inline void InitGoogleLogging(const char*) {} }
static bool FLAGS_logtostderr = true;
struct GxStubLogLine {
  ~GxStubLogLine() { std::cerr << std::endl; }
  template <class X> GxStubLogLine& operator<<(const X& x) { std::cerr << x; return *this; }
};
#define LOG(level) GxStubLogLine()
#endif

// Library-wide C-ABI helpers: error text, version, device query.
#include "common.cuh"
#include <atomic>
#include <cstring>

namespace pcg {
static thread_local char g_err[512] = {0};
static std::atomic<long long> g_launches{0};
constexpr long long kDefaultWaitNs = 4000000000LL;
static std::atomic<long long> g_wait_ns{kDefaultWaitNs};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long wait_limit_ns() { return (unsigned long long)g_wait_ns.load(); }

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
}  // namespace pcg

extern "C" const char* pcg_last_error(void) { return pcg::g_err; }

extern "C" int pcg_abi_version(void) { return 2; }

// Bound on any single device-side wait of the kernels launched from now on (ns); ns <= 0
// restores the 4 s default, larger bounds are capped at 600 s.  Returns the previous bound.
extern "C" long long pcg_set_wait_limit_ns(long long ns) {
  if (ns <= 0) ns = pcg::kDefaultWaitNs;
  if (ns > 600000000000LL) ns = 600000000000LL;
  return pcg::g_wait_ns.exchange(ns);
}

// Kernels launched by this library since it was loaded (all threads, all streams).
extern "C" long long pcg_launch_count(void) { return pcg::g_launches.load(); }

// Compute capability of the current device as major*10+minor, or a negative CUDA error.
extern "C" int pcg_device_cc(void) {
  int dev = 0, ma = 0, mi = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    pcg::set_error("pcg_device_cc: %s", cudaGetErrorString(e));
    return -(int)e;
  }
  cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, dev);
  return ma * 10 + mi;
}

// Blocks until the stream's work has finished; returns 0 or the CUDA error code.
extern "C" int pcg_stream_sync(void* stream) {
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) {
    pcg::set_error("pcg_stream_sync: %s", cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

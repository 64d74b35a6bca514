// Shared helpers of the pycc_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdarg>

namespace pcg {

// Host-side error text of the last failing entry point (per thread).
void set_error(const char* fmt, ...);
// Counts kernel launches issued by the library (read with pcg_launch_count).
void note_launch();

// Up to four sub-indices of one index group (M, N or K) of a contraction; each carries
// its extent and its element stride in the two tensors that hold it.
constexpr int kMaxSub = 4;
struct SubIdx {
  int n;
  long long ext[kMaxSub];
  long long s0[kMaxSub];
  long long s1[kMaxSub];
};

// Offsets of flat index r (row-major over ext[0..n), last fastest) in both tensors.
__host__ __device__ inline void sub_offsets(const SubIdx& d, long long r, long long& o0,
                                            long long& o1) {
  o0 = 0;
  o1 = 0;
  for (int q = d.n - 1; q >= 0; --q) {
    long long e = d.ext[q];
    long long x = r % e;
    r /= e;
    o0 += x * d.s0[q];
    o1 += x * d.s1[q];
  }
}

inline long long sub_total(const SubIdx& d) {
  long long t = 1;
  for (int q = 0; q < d.n; ++q) t *= d.ext[q];
  return t;
}

// Status word for device-side bounded waits (0 = fine).
enum DeviceStatus : int {
  kStatusOk = 0,
  kStatusTimeoutFull = 1,
  kStatusTimeoutEmpty = 2,
  kStatusTimeoutDone = 3,
};

}  // namespace pcg

#define PCG_CHECK_LAUNCH(name)                                                    \
  do {                                                                            \
    pcg::note_launch();                                                           \
    cudaError_t _e = cudaGetLastError();                                          \
    if (_e != cudaSuccess) {                                                      \
      pcg::set_error("%s: launch failed: %s", name, cudaGetErrorString(_e));      \
      return -2;                                                                  \
    }                                                                             \
  } while (0)

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
// Current bound (ns) on any single device-side wait of the tensor-core kernels
// (pcg_set_wait_limit_ns; 4 s by default).  Passed to the kernels as an argument.
unsigned long long wait_limit_ns();

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

// FP64 -> FP32, rounded to nearest even, in integer arithmetic.  GB300 issues FP64
// instructions (conversions from FP64 included) at a small fraction of its FP32 and integer
// rates, so streaming kernels that only need FP32 accuracy read FP64 data through this.
// Magnitudes below FP32's normal range flush to zero; above it, infinity; NaN stays NaN.
__device__ __forceinline__ float f64_to_f32(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
  const unsigned ex = (hi >> 20) & 0x7ffu;
  const int e = (int)ex - (1023 - 127);
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 of the 52 mantissa bits
  const unsigned rest = lo & 0x1fffffffu;                  // the 29 bits dropped
  unsigned f = ((unsigned)e << 23) + m;
  f += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
  if (e <= 0) f = 0u;
  if (e >= 255) f = (ex == 0x7ffu && ((hi & 0xfffffu) | lo)) ? 0x7fc00000u : 0x7f800000u;
  return __uint_as_float((hi & 0x80000000u) | f);
}

// FP32 -> FP64 (exact) in integer arithmetic, for the same reason.  FP32 subnormals, which
// an FP32 accumulator of this library's magnitudes does not produce, flush to zero.
__device__ __forceinline__ double f32_to_f64(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xffu;
  unsigned hi = u & 0x80000000u, lo = 0u;
  if (e == 0xffu) {
    hi |= 0x7ff00000u | ((u & 0x7fffffu) >> 3);
    lo = u << 29;
  } else if (e != 0u) {
    hi |= ((e + (1023u - 127u)) << 20) | ((u & 0x7fffffu) >> 3);
    lo = u << 29;
  }
  return __hiloint2double((int)hi, (int)lo);
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
  kStatusTimeoutProbe = 4,  // pcg_wait_probe: the self-test's wait expired, as it should
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

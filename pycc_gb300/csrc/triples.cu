// (T) energy from the connected triples of a batch of (i, j, k) triples, i >= j >= k.
//
// The connected triples W[a,b,c] of one triple arrive as three partial tensors, one per
// orientation of the twelve t3 terms (the terms of an orientation share their output
// layout, so each partial is written once by a single contraction).  Each is the output of
// a GEMM with rows (two virtual indices) and one column index, stored column-major:
//   orientation 1: rows (a,b), column c  ->  P1[c][a][b]
//   orientation 2: rows (a,c), column b  ->  P2[b][a][c]
//   orientation 3: rows (b,c), column a  ->  P3[a][b][c]
//   W[a,b,c] = P1[c][a][b] + P2[b][a][c] + P3[a][b][c]
// The Lee-Rendell energy of the reference (pycc/cctriples.py:177-240) is then evaluated
// for a >= b >= c with the same weights; one block per (triple, a), one FP64 partial per
// block (deterministic reduction by pcg_reduce_sum_f64).
#include "common.cuh"
#include <algorithm>

namespace pcg {
namespace {

constexpr int TE_THREADS = 256;

template <typename T>
struct TripArgs {
  const T* P1;
  const T* P2;
  const T* P3;
  long long pstride;  // elements between consecutive triples' partials
  const int* ijk;     // [ntrip][3]
  int ntrip;
  const double* eps;  // [nmo]
  const double* eoovv;  // <ij|ab> [o][o][v][v]
  const double* t1;   // [o][v]
  const double* t2;   // [o][o][v][v]
  const double* fov;  // [o][v] or null (canonical)
  long long no, nv;
  double* part;       // [ntrip][nv]
};

template <typename T>
__device__ __forceinline__ T wval(const TripArgs<T>& p, const T* P1, const T* P2, const T* P3,
                                  long long x, long long y, long long z) {
  const long long v = p.nv;
  return P1[(z * v + x) * v + y] + P2[(y * v + x) * v + z] + P3[(x * v + y) * v + z];
}

// disconnected triples (pycc/cctriples.py:133-140) at (x, y, z), in the arithmetic type T
// (FP32 for the tensor-core path: the FP64 pipe of GB300 is ~60x slower than FP32)
template <typename T>
__device__ __forceinline__ T dval(const TripArgs<T>& p, int i, int j, int k, long long x,
                                  long long y, long long z) {
  const long long o = p.no, v = p.nv;
  auto E = [&](int a, int b, long long c, long long d) {
    return (T)p.eoovv[((a * o + b) * v + c) * v + d];
  };
  auto A2 = [&](int a, int b, long long c, long long d) {
    return (T)p.t2[((a * o + b) * v + c) * v + d];
  };
  T d = E(i, j, x, y) * (T)p.t1[k * v + z] + E(i, k, x, z) * (T)p.t1[j * v + y] +
        E(j, k, y, z) * (T)p.t1[i * v + x];
  if (p.fov)
    d += A2(i, j, x, y) * (T)p.fov[k * v + z] + A2(i, k, x, z) * (T)p.fov[j * v + y] +
         A2(j, k, y, z) * (T)p.fov[i * v + x];
  return d;
}

template <typename T>
__global__ void __launch_bounds__(TE_THREADS) triples_energy_kernel(const TripArgs<T> p) {
  const int t = blockIdx.y;
  const long long a = blockIdx.x;
  const int i = p.ijk[3 * t], j = p.ijk[3 * t + 1], k = p.ijk[3 * t + 2];
  const T* P1 = p.P1 + t * p.pstride;
  const T* P2 = p.P2 + t * p.pstride;
  const T* P3 = p.P3 + t * p.pstride;
  const long long o = p.no;
  const double eo = p.eps[i] + p.eps[j] + p.eps[k];
  const double fac = 2.0 - ((i == j) + (i == k) + (j == k));
  const long long npair = (a + 1) * (a + 2) / 2;
  T acc_t = 0;  // per-thread partial (a few hundred terms); the block sum is FP64
  for (long long q = threadIdx.x; q < npair; q += TE_THREADS) {
    // q -> (b, c) with a >= b >= c
    long long b = (long long)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
    while (b * (b + 1) / 2 > q) --b;
    while ((b + 1) * (b + 2) / 2 <= q) ++b;
    const long long c = q - b * (b + 1) / 2;
    const long long idx[6][3] = {{a, b, c}, {a, c, b}, {b, a, c}, {b, c, a}, {c, a, b}, {c, b, a}};
    const T w = (T)(1 + (a == b) + (a == c) + (b == c));
    T W[6], V[6];
#pragma unroll
    for (int s = 0; s < 6; ++s) {
      W[s] = wval(p, P1, P2, P3, idx[s][0], idx[s][1], idx[s][2]);
      V[s] = (W[s] + dval(p, i, j, k, idx[s][0], idx[s][1], idx[s][2])) / w;
    }
    // perms: 0 abc, 1 acb, 2 bac, 3 bca, 4 cab, 5 cba
    T X = 0;
#pragma unroll
    for (int s = 0; s < 6; ++s) X += W[s] * V[s];
    const T Y = V[0] + V[3] + V[4];
    const T Z = V[1] + V[2] + V[5];
    const T Wc = W[0] + W[3] + W[4];
    const T Wa = W[1] + W[2] + W[5];
    const T S = (Y - (T)2 * Z) * Wc + (Z - (T)2 * Y) * Wa + (T)3 * X;
    const T D = (T)(eo - p.eps[o + a] - p.eps[o + b] - p.eps[o + c]);
    acc_t += S / D;
  }
  double acc = (double)acc_t;
  __shared__ double red[TE_THREADS / 32];
  for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < TE_THREADS / 32) ? red[threadIdx.x] : 0.0;
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    if (threadIdx.x == 0) p.part[(long long)t * p.nv + a] = fac * v;
  }
}

__global__ void reduce_sum_kernel(const double* x, long long n, double* out) {
  __shared__ double red[TE_THREADS / 32];
  double acc = 0.0;
  for (long long q = threadIdx.x; q < n; q += TE_THREADS) acc += x[q];
  for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < TE_THREADS / 32) ? red[threadIdx.x] : 0.0;
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    if (threadIdx.x == 0) *out += v;
  }
}

}  // namespace
}  // namespace pcg

using namespace pcg;

// (T) energy contributions of ntrip triples (see top of file).  fp32 selects FP32 partial
// tensors and FP32 element arithmetic (the tensor-core path); otherwise FP64 throughout.
// Writes part[t*nv + a] (FP64); the caller sums them.  pycc/cctriples.py:177-240.
extern "C" int pcg_triples_energy(int fp32, const void* P1, const void* P2, const void* P3,
                                  long long pstride, const int* ijk, int ntrip,
                                  const double* eps, const double* eoovv, const double* t1,
                                  const double* t2, const double* fov, long long no,
                                  long long nv, double* part, void* stream) {
  if (ntrip < 1 || ntrip > 65535 || nv < 1 || nv > 0x7fffffff || !P1 || !P2 || !P3 || !ijk ||
      !eps || !eoovv || !t1 || !t2 || !part) {
    set_error("pcg_triples_energy: bad arguments (ntrip=%d)", ntrip);
    return -1;
  }
  dim3 grid((unsigned)nv, (unsigned)ntrip);
  cudaStream_t st = (cudaStream_t)stream;
  if (fp32) {
    TripArgs<float> a{(const float*)P1, (const float*)P2, (const float*)P3, pstride, ijk, ntrip,
                      eps, eoovv, t1, t2, fov, no, nv, part};
    triples_energy_kernel<float><<<grid, TE_THREADS, 0, st>>>(a);
  } else {
    TripArgs<double> a{(const double*)P1, (const double*)P2, (const double*)P3, pstride, ijk,
                       ntrip, eps, eoovv, t1, t2, fov, no, nv, part};
    triples_energy_kernel<double><<<grid, TE_THREADS, 0, st>>>(a);
  }
  PCG_CHECK_LAUNCH("pcg_triples_energy");
  return 0;
}

// *out += sum(x[0:n]) in FP64, one block (deterministic order).
extern "C" int pcg_reduce_sum_f64(const double* x, long long n, double* out, void* stream) {
  if (!x || !out || n < 0) {
    set_error("pcg_reduce_sum_f64: bad arguments");
    return -1;
  }
  reduce_sum_kernel<<<1, TE_THREADS, 0, (cudaStream_t)stream>>>(x, n, out);
  PCG_CHECK_LAUNCH("pcg_reduce_sum_f64");
  return 0;
}

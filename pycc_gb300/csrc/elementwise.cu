// HBM-bound FP64 kernels of the CCSD iteration: tau builds, operand combinations, the
// r2 symmetrisation, the Jacobi amplitude update with its norm, the energy expression and
// the DIIS dot products / linear combinations.  All are grid-stride loops over the o^2 v^2
// amplitude space; the reductions are two-stage (per-block partials in a caller-provided
// work buffer, then one block) so every sum is deterministic run to run.
#include "common.cuh"
#include <algorithm>

namespace pcg {
namespace {

constexpr int EW_THREADS = 256;
constexpr int RED_BLOCKS = 1024;  // partials per reduced scalar

int ew_blocks(long long n) {
  long long b = (n + EW_THREADS - 1) / EW_THREADS;
  return (int)std::max<long long>(1, std::min<long long>(b, 152LL * 16));
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[EW_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  v = (threadIdx.x < EW_THREADS / 32) ? red[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;  // valid in thread 0
}

// out[j] = sum_b part[j * nb + b]
__global__ void finish_sum_kernel(const double* part, int nb, int k, double* out) {
  for (int j = 0; j < k; ++j) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += EW_THREADS) v += part[(long long)j * nb + b];
    v = block_sum(v);
    if (threadIdx.x == 0) out[j] = v;
    __syncthreads();
  }
}

__global__ void tau_kernel(const double* __restrict__ t1, const double* __restrict__ t2,
                           long long no, long long nv, double f1, double f2,
                           double* __restrict__ out) {
  long long total = no * no * nv * nv;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    unsigned r = (unsigned)idx;  // o^2 v^2 < 2^31 (host check)
    const long long b = r % (unsigned)nv;
    r /= (unsigned)nv;
    const long long a = r % (unsigned)nv;
    r /= (unsigned)nv;
    const long long j = r % (unsigned)no, i = r / (unsigned)no;
    double x = f1 * t2[idx];
    if (f2 != 0.0) x += f2 * t1[i * nv + a] * t1[j * nv + b];
    out[idx] = x;
  }
}

struct Strides4 {
  long long e[4], x[4], y[4], o[4];
};

// I: the index type of the decomposition (unsigned when the tensor has < 2^31 elements;
// 64-bit division is several times longer)
template <typename I>
__global__ void combine4_kernel(Strides4 s, double a, const double* __restrict__ X, double b,
                                const double* __restrict__ Y, double* __restrict__ out) {
  long long total = s.e[0] * s.e[1] * s.e[2] * s.e[3];
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    I r = (I)idx;
    long long ox = 0, oy = 0, oo = 0;
#pragma unroll
    for (int q = 3; q >= 0; --q) {
      const long long c = r % (I)s.e[q];
      r /= (I)s.e[q];
      ox += c * s.x[q];
      oy += c * s.y[q];
      oo += c * s.o[q];
    }
    double v = a * X[ox];
    if (Y) v += b * Y[oy];
    out[oo] = v;
  }
}

__global__ void symmetrize_kernel(const double* __restrict__ h, long long no, long long nv,
                                  double* __restrict__ out) {
  long long total = no * no * nv * nv;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    unsigned r = (unsigned)idx;  // o^2 v^2 < 2^31 (host check)
    const long long b = r % (unsigned)nv;
    r /= (unsigned)nv;
    const long long a = r % (unsigned)nv;
    r /= (unsigned)nv;
    const long long j = r % (unsigned)no, i = r / (unsigned)no;
    out[idx] = h[idx] + h[((j * no + i) * nv + b) * nv + a];
  }
}

__global__ void update_kernel(double* __restrict__ t1, double* __restrict__ t2,
                              const double* __restrict__ r1, const double* __restrict__ r2,
                              const double* __restrict__ eps, long long no, long long nv,
                              double* __restrict__ part) {
  long long n1 = no * nv, total = n1 + no * no * nv * nv;
  double acc = 0.0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    if (idx < n1) {
      const unsigned x = (unsigned)idx;  // o^2 v^2 < 2^31 (host check)
      const long long a = x % (unsigned)nv, i = x / (unsigned)nv;
      double u = r1[idx] / (eps[i] - eps[no + a]);
      t1[idx] += u;
      acc += u * u;
    } else {
      const long long q = idx - n1;
      unsigned r = (unsigned)q;
      const long long b = r % (unsigned)nv;
      r /= (unsigned)nv;
      const long long a = r % (unsigned)nv;
      r /= (unsigned)nv;
      const long long j = r % (unsigned)no, i = r / (unsigned)no;
      double u = r2[q] / (eps[i] + eps[j] - eps[no + a] - eps[no + b]);
      t2[q] += u;
      acc += u * u;
    }
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

__global__ void inv_denom_kernel(const double* __restrict__ eps, long long no, long long nv,
                                 double* __restrict__ inv1, double* __restrict__ inv2) {
  const long long n1 = no * nv, total = n1 + no * no * nv * nv;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    if (idx < n1) {
      const long long a = idx % nv, i = idx / nv;
      inv1[idx] = 1.0 / (eps[i] - eps[no + a]);
    } else {
      const long long q = idx - n1;
      long long b = q % nv, r = q / nv;
      const long long a = r % nv;
      r /= nv;
      const long long j = r % no, i = r / no;
      inv2[q] = 1.0 / (eps[i] + eps[j] - eps[no + a] - eps[no + b]);
    }
  }
}

// t += r * (1/D) with precomputed inverse denominators: three FP64 operations per element
// (the divide of update_kernel costs an order of magnitude more on the FP64 pipe).
__global__ void update_inv_kernel(double* __restrict__ t, const double* __restrict__ r,
                                  const double* __restrict__ inv, long long n,
                                  double* __restrict__ part) {
  double acc = 0.0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const double u = r[idx] * inv[idx];
    t[idx] += u;
    acc += u * u;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// One warp per row (i, j, a) of the doubles: the lanes walk b, so t2 and L are read in
// coalesced runs (L's b stride is 1 for the resident block) and the row's index
// decomposition and t_ia are paid once per row; two FP64 FMAs per element, the singles part
// by the first rows' warps.
__global__ void energy_kernel(const double* __restrict__ fov, long long fs0, long long fs1,
                              const double* __restrict__ L, Strides4 ls,
                              const double* __restrict__ t1, const double* __restrict__ t2,
                              long long no, long long nv, double* __restrict__ part) {
  const long long n1 = no * nv;
  const int lane = threadIdx.x & 31;
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  double acc = 0.0;
  for (long long x = warp0 * 32 + lane; x < n1; x += nwarps * 32) {
    const long long a = x % nv, i = x / nv;
    acc += 2.0 * fov[i * fs0 + a * fs1] * t1[x];
  }
  const long long rows = no * no * nv;  // (i, j, a); o^2 v^2 < 2^31 (host check)
  for (long long r = warp0; r < rows; r += nwarps) {
    unsigned q = (unsigned)r;
    const long long a = q % (unsigned)nv;
    q /= (unsigned)nv;
    const long long j = q % (unsigned)no, i = q / (unsigned)no;
    const double tia = t1[i * nv + a];
    const double* t2r = t2 + r * nv;
    const double* Lr = L + i * ls.o[0] + j * ls.o[1] + a * ls.o[2];
    const double* t1j = t1 + j * nv;
    const long long sb = ls.o[3];
    // four elements per lane in flight: the loads of a step are issued before its FMAs
    long long b = lane;
    double acc1 = 0.0, acc2 = 0.0, acc3 = 0.0;
    for (; b + 96 < nv; b += 128) {
      const double x0 = t2r[b], x1 = t2r[b + 32], x2 = t2r[b + 64], x3 = t2r[b + 96];
      const double l0 = Lr[b * sb], l1 = Lr[(b + 32) * sb], l2 = Lr[(b + 64) * sb],
                   l3 = Lr[(b + 96) * sb];
      acc = fma(fma(tia, t1j[b], x0), l0, acc);
      acc1 = fma(fma(tia, t1j[b + 32], x1), l1, acc1);
      acc2 = fma(fma(tia, t1j[b + 64], x2), l2, acc2);
      acc3 = fma(fma(tia, t1j[b + 96], x3), l3, acc3);
    }
    for (; b < nv; b += 32) acc = fma(fma(tia, t1j[b], t2r[b]), Lr[b * sb], acc);
    acc += (acc1 + acc2) + acc3;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

constexpr int kMaxVec = 16;
struct VecList {
  const double* p[kMaxVec];
  double c[kMaxVec];
};

__global__ void dots_kernel(const double* __restrict__ x, VecList ys, int k, long long n,
                            double* __restrict__ part) {
  double acc[kMaxVec];
#pragma unroll
  for (int j = 0; j < kMaxVec; ++j) acc[j] = 0.0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    double xv = x[idx];
#pragma unroll
    for (int j = 0; j < kMaxVec; ++j)
      if (j < k) acc[j] += xv * ys.p[j][idx];
  }
#pragma unroll
  for (int j = 0; j < kMaxVec; ++j) {  // constant indices keep acc in registers
    if (j >= k) break;
    double v = block_sum(acc[j]);
    if (threadIdx.x == 0) part[(long long)j * gridDim.x + blockIdx.x] = v;
    __syncthreads();
  }
}

// e = x - old (written) and part[j] = <e, ys[j]> for j < k-1, part[k-1] = <e, e>.
__global__ void diis_error_kernel(const double* __restrict__ x, const double* __restrict__ old,
                                  double* __restrict__ e, VecList ys, int k, long long n,
                                  double* __restrict__ part) {
  double acc[kMaxVec];
#pragma unroll
  for (int j = 0; j < kMaxVec; ++j) acc[j] = 0.0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const double ev = x[idx] - old[idx];
    e[idx] = ev;
#pragma unroll
    for (int j = 0; j < kMaxVec - 1; ++j)
      if (j < k - 1) acc[j] += ev * ys.p[j][idx];
    acc[kMaxVec - 1] += ev * ev;
  }
  // constant indices (unrolled) keep acc in registers; j < k is uniform over the block
#pragma unroll
  for (int j = 0; j < kMaxVec; ++j) {
    if (j >= k) break;
    double v = block_sum(j == k - 1 ? acc[kMaxVec - 1] : acc[j]);
    if (threadIdx.x == 0) part[(long long)j * gridDim.x + blockIdx.x] = v;
    __syncthreads();
  }
}

struct VecListF {
  const float* p[kMaxVec];
};

// Mixed-precision DIIS error pass: e = FP32(x - old) (the difference taken in FP64 and
// rounded once, in integer arithmetic) and its overlaps with the k-1 stored FP32 error
// vectors and itself.  Four consecutive elements per step: their FP32 products are summed
// in FP32 and each step's sum is accumulated in FP64, so a vector of n elements costs
// n + k n / 4 FP64 additions instead of the k n of the FP64 pass.
__global__ void diis_error_f32_kernel(const double* __restrict__ x,
                                      const double* __restrict__ old, float* __restrict__ e,
                                      VecListF ys, int k, long long n,
                                      double* __restrict__ part) {
  double acc[kMaxVec];
#pragma unroll
  for (int j = 0; j < kMaxVec; ++j) acc[j] = 0.0;
  const long long n4 = n >> 2;
  const double2* x2 = reinterpret_cast<const double2*>(x);
  const double2* o2 = reinterpret_cast<const double2*>(old);
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4;
       q += (long long)gridDim.x * blockDim.x) {
    const double2 xa = x2[2 * q], xb = x2[2 * q + 1], oa = o2[2 * q], ob = o2[2 * q + 1];
    const float4 ev = make_float4(f64_to_f32(xa.x - oa.x), f64_to_f32(xa.y - oa.y),
                                  f64_to_f32(xb.x - ob.x), f64_to_f32(xb.y - ob.y));
    reinterpret_cast<float4*>(e)[q] = ev;
#pragma unroll
    for (int j = 0; j < kMaxVec - 1; ++j)
      if (j < k - 1) {
        const float4 y = reinterpret_cast<const float4*>(ys.p[j])[q];
        acc[j] += f32_to_f64(ev.x * y.x + ev.y * y.y + ev.z * y.z + ev.w * y.w);
      }
    acc[kMaxVec - 1] += f32_to_f64(ev.x * ev.x + ev.y * ev.y + ev.z * ev.z + ev.w * ev.w);
  }
  if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {  // the last n mod 4 elements
    const long long i = (n4 << 2) + threadIdx.x;
    const float v = f64_to_f32(x[i] - old[i]);
    e[i] = v;
#pragma unroll
    for (int j = 0; j < kMaxVec - 1; ++j)
      if (j < k - 1) acc[j] += f32_to_f64(v * ys.p[j][i]);
    acc[kMaxVec - 1] += f32_to_f64(v * v);
  }
  // constant indices (unrolled) keep acc in registers; j < k is uniform over the block
#pragma unroll
  for (int j = 0; j < kMaxVec; ++j) {
    if (j >= k) break;
    double v = block_sum(j == k - 1 ? acc[kMaxVec - 1] : acc[j]);
    if (threadIdx.x == 0) part[(long long)j * gridDim.x + blockIdx.x] = v;
    __syncthreads();
  }
}

__global__ void lincomb_kernel(VecList xs, int k, long long n, double* __restrict__ out) {
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    double v = 0.0;
#pragma unroll
    for (int j = 0; j < kMaxVec; ++j)
      if (j < k) v += xs.c[j] * xs.p[j][idx];
    out[idx] = v;
  }
}

// x = hi + lo with hi the FP32 rounding of x and lo the FP32 rounding of the remainder
// x - hi, both in integer arithmetic: hi keeps the top 24 of the 53 significand bits, lo the
// next 24 (remainders of FP64 values below 2^-74 in magnitude flush to zero).
__device__ __forceinline__ void split_f64(double x, float& hi, float& lo) {
  hi = f64_to_f32(x);
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned uh = (unsigned)(u >> 32), ul = (unsigned)u;
  const int ex = (int)((uh >> 20) & 0x7ffu);
  const unsigned m = ((uh & 0xfffffu) << 3) | (ul >> 29);
  const int rest = (int)(ul & 0x1fffffffu);  // the 29 bits hi dropped
  const bool up = rest > 0x10000000 || (rest == 0x10000000 && (m & 1u));
  const int r = up ? rest - 0x20000000 : rest;  // x - hi in units of 2^(e - 52)
  const int e2 = ex - 1023 - 52 + 127;          // FP32 exponent field of 2^(e - 52)
  float lo_ = 0.f;
  if (ex != 0 && ex != 0x7ff && e2 > 0 && e2 < 255)
    lo_ = __int2float_rn(r) * __uint_as_float((unsigned)e2 << 23);
  lo = (uh & 0x80000000u) ? -lo_ : lo_;
}

// out = sum_j c_j x_j in double-float arithmetic: each term's FP32 pieces and the
// coefficient's (c_hi, c_lo) give the product with its exact rounding error (FMA), the
// running sum is kept as an unevaluated FP32 pair (TwoSum), about 48 significant bits; one
// FP64 addition per element assembles the result.
__device__ __forceinline__ void df_term(double x, float ch, float cl, float& S, float& E) {
  float h, l;
  split_f64(x, h, l);
  const float p = ch * h;
  float e = fmaf(ch, h, -p);
  e = fmaf(ch, l, e);
  e = fmaf(cl, h, e);
  const float t = S + p;
  const float bp = t - S;
  E += ((S - (t - bp)) + (p - bp)) + e;
  S = t;
}

// Two elements per step through 16-byte loads (the inputs and the output are 16-byte
// aligned, checked by the host).  All k loads of a step are issued before its arithmetic
// (KMAX bounds k at compile time, so the loaded values stay in registers); the
// coefficients' FP32 pieces live in shared memory.  The last element of an odd n is done
// by one thread.
template <int KMAX>
__global__ void lincomb_df_kernel(VecList xs, int k, long long n, double* __restrict__ out) {
  __shared__ float sch[kMaxVec], scl[kMaxVec];
  if (threadIdx.x < kMaxVec) {
    const float h = (float)xs.c[threadIdx.x];
    sch[threadIdx.x] = h;
    scl[threadIdx.x] = (float)(xs.c[threadIdx.x] - (double)h);
  }
  __syncthreads();
  const long long n2 = n >> 1;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n2;
       q += (long long)gridDim.x * blockDim.x) {
    double2 x[KMAX];
#pragma unroll
    for (int j = 0; j < KMAX; ++j)
      if (j < k) x[j] = reinterpret_cast<const double2*>(xs.p[j])[q];
    float S0 = 0.f, E0 = 0.f, S1 = 0.f, E1 = 0.f;
#pragma unroll
    for (int j = 0; j < KMAX; ++j)
      if (j < k) {
        df_term(x[j].x, sch[j], scl[j], S0, E0);
        df_term(x[j].y, sch[j], scl[j], S1, E1);
      }
    reinterpret_cast<double2*>(out)[q] =
        make_double2(f32_to_f64(S0) + f32_to_f64(E0), f32_to_f64(S1) + f32_to_f64(E1));
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    float S = 0.f, E = 0.f;
    for (int j = 0; j < k; ++j) df_term(xs.p[j][n - 1], sch[j], scl[j], S, E);
    out[n - 1] = f32_to_f64(S) + f32_to_f64(E);
  }
}

bool check_work(long long work_len, long long need, const char* who) {
  if (work_len < need) {
    set_error("%s: work buffer holds %lld doubles, needs %lld", who, work_len, need);
    return false;
  }
  return true;
}

}  // namespace
}  // namespace pcg

using namespace pcg;

extern "C" int pcg_tau_f64(const double* t1, const double* t2, long long no, long long nv,
                           double f1, double f2, double* out, void* stream) {
  if (!t1 || !t2 || !out || no <= 0 || nv <= 0 || no * no * nv * nv > 0x7fffffffLL) {
    set_error("pcg_tau_f64: bad arguments (o^2 v^2 must be below 2^31)");
    return -1;
  }
  long long n = no * no * nv * nv;
  tau_kernel<<<ew_blocks(n), EW_THREADS, 0, (cudaStream_t)stream>>>(t1, t2, no, nv, f1, f2, out);
  PCG_CHECK_LAUNCH("pcg_tau_f64");
  return 0;
}

extern "C" int pcg_combine4_f64(const long long* ext, double a, const double* X,
                                const long long* xs, double b, const double* Y,
                                const long long* ys, double* out, const long long* os,
                                void* stream) {
  if (!X || !out || !ext || !xs || !os || (Y && !ys)) {
    set_error("pcg_combine4_f64: null pointer");
    return -1;
  }
  Strides4 s;
  long long n = 1;
  for (int q = 0; q < 4; ++q) {
    s.e[q] = ext[q];
    s.x[q] = xs[q];
    s.y[q] = Y ? ys[q] : 0;
    s.o[q] = os[q];
    if (ext[q] <= 0) {
      set_error("pcg_combine4_f64: extent %d is %lld", q, ext[q]);
      return -1;
    }
    n *= ext[q];
  }
  if (n <= 0x7fffffffLL)
    combine4_kernel<unsigned><<<ew_blocks(n), EW_THREADS, 0, (cudaStream_t)stream>>>(s, a, X, b,
                                                                                    Y, out);
  else
    combine4_kernel<unsigned long long>
        <<<ew_blocks(n), EW_THREADS, 0, (cudaStream_t)stream>>>(s, a, X, b, Y, out);
  PCG_CHECK_LAUNCH("pcg_combine4_f64");
  return 0;
}

extern "C" int pcg_symmetrize_f64(const double* h, long long no, long long nv, double* out,
                                  void* stream) {
  if (!h || !out || h == out) {
    set_error("pcg_symmetrize_f64: bad pointers (input and output must differ)");
    return -1;
  }
  if (no <= 0 || nv <= 0 || no * no * nv * nv > 0x7fffffffLL) {
    set_error("pcg_symmetrize_f64: o^2 v^2 must be in [1, 2^31)");
    return -1;
  }
  long long n = no * no * nv * nv;
  symmetrize_kernel<<<ew_blocks(n), EW_THREADS, 0, (cudaStream_t)stream>>>(h, no, nv, out);
  PCG_CHECK_LAUNCH("pcg_symmetrize_f64");
  return 0;
}

extern "C" int pcg_update_amps_f64(double* t1, double* t2, const double* r1, const double* r2,
                                   const double* eps, long long no, long long nv, double* work,
                                   long long work_len, double* rms2, void* stream) {
  if (!t1 || !t2 || !r1 || !r2 || !eps || !work || !rms2) {
    set_error("pcg_update_amps_f64: null pointer");
    return -1;
  }
  if (!check_work(work_len, RED_BLOCKS, "pcg_update_amps_f64")) return -1;
  if (no <= 0 || nv <= 0 || no * no * nv * nv > 0x7fffffffLL) {
    set_error("pcg_update_amps_f64: o^2 v^2 must be in [1, 2^31)");
    return -1;
  }
  cudaStream_t st = (cudaStream_t)stream;
  long long n = no * nv + no * no * nv * nv;
  int nb = std::min(ew_blocks(n), RED_BLOCKS);
  update_kernel<<<nb, EW_THREADS, 0, st>>>(t1, t2, r1, r2, eps, no, nv, work);
  PCG_CHECK_LAUNCH("pcg_update_amps_f64/update");
  finish_sum_kernel<<<1, EW_THREADS, 0, st>>>(work, nb, 1, rms2);
  PCG_CHECK_LAUNCH("pcg_update_amps_f64");
  return 0;
}

extern "C" int pcg_energy_f64(const double* fov, const long long* fs, const double* L,
                              const long long* ls, const double* t1, const double* t2,
                              long long no, long long nv, double* work, long long work_len,
                              double* out, void* stream) {
  if (!fov || !fs || !L || !ls || !t1 || !t2 || !work || !out) {
    set_error("pcg_energy_f64: null pointer");
    return -1;
  }
  if (!check_work(work_len, RED_BLOCKS, "pcg_energy_f64")) return -1;
  cudaStream_t st = (cudaStream_t)stream;
  Strides4 s{};
  for (int q = 0; q < 4; ++q) s.o[q] = ls[q];
  if (no < 1 || nv < 1 || no * no * nv * nv > 0x7fffffffLL) {
    set_error("pcg_energy_f64: o^2 v^2 must be in [1, 2^31)");
    return -1;
  }
  long long n = no * nv + no * no * nv * nv;
  int nb = std::min(ew_blocks(n), RED_BLOCKS);
  energy_kernel<<<nb, EW_THREADS, 0, st>>>(fov, fs[0], fs[1], L, s, t1, t2, no, nv, work);
  PCG_CHECK_LAUNCH("pcg_energy_f64/terms");
  finish_sum_kernel<<<1, EW_THREADS, 0, st>>>(work, nb, 1, out);
  PCG_CHECK_LAUNCH("pcg_energy_f64");
  return 0;
}

extern "C" int pcg_dots_f64(const double* x, const double* const* ys, int k, long long n,
                            double* work, long long work_len, double* out, void* stream) {
  if (k < 1 || k > kMaxVec) {
    set_error("pcg_dots_f64: k=%d outside [1, %d]", k, kMaxVec);
    return -1;
  }
  if (!x || !ys || !work || !out || n < 0) {
    set_error("pcg_dots_f64: null pointer or negative length");
    return -1;
  }
  for (int j = 0; j < k; ++j)
    if (!ys[j]) {
      set_error("pcg_dots_f64: vector %d is null", j);
      return -1;
    }
  if (!check_work(work_len, (long long)k * RED_BLOCKS, "pcg_dots_f64")) return -1;
  cudaStream_t st = (cudaStream_t)stream;
  VecList v{};
  for (int j = 0; j < k; ++j) v.p[j] = ys[j];
  int nb = std::min(ew_blocks(n), RED_BLOCKS);
  dots_kernel<<<nb, EW_THREADS, 0, st>>>(x, v, k, n, work);
  PCG_CHECK_LAUNCH("pcg_dots_f64/partials");
  finish_sum_kernel<<<1, EW_THREADS, 0, st>>>(work, nb, k, out);
  PCG_CHECK_LAUNCH("pcg_dots_f64");
  return 0;
}

extern "C" int pcg_lincomb_f64(const double* const* xs, const double* c, int k, long long n,
                               double* out, void* stream) {
  if (k < 1 || k > kMaxVec) {
    set_error("pcg_lincomb_f64: k=%d outside [1, %d]", k, kMaxVec);
    return -1;
  }
  if (!xs || !c || !out || n < 0) {
    set_error("pcg_lincomb_f64: null pointer or negative length");
    return -1;
  }
  for (int j = 0; j < k; ++j)
    if (!xs[j]) {
      set_error("pcg_lincomb_f64: input %d is null", j);
      return -1;
    }
  VecList v{};
  for (int j = 0; j < k; ++j) {
    v.p[j] = xs[j];
    v.c[j] = c[j];
    if (xs[j] == out) {
      set_error("pcg_lincomb_f64: output aliases input %d", j);
      return -1;
    }
  }
  lincomb_kernel<<<ew_blocks(n), EW_THREADS, 0, (cudaStream_t)stream>>>(v, k, n, out);
  PCG_CHECK_LAUNCH("pcg_lincomb_f64");
  return 0;
}

// pcg_lincomb_f64 in double-float arithmetic (see lincomb_df_kernel), for the
// mixed-precision solver: one FP64 instruction per element instead of k.
extern "C" int pcg_lincomb_f64_df(const double* const* xs, const double* c, int k, long long n,
                                  double* out, void* stream) {
  if (k < 1 || k > kMaxVec || !xs || !c || !out || n < 0) {
    set_error("pcg_lincomb_f64_df: bad arguments (k=%d)", k);
    return -1;
  }
  VecList v{};
  bool aligned = ((uintptr_t)out & 15u) == 0;
  for (int j = 0; j < k; ++j) {
    if (!xs[j] || xs[j] == out) {
      set_error("pcg_lincomb_f64_df: input %d is null or aliases the output", j);
      return -1;
    }
    aligned = aligned && ((uintptr_t)xs[j] & 15u) == 0;
    v.p[j] = xs[j];
    v.c[j] = c[j];
  }
  if (!aligned) {
    set_error("pcg_lincomb_f64_df: vectors must be 16-byte aligned");
    return -1;
  }
  const int nb = ew_blocks(std::max(n / 2, 1LL));
  cudaStream_t st = (cudaStream_t)stream;
  if (k <= 4)
    lincomb_df_kernel<4><<<nb, EW_THREADS, 0, st>>>(v, k, n, out);
  else if (k <= 8)
    lincomb_df_kernel<8><<<nb, EW_THREADS, 0, st>>>(v, k, n, out);
  else
    lincomb_df_kernel<kMaxVec><<<nb, EW_THREADS, 0, st>>>(v, k, n, out);
  PCG_CHECK_LAUNCH("pcg_lincomb_f64_df");
  return 0;
}

extern "C" int pcg_diis_error_f64(const double* x, const double* old, double* e,
                                  const double* const* ys, int k, long long n, double* work,
                                  long long work_len, double* out, void* stream) {
  if (k < 1 || k > kMaxVec) {
    set_error("pcg_diis_error_f64: k=%d outside [1, %d]", k, kMaxVec);
    return -1;
  }
  if (!x || !old || !e || e == x || e == old || !work || !out || n < 0 || (k > 1 && !ys)) {
    set_error("pcg_diis_error_f64: bad pointers");
    return -1;
  }
  for (int j = 0; j + 1 < k; ++j)
    if (!ys[j]) {
      set_error("pcg_diis_error_f64: stored error vector %d is null", j);
      return -1;
    }
  if (!check_work(work_len, (long long)k * RED_BLOCKS, "pcg_diis_error_f64")) return -1;
  cudaStream_t st = (cudaStream_t)stream;
  VecList v{};
  for (int j = 0; j + 1 < k; ++j) v.p[j] = ys[j];
  int nb = std::min(ew_blocks(n), RED_BLOCKS);
  diis_error_kernel<<<nb, EW_THREADS, 0, st>>>(x, old, e, v, k, n, work);
  PCG_CHECK_LAUNCH("pcg_diis_error_f64/partials");
  finish_sum_kernel<<<1, EW_THREADS, 0, st>>>(work, nb, k, out);
  PCG_CHECK_LAUNCH("pcg_diis_error_f64");
  return 0;
}

// FP32 error storage for the mixed-precision solver (see diis_error_f32_kernel); the
// pointers are 16-byte aligned (vector loads of four elements).
extern "C" int pcg_diis_error_f32(const double* x, const double* old, float* e,
                                  const float* const* ys, int k, long long n, double* work,
                                  long long work_len, double* out, void* stream) {
  if (k < 1 || k > kMaxVec) {
    set_error("pcg_diis_error_f32: k=%d outside [1, %d]", k, kMaxVec);
    return -1;
  }
  if (!x || !old || !e || !out || !work || n < 0 || (k > 1 && !ys)) {
    set_error("pcg_diis_error_f32: bad arguments");
    return -1;
  }
  auto al16 = [](const void* q) { return ((uintptr_t)q & 15u) == 0; };
  bool ok = al16(x) && al16(old) && al16(e);
  VecListF v{};
  for (int j = 0; j + 1 < k; ++j) {
    if (!ys || !ys[j]) {
      set_error("pcg_diis_error_f32: null stored error vector %d", j);
      return -1;
    }
    v.p[j] = ys[j];
    ok = ok && al16(ys[j]);
  }
  if (!ok) {
    set_error("pcg_diis_error_f32: vectors must be 16-byte aligned");
    return -1;
  }
  if (!check_work(work_len, (long long)k * RED_BLOCKS, "pcg_diis_error_f32")) return -1;
  cudaStream_t st = (cudaStream_t)stream;
  int nb = std::min(ew_blocks(std::max(n / 4, 1LL)), RED_BLOCKS);
  diis_error_f32_kernel<<<nb, EW_THREADS, 0, st>>>(x, old, e, v, k, n, work);
  PCG_CHECK_LAUNCH("pcg_diis_error_f32/partials");
  finish_sum_kernel<<<1, EW_THREADS, 0, st>>>(work, nb, k, out);
  PCG_CHECK_LAUNCH("pcg_diis_error_f32");
  return 0;
}

// ---------------------------------------------------------------------------------------
// Allocation-free variant of pcg_dots_f64.
//
// Some host programs cannot let a library allocate device memory: quantum-chemistry codes
// that carve the whole GPU into their own arena up front (a library cudaMalloc then fails
// or fragments it), and loops that must not pay cudaMalloc/cudaFree, which can synchronise
// the device.  pcg_dots_f64 needs k*1024 doubles of scratch for its per-block partial
// sums; this variant keeps that scratch in a fixed array of this library instead, so the
// caller passes only the inputs and the output.
//
// * Limit: at most kNoAllocMaxVec (8) vectors per call, i.e. 8*1024 doubles (64 KB) of
//   scratch, which every GPU that loads the library holds until the process exits.
// * The array lives in device memory; host code only sees a stand-in symbol, so its device
//   address is looked up once per device (cudaGetSymbolAddress) on the first call made
//   with that device current.  Make that first call before any stream capture.  The
//   address is cached for the life of the process: do not keep using the library across a
//   cudaDeviceReset of that device (the reset unloads the module, and the array may come
//   back at another address).
// * Every call shares the array.  Each call writes every partial it later reads, so no
//   clearing is needed, but calls that overlap on the GPU (different streams, or several
//   host threads) race on it: serialise them.
// ---------------------------------------------------------------------------------------
#include <mutex>

namespace pcg {
namespace {
constexpr int kNoAllocMaxVec = 8;
static __device__ __align__(256) double g_dots_scratch[kNoAllocMaxVec * RED_BLOCKS];

constexpr int kMaxDevices = 64;
double* g_dots_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_dots_scratch_mu;

// Device address of g_dots_scratch on the current device (looked up once per device).
double* dots_scratch_address() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("pcg_dots_f64_noalloc: cudaGetDevice failed: %s", cudaGetErrorString(e));
    return nullptr;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("pcg_dots_f64_noalloc: device ordinal %d out of range", dev);
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_dots_scratch_mu);
  if (!g_dots_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_dots_scratch);
    if (e != cudaSuccess || !p) {
      set_error("pcg_dots_f64_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return nullptr;
    }
    g_dots_scratch_ptr[dev] = static_cast<double*>(p);
  }
  return g_dots_scratch_ptr[dev];
}
}  // namespace
}  // namespace pcg

// out[j] = <x, ys[j]> for 1 <= k <= 8, with no device allocation (see above).
extern "C" int pcg_dots_f64_noalloc(const double* x, const double* const* ys, int k, long long n,
                                    double* out, void* stream) {
  if (k < 1 || k > kNoAllocMaxVec) {
    set_error("pcg_dots_f64_noalloc: k=%d outside [1, %d] (the fixed scratch holds %d vectors; "
              "use pcg_dots_f64 with a caller-provided work buffer for more)",
              k, kNoAllocMaxVec, kNoAllocMaxVec);
    return -1;
  }
  if (!x || !ys || !out || n < 0) {
    set_error("pcg_dots_f64_noalloc: bad arguments");
    return -1;
  }
  for (int j = 0; j < k; ++j)
    if (!ys[j]) {
      set_error("pcg_dots_f64_noalloc: ys[%d] is null", j);
      return -1;
    }
  double* scratch = dots_scratch_address();
  if (!scratch) return -3;
  cudaStream_t st = (cudaStream_t)stream;
  VecList v{};
  for (int j = 0; j < k; ++j) v.p[j] = ys[j];
  const int nb = std::min(ew_blocks(n), RED_BLOCKS);
  dots_kernel<<<nb, EW_THREADS, 0, st>>>(x, v, k, n, scratch);
  PCG_CHECK_LAUNCH("pcg_dots_f64_noalloc/partials");
  finish_sum_kernel<<<1, EW_THREADS, 0, st>>>(scratch, nb, k, out);
  PCG_CHECK_LAUNCH("pcg_dots_f64_noalloc");
  return 0;
}

// inv1[i,a] = 1/(e_i - e_a), inv2[i,j,a,b] = 1/(e_i + e_j - e_a - e_b): the Jacobi
// preconditioner of the amplitude update (pycc/ccwfn.py:195-198), computed once.
extern "C" int pcg_inv_denominators_f64(const double* eps, long long no, long long nv,
                                        double* inv1, double* inv2, void* stream) {
  if (!eps || !inv1 || !inv2 || no <= 0 || nv <= 0) {
    set_error("pcg_inv_denominators_f64: bad arguments");
    return -1;
  }
  const long long n = no * nv + no * no * nv * nv;
  inv_denom_kernel<<<ew_blocks(n), EW_THREADS, 0, (cudaStream_t)stream>>>(eps, no, nv, inv1, inv2);
  PCG_CHECK_LAUNCH("pcg_inv_denominators_f64");
  return 0;
}

// t += r * inv over n elements (t1 and t2 as one flat vector when they are adjacent);
// *rms2 = sum (r*inv)^2.  work >= 1024 doubles.  solve_cc update (pycc/ccwfn.py:281-284).
extern "C" int pcg_update_inv_f64(double* t, const double* r, const double* inv, long long n,
                                  double* work, long long work_len, double* rms2, void* stream) {
  if (!t || !r || !inv || !rms2 || !work || n < 0) {
    set_error("pcg_update_inv_f64: bad arguments");
    return -1;
  }
  if (!check_work(work_len, RED_BLOCKS, "pcg_update_inv_f64")) return -1;
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = std::min(ew_blocks(n), RED_BLOCKS);
  update_inv_kernel<<<nb, EW_THREADS, 0, st>>>(t, r, inv, n, work);
  PCG_CHECK_LAUNCH("pcg_update_inv_f64/update");
  finish_sum_kernel<<<1, EW_THREADS, 0, st>>>(work, nb, 1, rms2);
  PCG_CHECK_LAUNCH("pcg_update_inv_f64");
  return 0;
}

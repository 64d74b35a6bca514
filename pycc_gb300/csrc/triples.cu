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
  const T* eoovv;     // <ij|ab> [o][o][v][v], in the partials' type
  const double* t1;   // [o][v]
  const T* t2;        // [o][o][v][v], in the partials' type
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

// ---- FP32 path: tiles of the (a, b, c) cube -------------------------------------------
// One block per (triple, tile triple A >= B >= C) of TT^3 tiles.  W at the six orderings of
// the tile sets, W[XYZ][x][y][z] with (X, Y, Z) = (A,B,C), (A,C,B), (B,A,C), (B,C,A),
// (C,A,B), (C,B,A), is staged in shared memory from the column-major partials, each read
// as aligned runs of TT consecutive floats (one 32-byte sector): P3[x][y][z] and P2[y][x][z]
// along z, P1[z][x][y] along y.  <ij|xy>, <ik|xz>, <jk|yz> (and t2 when f_ov is present)
// over the 3 TT indices of A, B and C, the t1 rows and the orbital energies are staged
// too.  The block then evaluates every a >= b >= c of its tiles with the same weights and
// formula as the per-(triple, a) kernel, in FP32, and writes one FP64 partial.
constexpr int TT = 8;
constexpr int TT3 = 3 * TT;
constexpr int TE2_THREADS = 256;

struct TiledStage {
  float w[6][TT][TT][TT + 1];
  float e[3][TT3][TT3 + 1];   // <ij|..>, <ik|..>, <jk|..> over the union of A, B, C
  float d2[3][TT3][TT3 + 1];  // t2_ij.., t2_ik.., t2_jk.. (non-canonical only)
  float t1r[3][TT3];          // t1[i], t1[j], t1[k] over the union
  float fr[3][TT3];           // f_ov[i], f_ov[j], f_ov[k] over the union
  float ev[TT3];              // eps of the virtual orbitals of the union
  double red[TE2_THREADS / 32];
};

// Tile triple u -> (A, B, C), A >= B >= C, in the order u = A(A+1)(A+2)/6 + B(B+1)/2 + C:
// root estimates, then exact integer corrections (u < 2^31).
__device__ __forceinline__ void tile_triple(long long u, int& A, int& B, int& C) {
  auto tet = [](long long a) { return a * (a + 1) * (a + 2) / 6; };
  auto tri = [](long long b) { return b * (b + 1) / 2; };
  long long a = (long long)cbrtf(6.0f * (float)u);
  while (a > 0 && tet(a) > u) --a;
  while (tet(a + 1) <= u) ++a;
  const long long r = u - tet(a);
  long long b = (long long)((sqrtf(8.0f * (float)r + 1.0f) - 1.0f) * 0.5f);
  while (b > 0 && tri(b) > r) --b;
  while (tri(b + 1) <= r) ++b;
  A = (int)a;
  B = (int)b;
  C = (int)(r - tri(b));
}

__device__ __forceinline__ float dval_tiled(const TiledStage& s, bool fov, int lx, int ly,
                                            int lz) {
  float d = s.e[0][lx][ly] * s.t1r[2][lz] + s.e[1][lx][lz] * s.t1r[1][ly] +
            s.e[2][ly][lz] * s.t1r[0][lx];
  if (fov)
    d += s.d2[0][lx][ly] * s.fr[2][lz] + s.d2[1][lx][lz] * s.fr[1][ly] +
         s.d2[2][ly][lz] * s.fr[0][lx];
  return d;
}

// orderings of the tile sets (A, B, C), so = 0..5: (A,B,C), (A,C,B), (B,A,C), (B,C,A),
// (C,A,B), (C,B,A); kord(so, q) is the set in position q, two bits per entry
__host__ __device__ constexpr int kord(int so, int q) {
  return (int)((0x192261624ULL >> (2 * (3 * so + q))) & 3u);
}

// five resident blocks per SM (48 registers): short, latency-bound blocks gain more from the
// extra block than they lose to the few spilled registers of the staging phase
__global__ void __launch_bounds__(TE2_THREADS, 5) triples_energy_tiled_kernel(
    const TripArgs<float> p, long long ntt) {
  __shared__ TiledStage s;
  const int t = blockIdx.y;
  const long long u = blockIdx.x;
  int A, B, C;
  tile_triple(u, A, B, C);
  const long long org[3] = {(long long)A * TT, (long long)B * TT, (long long)C * TT};
  const int i = p.ijk[3 * t], j = p.ijk[3 * t + 1], k = p.ijk[3 * t + 2];
  const float* P1 = p.P1 + t * p.pstride;
  const float* P2 = p.P2 + t * p.pstride;
  const float* P3 = p.P3 + t * p.pstride;
  const long long o = p.no, v = p.nv;
  const int tid = threadIdx.x;
  constexpr int NE = TT * TT * TT / TE2_THREADS;  // tile elements per thread and ordering
  static_assert(TT * TT * TT % TE2_THREADS == 0, "whole tile elements per thread");
  // orbital of staged-union index l (8 q + r is orbital org[q] + r)
  auto uorb = [&](int l) -> long long {
    return (l < TT ? org[0] : (l < 2 * TT ? org[1] : org[2])) + (l % TT);
  };
  // Every global load of the block is issued before the first shared-memory store:
  // P3[x][y][z] + P2[y][x][z] (runs along z), P1[z][x][y] (runs along y), the integral
  // and amplitude slices.  The ordering index is unrolled, so the tile origins are
  // registers; offsets are 32-bit (v^3 < 2^31, checked by the host), and a thread's
  // repeats differ by a constant stride (TE2_THREADS / TT^2 steps of the slowest index).
  const int vv = (int)v, v2 = vv * vv;
  const bool full = (vv % TT) == 0;  // every tile inside the cube: no bounds checks
  constexpr int RS = TE2_THREADS / (TT * TT);
  const int e0 = tid;
  const int s_hi = e0 / (TT * TT), s_mid = (e0 / TT) % TT, s_lo = e0 % TT;
  float p32[6][NE], p1v[6][NE];
#pragma unroll
  for (int so = 0; so < 6; ++so) {
    const int X0 = (int)org[kord(so, 0)], Y0 = (int)org[kord(so, 1)], Z0 = (int)org[kord(so, 2)];
    // pass-1 mapping (x, y, z) = (hi, mid, lo); pass-2 mapping (z, x, y) = (hi, mid, lo)
    const int x1 = X0 + s_hi, y1 = Y0 + s_mid, z1 = Z0 + s_lo;
    const int z2 = Z0 + s_hi, x2 = X0 + s_mid, y2 = Y0 + s_lo;
    const int o3 = (x1 * vv + y1) * vv + z1, o2 = (y1 * vv + x1) * vv + z1;
    const int o1 = (z2 * vv + x2) * vv + y2;
#pragma unroll
    for (int rep = 0; rep < NE; ++rep) {
      const int d = rep * RS;  // steps of the slowest index
      if (full) {
        p32[so][rep] = P3[o3 + d * v2] + P2[o2 + d * vv];
        p1v[so][rep] = P1[o1 + d * v2];
      } else {
        p32[so][rep] = (x1 + d < vv && y1 < vv && z1 < vv)
                           ? P3[o3 + d * v2] + P2[o2 + d * vv] : 0.f;
        p1v[so][rep] = (z2 + d < vv && x2 < vv && y2 < vv) ? P1[o1 + d * v2] : 0.f;
      }
    }
  }
  // <ij|xy>, <ik|xz>, <jk|yz> (and t2) over the union of the tiles, FP32: per pair and
  // row, three runs of TT orbitals, read as float4 when the tiles are whole (v % TT == 0
  // keeps every run 16-byte aligned)
  constexpr int QPR = TT / 4;                      // float4 per run
  constexpr int NSEG = 3 * TT3 * 3 * QPR;          // pairs x rows x runs x float4
  constexpr int NS = (NSEG + TE2_THREADS - 1) / TE2_THREADS;
  float4 ev[NS], tv[NS];
#pragma unroll
  for (int rp = 0; rp < NS; ++rp) {
    const int e = tid + rp * TE2_THREADS;
    ev[rp] = make_float4(0.f, 0.f, 0.f, 0.f);
    tv[rp] = ev[rp];
    if (e < NSEG) {
      const int pr = e / (TT3 * 3 * QPR), r = e % (TT3 * 3 * QPR);
      const int l1 = r / (3 * QPR), c = r % (3 * QPR);
      const long long x = uorb(l1), y = uorb((c / QPR) * TT) + 4 * (c % QPR);
      const int a0 = pr == 2 ? j : i, a1 = pr == 0 ? j : k;  // pairs ij, ik, jk
      const long long at = ((a0 * o + a1) * v + x) * v + y;
      if (full) {
        ev[rp] = *reinterpret_cast<const float4*>(p.eoovv + at);
        if (p.fov) tv[rp] = *reinterpret_cast<const float4*>(p.t2 + at);
      } else if (x < v) {
        float* pe = &ev[rp].x;
        float* pt = &tv[rp].x;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (y + q < v) {
            pe[q] = p.eoovv[at + q];
            if (p.fov) pt[q] = p.t2[at + q];
          }
      }
    }
  }
  if (tid < 3 * TT3) {
    const int q = tid / TT3, l = tid % TT3;
    const long long x = uorb(l);
    const int occ = q == 0 ? i : (q == 1 ? j : k);
    s.t1r[q][l] = x < v ? f64_to_f32(p.t1[occ * v + x]) : 0.f;
    s.fr[q][l] = (x < v && p.fov) ? f64_to_f32(p.fov[occ * v + x]) : 0.f;
    if (q == 0) s.ev[l] = x < v ? f64_to_f32(p.eps[o + x]) : 0.f;
  }
#pragma unroll
  for (int so = 0; so < 6; ++so)
#pragma unroll
    for (int rep = 0; rep < NE; ++rep) {
      const int e = tid + rep * TE2_THREADS;
      s.w[so][e / (TT * TT)][(e / TT) % TT][e % TT] = p32[so][rep];
    }
#pragma unroll
  for (int rp = 0; rp < NS; ++rp) {
    const int e = tid + rp * TE2_THREADS;
    if (e < NSEG) {
      const int pr = e / (TT3 * 3 * QPR), r = e % (TT3 * 3 * QPR);
      const int l1 = r / (3 * QPR), c = r % (3 * QPR);
      const int l2 = (c / QPR) * TT + 4 * (c % QPR);
      const float* pe = &ev[rp].x;
      const float* pt = &tv[rp].x;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        s.e[pr][l1][l2 + q] = pe[q];
        s.d2[pr][l1][l2 + q] = pt[q];
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int so = 0; so < 6; ++so)
#pragma unroll
    for (int rep = 0; rep < NE; ++rep) {
      const int e = tid + rep * TE2_THREADS;
      s.w[so][(e / TT) % TT][e % TT][e / (TT * TT)] += p1v[so][rep];
    }
  __syncthreads();
  const float eo = f64_to_f32(p.eps[i] + p.eps[j] + p.eps[k]);
  const bool fov = p.fov != nullptr;
  float acc = 0.f;
#pragma unroll
  for (int rep = 0; rep < NE; ++rep) {
    const int e = tid + rep * TE2_THREADS;
    const int al = e / (TT * TT), bl = (e / TT) % TT, cl = e % TT;
    const long long a = org[0] + al, b = org[1] + bl, c = org[2] + cl;
    if (a >= v || b > a || c > b) continue;
    const int la = al, lb = TT + bl, lc = 2 * TT + cl;  // indices in the staged union
    float W[6], V[6];
    W[0] = s.w[0][al][bl][cl];
    W[1] = s.w[1][al][cl][bl];
    W[2] = s.w[2][bl][al][cl];
    W[3] = s.w[3][bl][cl][al];
    W[4] = s.w[4][cl][al][bl];
    W[5] = s.w[5][cl][bl][al];
    const float wt = (float)(1 + (a == b) + (a == c) + (b == c));
    const float rw = 1.f / wt;
    V[0] = (W[0] + dval_tiled(s, fov, la, lb, lc)) * rw;
    V[1] = (W[1] + dval_tiled(s, fov, la, lc, lb)) * rw;
    V[2] = (W[2] + dval_tiled(s, fov, lb, la, lc)) * rw;
    V[3] = (W[3] + dval_tiled(s, fov, lb, lc, la)) * rw;
    V[4] = (W[4] + dval_tiled(s, fov, lc, la, lb)) * rw;
    V[5] = (W[5] + dval_tiled(s, fov, lc, lb, la)) * rw;
    float X = 0.f;
#pragma unroll
    for (int q = 0; q < 6; ++q) X += W[q] * V[q];
    const float Y = V[0] + V[3] + V[4], Z = V[1] + V[2] + V[5];
    const float Wc = W[0] + W[3] + W[4], Wa = W[1] + W[2] + W[5];
    const float S = (Y - 2.f * Z) * Wc + (Z - 2.f * Y) * Wa + 3.f * X;
    const float D = eo - s.ev[la] - s.ev[lb] - s.ev[lc];
    acc += S / D;
  }
  // warp sums as an FP32 tree (a few combinations per thread), the block's eight warp
  // sums in FP64
  float wsum = acc;
  for (int sh = 16; sh > 0; sh >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, sh);
  if ((tid & 31) == 0) s.red[tid >> 5] = f32_to_f64(wsum);
  __syncthreads();
  if (tid < 32) {
    double r = (tid < TE2_THREADS / 32) ? s.red[tid] : 0.0;
    for (int sh = 16; sh > 0; sh >>= 1) r += __shfl_xor_sync(0xffffffffu, r, sh);
    const double fac = 2.0 - ((i == j) + (i == k) + (j == k));
    if (tid == 0) p.part[(long long)t * ntt + u] = fac * r;
  }
}

long long tile_triples(long long nv) {
  const long long nt = (nv + TT - 1) / TT;
  return nt * (nt + 1) * (nt + 2) / 6;
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
// tensors and FP32 element arithmetic (the tensor-core path, tiled kernel); otherwise FP64
// throughout.  Writes pcg_triples_part_len(fp32, nv) FP64 partials per triple; the caller
// sums them.  pycc/cctriples.py:177-240.
extern "C" int pcg_triples_energy(int fp32, const void* P1, const void* P2, const void* P3,
                                  long long pstride, const int* ijk, int ntrip,
                                  const double* eps, const void* eoovv, const double* t1,
                                  const void* t2, const double* fov, long long no,
                                  long long nv, double* part, void* stream) {
  if (ntrip < 1 || ntrip > 65535 || nv < 1 || nv > 0x7fffffff || !P1 || !P2 || !P3 || !ijk ||
      !eps || !eoovv || !t1 || !t2 || !part) {
    set_error("pcg_triples_energy: bad arguments (ntrip=%d)", ntrip);
    return -1;
  }
  dim3 grid((unsigned)nv, (unsigned)ntrip);
  cudaStream_t st = (cudaStream_t)stream;
  if (fp32) {
    const long long ntt = tile_triples(nv);
    if (ntt > 0x7fffffffLL || nv * nv * nv > 0x7fffffffLL) {
      set_error("pcg_triples_energy: nv=%lld too large", nv);
      return -1;
    }
    if (((uintptr_t)eoovv & 15u) || ((uintptr_t)t2 & 15u)) {
      set_error("pcg_triples_energy: FP32 eoovv and t2 must be 16-byte aligned");
      return -1;
    }
    TripArgs<float> a{(const float*)P1, (const float*)P2, (const float*)P3, pstride, ijk, ntrip,
                      eps, (const float*)eoovv, t1, (const float*)t2, fov, no, nv, part};
    triples_energy_tiled_kernel<<<dim3((unsigned)ntt, (unsigned)ntrip), TE2_THREADS, 0, st>>>(
        a, ntt);
  } else {
    TripArgs<double> a{(const double*)P1, (const double*)P2, (const double*)P3, pstride, ijk,
                       ntrip, eps, (const double*)eoovv, t1, (const double*)t2, fov, no, nv,
                       part};
    triples_energy_kernel<double><<<grid, TE_THREADS, 0, st>>>(a);
  }
  PCG_CHECK_LAUNCH("pcg_triples_energy");
  return 0;
}

// FP64 partials per triple written by pcg_triples_energy: one per virtual index a (FP64),
// one per tile triple of the (a, b, c) cube (FP32).
extern "C" long long pcg_triples_part_len(int fp32, long long nv) {
  return fp32 ? tile_triples(nv) : nv;
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

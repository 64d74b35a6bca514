// FP64 strided tensor contraction on the FP64 tensor pipe (DMMA, mma.sync m8n8k4 f64).
//
//   C[m, n] = beta * C[m, n] + alpha * sum_k A[m, k] * B[n, k]
//
// m, n and k are flat indices over up to four sub-indices each; every sub-index carries
// its own element stride in both tensors that hold it, so index permutations of the
// operands and of the output (the einsum strings of the CCSD residual, e.g.
// 'imae,mbej->ijab') are folded into address generation and never materialised.
// This is the oracle-grade GPU path of the engine: exact FP64 products, FP64 sums.
#include "common.cuh"
#include <algorithm>

namespace pcg {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 128;

struct F64Args {
  SubIdx m, n, k;  // m: (A, C) strides; n: (B, C) strides; k: (A, B) strides
  long long M, N, K;
  long long k_per_split;
  double alpha, beta;
  const double* A;
  const double* B;
  double* C;
  int a_kfast, b_kfast, atomic_out;
};

__device__ __forceinline__ void dmma(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(NT) contract_f64_kernel(const F64Args p) {
  __shared__ double As[BK][BM + 2];
  __shared__ double Bs[BK][BN + 2];
  __shared__ long long aoff[BM], coffm[BM], boff[BN], coffn[BN];
  __shared__ long long akoff[BK], bkoff[BK];

  const int tid = threadIdx.x;
  const long long m0 = (long long)blockIdx.y * BM;
  const long long n0 = (long long)blockIdx.x * BN;
  const long long kbeg = (long long)blockIdx.z * p.k_per_split;
  const long long kend = min(p.K, kbeg + p.k_per_split);

  if (tid < BM) {
    long long r = m0 + tid, o0 = 0, o1 = 0;
    if (r < p.M) sub_offsets(p.m, r, o0, o1);
    aoff[tid] = o0;
    coffm[tid] = o1;
  } else {
    int t = tid - BM;
    long long r = n0 + t, o0 = 0, o1 = 0;
    if (r < p.N) sub_offsets(p.n, r, o0, o1);
    boff[t] = o0;
    coffn[t] = o1;
  }

  const int warp = tid >> 5, lane = tid & 31;
  const int wm = warp >> 1, wn = warp & 1;
  const int g = lane >> 2, t4 = lane & 3;
  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

  double ra[8], rb[8];
  auto kofs = [&](long long kt) {
    if (tid < BK) {
      long long r = kt + tid, o0 = 0, o1 = 0;
      if (r < kend) sub_offsets(p.k, r, o0, o1);
      akoff[tid] = o0;
      bkoff[tid] = o1;
    }
  };
  auto load = [&](long long kt) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      int e = tid + NT * i;
      int mm, kk;
      if (p.a_kfast) { kk = e % BK; mm = e / BK; } else { mm = e % BM; kk = e / BM; }
      bool ok = (m0 + mm < p.M) && (kt + kk < kend);
      ra[i] = ok ? __ldg(p.A + aoff[mm] + akoff[kk]) : 0.0;
      int nn;
      if (p.b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BN; kk = e / BN; }
      ok = (n0 + nn < p.N) && (kt + kk < kend);
      rb[i] = ok ? __ldg(p.B + boff[nn] + bkoff[kk]) : 0.0;
    }
  };
  auto store = [&]() {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      int e = tid + NT * i;
      int mm, kk;
      if (p.a_kfast) { kk = e % BK; mm = e / BK; } else { mm = e % BM; kk = e / BM; }
      As[kk][mm] = ra[i];
      int nn;
      if (p.b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BN; kk = e / BN; }
      Bs[kk][nn] = rb[i];
    }
  };

  kofs(kbeg);
  __syncthreads();
  if (kbeg < kend) load(kbeg);
  for (long long kt = kbeg; kt < kend; kt += BK) {
    __syncthreads();  // previous compute done with As/Bs and akoff
    store();
    if (kt + BK < kend) kofs(kt + BK);
    __syncthreads();
    if (kt + BK < kend) load(kt + BK);  // global loads overlap the DMMAs below
#pragma unroll
    for (int ks = 0; ks < BK; ks += 4) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[ks + t4][wm * 32 + i * 8 + g];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[ks + t4][wn * 32 + j * 8 + g];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) dmma(acc[i][j], a[i], b[j]);
    }
  }

#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int row = wm * 32 + i * 8 + g;
    if (m0 + row >= p.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        int col = wn * 32 + j * 8 + 2 * t4 + h;
        if (n0 + col >= p.N) continue;
        double* dst = p.C + coffm[row] + coffn[col];
        double v = p.alpha * acc[i][j][h];
        if (p.atomic_out) {
          atomicAdd(dst, v);
        } else if (p.beta == 0.0) {
          *dst = v;
        } else {
          *dst = p.beta * *dst + v;
        }
      }
    }
  }
}

// C[m, n] *= beta over the strided M x N range (used before a split-K accumulation).
__global__ void scale_strided_kernel(SubIdx m, SubIdx n, long long M, long long N, double beta,
                                     double* C) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = M * N;
  for (; idx < total; idx += (long long)gridDim.x * blockDim.x) {
    long long r = idx / N, c = idx % N, a0, a1, b0, b1;
    sub_offsets(m, r, a0, a1);
    sub_offsets(n, c, b0, b1);
    double* dst = C + a1 + b1;
    *dst = (beta == 0.0) ? 0.0 : beta * *dst;
  }
}

// Stores one partial (or the whole) dot product of an output element: with K split across
// blocks (blockIdx.y) the partials are atomic FP64 adds onto C, which the host scaled by
// beta first.
__device__ __forceinline__ void gemv_store(const F64Args& p, double* dst, double acc) {
  const double v = p.alpha * acc;
  if (p.atomic_out)
    atomicAdd(dst, v);
  else
    *dst = (p.beta == 0.0) ? v : p.beta * *dst + v;
}

// Outputs with a degenerate free dimension (matrix-vector shapes such as 'nf,mnef->me', and
// full dot products): one warp per output element and K slice (blockIdx.y), a warp-wide FP64
// dot over the slice.  HBM-bound.
__global__ void contract_gemv_kernel(const F64Args p) {
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  const long long total = p.M * p.N;
  const long long kbeg = (long long)blockIdx.y * p.k_per_split;
  const long long kend = min(p.K, kbeg + p.k_per_split);
  for (long long o = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; o < total;
       o += warps) {
    const long long m = o / p.N, n = o % p.N;
    long long am, cm, bn, cn;
    sub_offsets(p.m, m, am, cm);
    sub_offsets(p.n, n, bn, cn);
    double acc = 0.0;
    if (p.k.n == 1) {
      const long long sa = p.k.s0[0], sb = p.k.s1[0];
      for (long long k = kbeg + lane; k < kend; k += 32) acc += p.A[am + k * sa] * p.B[bn + k * sb];
    } else {
      for (long long k = kbeg + lane; k < kend; k += 32) {
        long long ka, kb;
        sub_offsets(p.k, k, ka, kb);
        acc += p.A[am + ka] * p.B[bn + kb];
      }
    }
    for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
    if (lane == 0) gemv_store(p, p.C + cm + cn, acc);
  }
}

// Matrix-vector shapes whose operand B is unit-stride along the output's innermost
// sub-index: one thread per output, consecutive threads on consecutive outputs (coalesced
// B reads); the K offsets are staged in shared memory once per block; blockIdx.y is the K
// slice.
__global__ void __launch_bounds__(256) contract_gemv_thread_kernel(const F64Args p) {
  __shared__ long long ka[256], kb[256];
  const long long o = (long long)blockIdx.x * 256 + threadIdx.x;
  const bool valid = o < p.M * p.N;
  const long long kbeg = (long long)blockIdx.y * p.k_per_split;
  const long long kend = min(p.K, kbeg + p.k_per_split);
  long long am = 0, cm = 0, bn = 0, cn = 0;
  if (valid) {
    sub_offsets(p.m, o / p.N, am, cm);
    sub_offsets(p.n, o % p.N, bn, cn);
  }
  double acc = 0.0;
  for (long long k0 = kbeg; k0 < kend; k0 += 256) {
    __syncthreads();
    const long long k = k0 + threadIdx.x;
    if (k < kend) sub_offsets(p.k, k, ka[threadIdx.x], kb[threadIdx.x]);
    __syncthreads();
    const int kn = (int)min((long long)256, kend - k0);
    if (valid)
      for (int j = 0; j < kn; ++j) acc += p.A[am + ka[j]] * p.B[bn + kb[j]];
  }
  if (valid) gemv_store(p, p.C + cm + cn, acc);
}

// K slices for a matrix-vector launch of `blocks` output blocks: enough blocks for about
// eight per SM, each slice at least `kmin` long; beta is applied up front when split.
long long gemv_splits(const F64Args& p, long long blocks, long long kmin);

// Reorder sub-indices by decreasing |stride| in the operand (s0), unit stride innermost.
void sort_by_operand_stride(SubIdx& d) {
  for (int i = 0; i < d.n; ++i)
    for (int j = i + 1; j < d.n; ++j)
      if (llabs(d.s0[j]) > llabs(d.s0[i])) {
        std::swap(d.ext[i], d.ext[j]);
        std::swap(d.s0[i], d.s0[j]);
        std::swap(d.s1[i], d.s1[j]);
      }
}

bool fill_sub(SubIdx& d, int n, const long long* ext, const long long* s0, const long long* s1,
              const char* what) {
  if (n < 0 || n > kMaxSub) {
    set_error("pcg_contract_f64: %s has %d sub-indices (max %d)", what, n, kMaxSub);
    return false;
  }
  if (n > 0 && (!ext || !s0 || !s1)) {
    set_error("pcg_contract_f64: %s extents or strides missing", what);
    return false;
  }
  d.n = n;
  for (int q = 0; q < n; ++q) {
    if (ext[q] <= 0) {
      set_error("pcg_contract_f64: %s extent %lld must be positive", what, ext[q]);
      return false;
    }
    d.ext[q] = ext[q];
    d.s0[q] = s0[q];
    d.s1[q] = s1[q];
  }
  if (n == 0) {  // an empty group is a single index of extent 1
    d.n = 1;
    d.ext[0] = 1;
    d.s0[0] = 0;
    d.s1[0] = 0;
  }
  return true;
}

long long gemv_splits(const F64Args& p, long long blocks, long long kmin) {
  const long long want = 8LL * 152;
  if (blocks >= want || p.K < 2 * kmin) return 1;
  long long splits = std::min((want + blocks - 1) / blocks, p.K / kmin);
  return std::max(1LL, std::min(splits, 65535LL));
}

int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
  }
  return sms;
}

}  // namespace
}  // namespace pcg

extern "C" int pcg_contract_f64(int m_n, const long long* m_ext, const long long* m_sa,
                                const long long* m_sc, int n_n, const long long* n_ext,
                                const long long* n_sb, const long long* n_sc, int k_n,
                                const long long* k_ext, const long long* k_sa,
                                const long long* k_sb, double alpha, const double* A,
                                const double* B, double beta, double* C, void* stream) {
  using namespace pcg;
  F64Args p{};
  if (!fill_sub(p.m, m_n, m_ext, m_sa, m_sc, "M") || !fill_sub(p.n, n_n, n_ext, n_sb, n_sc, "N") ||
      !fill_sub(p.k, k_n, k_ext, k_sa, k_sb, "K"))
    return -1;
  if (!A || !B || !C) {
    set_error("pcg_contract_f64: null operand pointer");
    return -1;
  }
  p.M = sub_total(p.m);
  p.N = sub_total(p.n);
  p.K = sub_total(p.k);
  p.alpha = alpha;
  p.beta = beta;
  p.A = A;
  p.B = B;
  p.C = C;
  // Load the operand tile along whichever index is unit-stride in memory.
  p.a_kfast = (p.k.s0[p.k.n - 1] == 1) ? 1 : 0;
  p.b_kfast = (p.k.s1[p.k.n - 1] == 1) ? 1 : 0;
  cudaStream_t st = (cudaStream_t)stream;
  if (p.M == 1 || p.N == 1) {
    // one free side: enumerate the outputs along the big operand's unit-stride index
    F64Args q = p;
    if (q.M == 1) {
      sort_by_operand_stride(q.n);
    } else {  // N == 1: swap roles so the free index is on the B side
      std::swap(q.m, q.n);
      std::swap(q.M, q.N);
      std::swap(q.A, q.B);
      for (int i = 0; i < q.k.n; ++i) std::swap(q.k.s0[i], q.k.s1[i]);
      sort_by_operand_stride(q.n);
    }
    if (q.n.s0[q.n.n - 1] == 1 && q.M * q.N >= 1024) {
      const long long blocks = (q.M * q.N + 255) / 256;
      const long long splits = gemv_splits(q, blocks, 1024);
      q.k_per_split = (q.K + splits - 1) / splits;
      q.atomic_out = splits > 1;
      if (q.atomic_out && beta != 1.0) {
        scale_strided_kernel<<<(int)std::min<long long>((q.M * q.N + 255) / 256, 4096), 256, 0,
                               st>>>(q.m, q.n, q.M, q.N, beta, C);
        PCG_CHECK_LAUNCH("pcg_contract_f64/gemv_scale");
      }
      contract_gemv_thread_kernel<<<dim3((unsigned)blocks, (unsigned)splits), 256, 0, st>>>(q);
      PCG_CHECK_LAUNCH("pcg_contract_f64/gemv_thread");
      return 0;
    }
  }
  if (p.M < 8 || p.N < 8) {
    long long warps = p.M * p.N;
    int blocks = (int)std::min<long long>((warps * 32 + 255) / 256, 152LL * 64);
    const long long splits = gemv_splits(p, blocks, 4096);
    p.k_per_split = (p.K + splits - 1) / splits;
    p.atomic_out = splits > 1;
    if (p.atomic_out && beta != 1.0) {
      scale_strided_kernel<<<(int)std::min<long long>((p.M * p.N + 255) / 256, 4096), 256, 0,
                             st>>>(p.m, p.n, p.M, p.N, beta, C);
      PCG_CHECK_LAUNCH("pcg_contract_f64/gemv_scale");
    }
    contract_gemv_kernel<<<dim3((unsigned)blocks, (unsigned)splits), 256, 0, st>>>(p);
    PCG_CHECK_LAUNCH("pcg_contract_f64/gemv");
    return 0;
  }
  long long mt = (p.M + BM - 1) / BM, nt = (p.N + BN - 1) / BN;
  if (mt > 65535) {
    set_error("pcg_contract_f64: M=%lld too large", p.M);
    return -1;
  }
  long long tiles = mt * nt;
  long long target = 2LL * num_sms();
  long long splits = 1;
  if (tiles < target && p.K >= 8 * BK) {
    splits = (target + tiles - 1) / tiles;
    long long maxs = p.K / (4 * BK);
    if (splits > maxs) splits = maxs;
    if (splits > 64) splits = 64;
    if (splits < 1) splits = 1;
  }
  long long kps = (p.K + splits - 1) / splits;
  kps = ((kps + BK - 1) / BK) * BK;
  splits = (p.K + kps - 1) / kps;
  p.k_per_split = kps;
  p.atomic_out = splits > 1;
  if (p.atomic_out && beta != 1.0) {
    long long total = p.M * p.N;
    int blocks = (int)std::min<long long>((total + 255) / 256, 4096);
    scale_strided_kernel<<<blocks, 256, 0, st>>>(p.m, p.n, p.M, p.N, beta, C);
    PCG_CHECK_LAUNCH("pcg_contract_f64/scale");
  }
  dim3 grid((unsigned)nt, (unsigned)mt, (unsigned)splits);
  contract_f64_kernel<<<grid, NT, 0, st>>>(p);
  PCG_CHECK_LAUNCH("pcg_contract_f64");
  return 0;
}

// ---------------------------------------------------------------------------------------
// Sum of up to four FP64 contractions into one output tile:
//   C[m, n] = beta * C[m, n] + sum_t alpha_t * sum_k A_t[m, k] * B_t[n, k]
// All terms share the M / N extents and the C strides; each term has its own operands, A / B
// strides and K range.  Used where several einsum terms land on the same output (the four
// terms of one orientation of the connected triples), so the output is written once.
// ---------------------------------------------------------------------------------------
namespace pcg {
namespace {
constexpr int kMaxTerms = 4;

struct MultiArgs {
  int nterm;
  SubIdx m, n;                 // ext + C strides (s1); s0 unused
  long long ma[kMaxTerms][kMaxSub];  // per-term A strides of the M sub-indices
  long long nb[kMaxTerms][kMaxSub];  // per-term B strides of the N sub-indices
  SubIdx k[kMaxTerms];         // per-term K (A strides s0, B strides s1)
  long long K[kMaxTerms];
  double alpha[kMaxTerms];
  const double* A[kMaxTerms];
  const double* B[kMaxTerms];
  long long M, N;
  double beta;
  double* C;
};

__device__ __forceinline__ long long strided_offset(const SubIdx& d, const long long* s,
                                                    long long r) {
  long long o = 0;
  for (int q = d.n - 1; q >= 0; --q) {
    const long long e = d.ext[q];
    o += (r % e) * s[q];
    r /= e;
  }
  return o;
}

__global__ void __launch_bounds__(NT) contract_multi_f64_kernel(const MultiArgs p) {
  __shared__ double As[BK][BM + 2];
  __shared__ double Bs[BK][BN + 2];
  __shared__ long long aoff[BM], coffm[BM], boff[BN], coffn[BN];
  __shared__ long long akoff[BK], bkoff[BK];
  const int tid = threadIdx.x;
  const long long m0 = (long long)blockIdx.y * BM;
  const long long n0 = (long long)blockIdx.x * BN;
  const int warp = tid >> 5, lane = tid & 31;
  const int wm = warp >> 1, wn = warp & 1;
  const int g = lane >> 2, t4 = lane & 3;
  double acc[4][4][2];
  if (tid < BM) {
    const long long r = m0 + tid;
    coffm[tid] = (r < p.M) ? strided_offset(p.m, p.m.s1, r) : 0;
  } else {
    const int t = tid - BM;
    const long long r = n0 + t;
    coffn[t] = (r < p.N) ? strided_offset(p.n, p.n.s1, r) : 0;
  }
  double out[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) out[i][j][0] = out[i][j][1] = 0.0;

  for (int term = 0; term < p.nterm; ++term) {
    __syncthreads();
    if (tid < BM) {
      const long long r = m0 + tid;
      aoff[tid] = (r < p.M) ? strided_offset(p.m, p.ma[term], r) : 0;
    } else {
      const int t = tid - BM;
      const long long r = n0 + t;
      boff[t] = (r < p.N) ? strided_offset(p.n, p.nb[term], r) : 0;
    }
    const SubIdx& kd = p.k[term];
    const long long K = p.K[term];
    const double* Ap = p.A[term];
    const double* Bp = p.B[term];
    const int a_kfast = (kd.s0[kd.n - 1] == 1);
    const int b_kfast = (kd.s1[kd.n - 1] == 1);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
    for (long long kt = 0; kt < K; kt += BK) {
      __syncthreads();
      if (tid < BK) {
        long long o0 = 0, o1 = 0;
        if (kt + tid < K) sub_offsets(kd, kt + tid, o0, o1);
        akoff[tid] = o0;
        bkoff[tid] = o1;
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int e = tid + NT * i;
        int mm, kk;
        if (a_kfast) { kk = e % BK; mm = e / BK; } else { mm = e % BM; kk = e / BM; }
        As[kk][mm] = (m0 + mm < p.M && kt + kk < K) ? __ldg(Ap + aoff[mm] + akoff[kk]) : 0.0;
        int nn;
        if (b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BN; kk = e / BN; }
        Bs[kk][nn] = (n0 + nn < p.N && kt + kk < K) ? __ldg(Bp + boff[nn] + bkoff[kk]) : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int ks = 0; ks < BK; ks += 4) {
        double a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[ks + t4][wm * 32 + i * 8 + g];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[ks + t4][wn * 32 + j * 8 + g];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) dmma(acc[i][j], a[i], b[j]);
      }
    }
    const double al = p.alpha[term];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        out[i][j][0] += al * acc[i][j][0];
        out[i][j][1] += al * acc[i][j][1];
      }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int row = wm * 32 + i * 8 + g;
    if (m0 + row >= p.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int col = wn * 32 + j * 8 + 2 * t4 + h;
        if (n0 + col >= p.N) continue;
        double* dst = p.C + coffm[row] + coffn[col];
        *dst = (p.beta == 0.0) ? out[i][j][h] : p.beta * *dst + out[i][j][h];
      }
  }
}
}  // namespace
}  // namespace pcg

// C = beta*C + sum_t alpha[t] * A_t . B_t^T over nterm (<= 4) terms.  The M / N sub-index
// extents (m_ext, n_ext) and C strides (m_sc, n_sc) are common; per term t: A strides of the
// M sub-indices m_sa[t*4 + q], B strides of the N sub-indices n_sb[t*4 + q], and its K
// group k_n[t], k_ext[t*4 + q], k_sa[t*4 + q], k_sb[t*4 + q].
extern "C" int pcg_contract_multi_f64(int nterm, int m_n, const long long* m_ext,
                                      const long long* m_sc, const long long* m_sa, int n_n,
                                      const long long* n_ext, const long long* n_sc,
                                      const long long* n_sb, const int* k_n,
                                      const long long* k_ext, const long long* k_sa,
                                      const long long* k_sb, const double* alpha,
                                      const double* const* A, const double* const* B,
                                      double beta, double* C, void* stream) {
  using namespace pcg;
  if (nterm < 1 || nterm > kMaxTerms || m_n < 0 || m_n > kMaxSub || n_n < 0 || n_n > kMaxSub ||
      !C || !k_n || !alpha || !A || !B || (m_n > 0 && !m_sa) || (n_n > 0 && !n_sb) ||
      !k_ext || !k_sa || !k_sb) {
    set_error("pcg_contract_multi_f64: bad term / sub-index counts or missing arrays");
    return -1;
  }
  MultiArgs p{};
  p.nterm = nterm;
  const long long zero[kMaxSub] = {0, 0, 0, 0};
  if (!fill_sub(p.m, m_n, m_ext, zero, m_sc, "M") || !fill_sub(p.n, n_n, n_ext, zero, n_sc, "N"))
    return -1;
  for (int t = 0; t < nterm; ++t) {
    for (int q = 0; q < kMaxSub; ++q) {
      p.ma[t][q] = (q < m_n) ? m_sa[t * kMaxSub + q] : 0;
      p.nb[t][q] = (q < n_n) ? n_sb[t * kMaxSub + q] : 0;
    }
    if (!fill_sub(p.k[t], k_n[t], k_ext + t * kMaxSub, k_sa + t * kMaxSub, k_sb + t * kMaxSub,
                  "K"))
      return -1;
    p.K[t] = sub_total(p.k[t]);
    p.alpha[t] = alpha[t];
    p.A[t] = A[t];
    p.B[t] = B[t];
    if (!A[t] || !B[t]) {
      set_error("pcg_contract_multi_f64: null operand of term %d", t);
      return -1;
    }
  }
  p.M = sub_total(p.m);
  p.N = sub_total(p.n);
  p.beta = beta;
  p.C = C;
  const long long mt = (p.M + BM - 1) / BM, nt = (p.N + BN - 1) / BN;
  if (mt > 65535) {
    set_error("pcg_contract_multi_f64: M=%lld too large", p.M);
    return -1;
  }
  dim3 grid((unsigned)nt, (unsigned)mt);
  contract_multi_f64_kernel<<<grid, NT, 0, (cudaStream_t)stream>>>(p);
  PCG_CHECK_LAUNCH("pcg_contract_multi_f64");
  return 0;
}

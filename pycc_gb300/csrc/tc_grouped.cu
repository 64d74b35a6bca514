// Grouped, segmented tcgen05 GEMM with FP32 output (the connected-triples builder).
//
// A launch computes G groups of C_g[m, n] = sum_s A_s[arow_gs + m, :] . B_s[brow_gs + n, :]
// (m < M, n < N) where each group has up to four K segments; segment s reads K-major BF16
// rows from one of four A operand matrices and one of four B operand matrices (TMA maps),
// starting at a per-group row.  All segments of a group accumulate in one TMEM tile, so
// the output (FP32, C[out_g + m*ldm + n*ldn]) is written once.  For the (T) correction a group
// is one (triple, orientation) and its segments are the four t3 terms of that orientation;
// its partial is stored column-major (ldm = 1), so that the 32 rows a warp drains from
// TMEM (one per lane) are 32 consecutive floats.
//
// Persistent and warp-specialised like tc_gemm_kernel: warp 0 TMA, warp 1 MMA, warps 2-9
// epilogue (two per TMEM lane quarter, one per column half), two TMEM accumulators; every
// mbarrier wait is bounded.
#include "tc_common.cuh"
#include <algorithm>

namespace pcg {
namespace tc {

constexpr int kMaxSeg = 4;

struct GroupDesc {
  int nseg;
  int amap[kMaxSeg], arow[kMaxSeg], bmap[kMaxSeg], brow[kMaxSeg], nkb[kMaxSeg];
  long long out;
};

struct GMaps {
  CUtensorMap a[4];
  CUtensorMap b[4];
};

constexpr int GROUPED_EPI_WARPS = 8;
constexpr int GROUPED_THREADS = 64 + 32 * GROUPED_EPI_WARPS;

struct GArgs {
  const GroupDesc* groups;
  int ngroups;
  long long M, N, ldm, ldn;
  long long mt, nt;
  float* C;
  int* status;
  unsigned long long wait_ns;  // bound on any single device-side wait
};

template <int BN>
struct GSmem {
  static constexpr int A_BYTES = BM * KBYTES;
  static constexpr int B_BYTES = BN * KBYTES;
  static constexpr int STAGE = A_BYTES + B_BYTES;
  static constexpr int TAIL = 512;
  static constexpr int FIT = (232448 - 1024 - TAIL) / STAGE;
  static constexpr int STAGES = FIT > 8 ? 8 : FIT;
  static constexpr int TOTAL = 1024 + STAGES * STAGE + TAIL;
  static constexpr unsigned TMEM_COLS = (2 * BN <= 128) ? 128 : ((2 * BN <= 256) ? 256 : 512);
};

template <int BN>
__global__ void __launch_bounds__(GROUPED_THREADS, 1)
    tc_grouped_kernel(const __grid_constant__ GMaps maps, const GArgs p) {
  using L = GSmem<BN>;
  constexpr int S = L::STAGES;
  constexpr uint32_t TMEM_COLS = L::TMEM_COLS;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint8_t* sA = base;
  uint8_t* sB = base + S * L::A_BYTES;
  uint8_t* tail = base + S * L::STAGE;
  uint64_t* full = reinterpret_cast<uint64_t*>(tail);
  uint64_t* empty = full + S;
  uint64_t* tfull = empty + S;
  uint64_t* tempty = tfull + 2;
  uint64_t* mdone = tempty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mdone + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long per = p.mt * p.nt;
  const long long nunits = per * p.ngroups;

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], GROUPED_EPI_WARPS);
    }
    mbar_init(mdone, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int it = 0;
      bool stop = false;
      for (long long u = blockIdx.x; u < nunits && !stop; u += gridDim.x) {
        const GroupDesc& g = p.groups[u / per];
        const long long r = u % per;
        const int m0 = (int)((r / p.nt) * BM), n0 = (int)((r % p.nt) * BN);
        for (int s = 0; s < g.nseg && !stop; ++s) {
          const CUtensorMap* ta = &maps.a[g.amap[s]];
          const CUtensorMap* tb = &maps.b[g.bmap[s]];
          for (int kb = 0; kb < g.nkb[s]; ++kb, ++it) {
            const int st = it % S;
            if (it >= S && !mbar_wait(&empty[st], ((it / S) - 1) & 1, p.wait_ns)) {
              atomicExch(p.status, kStatusTimeoutEmpty);
              *abort_flag = 1;
            }
            if (*abort_flag) {
              stop = true;
              break;
            }
            mbar_expect_tx(&full[st], L::STAGE);
            tma_load_2d(ta, &full[st], sA + st * L::A_BYTES, kb * 64, g.arow[s] + m0);
            tma_load_2d(tb, &full[st], sB + st * L::B_BYTES, kb * 64, g.brow[s] + n0);
          }
        }
      }
      if (stop)
        for (int j = max(0, it - S); j < it; ++j)
          mbar_wait(&full[j % S], (j / S) & 1, p.wait_ns);
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) |
                             ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
      int it = 0, ui = 0;
      bool stop = false;
      for (long long u = blockIdx.x; u < nunits && !stop; u += gridDim.x, ++ui) {
        const GroupDesc& g = p.groups[u / per];
        const int b = ui & 1;
        if (ui >= 2 && !mbar_wait(&tempty[b], ((ui >> 1) - 1) & 1, p.wait_ns)) {
          atomicExch(p.status, kStatusTimeoutEmpty);
          *abort_flag = 1;
        }
        if (*abort_flag) break;
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(b * BN);
        uint32_t acc = 0u;
        for (int s = 0; s < g.nseg && !stop; ++s) {
          for (int kb = 0; kb < g.nkb[s]; ++kb, ++it) {
            const int st = it % S;
            if (!mbar_wait(&full[st], (it / S) & 1, p.wait_ns)) {
              atomicExch(p.status, kStatusTimeoutFull);
              *abort_flag = 1;
            }
            if (*abort_flag) {
              stop = true;
              break;
            }
            tc_fence_after();
            const uint64_t da = sw128_desc(smem_u32(sA + st * L::A_BYTES));
            const uint64_t db = sw128_desc(smem_u32(sB + st * L::B_BYTES));
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              umma_f16(d, da + 2 * k, db + 2 * k, idesc, acc);
              acc = 1u;
            }
            umma_commit(&empty[st]);
          }
        }
        umma_commit(&tfull[b]);
      }
      umma_commit(mdone);
      mbar_wait(mdone, 0, p.wait_ns);
    }
    __syncwarp();
  } else {
    const int q = warp & 3;         // TMEM lane quarter
    const int h = (warp - 2) >> 2;  // column half: alternate 32-column blocks, last odd
                                    // block split 16 / 16 (loads start at their width)
    constexpr int NFULL = BN / 64;
    int ui = 0;
    for (long long u = blockIdx.x; u < nunits; u += gridDim.x, ++ui) {
      const GroupDesc& g = p.groups[u / per];
      const long long r = u % per;
      const long long m0 = (r / p.nt) * BM, n0 = (r % p.nt) * BN;
      const int b = ui & 1;
      int okw = 1;
      if (lane == 0) {
        okw = mbar_wait_sleep(&tfull[b], (ui >> 1) & 1, p.wait_ns) ? 1 : 0;
        if (!okw) {
          atomicExch(p.status, kStatusTimeoutDone);
          *abort_flag = 1;
        }
        if (*abort_flag) okw = 0;
      }
      if (!__shfl_sync(0xffffffffu, okw, 0)) break;
      tc_fence_after();
      const long long row = m0 + q * 32 + lane;
      const bool row_ok = row < p.M;
      float* crow = p.C + g.out + row * p.ldm;
      const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN);
#pragma unroll 1
      for (int fb = 0; fb < NFULL; ++fb) {
        const int c0 = 32 * (2 * fb + h);
        uint32_t v[32];
        tmem_ld32(tb + c0, v);
        if (row_ok)
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (n0 + c0 + j < p.N) crow[(n0 + c0 + j) * p.ldn] = __uint_as_float(v[j]);
      }
      if constexpr (BN % 64 != 0) {
        const int c0 = BN - 32 + 16 * h;
        uint32_t v[16];
        tmem_ld16(tb + c0, v);
        if (row_ok)
#pragma unroll
          for (int j = 0; j < 16; ++j)
            if (n0 + c0 + j < p.N) crow[(n0 + c0 + j) * p.ldn] = __uint_as_float(v[j]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[b]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS));
  }
}

template <int BN>
int glaunch(const GMaps& maps, GArgs a, cudaStream_t st) {
  static bool attr = false;
  const int smem = GSmem<BN>::TOTAL;
  if (!attr) {
    cudaFuncSetAttribute(tc_grouped_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  a.nt = (a.N + BN - 1) / BN;
  const long long units = a.mt * a.nt * a.ngroups;
  const long long grid = std::min<long long>(units, num_sms());
  tc_grouped_kernel<BN><<<(unsigned)grid, GROUPED_THREADS, smem, st>>>(maps, a);
  PCG_CHECK_LAUNCH("pcg_tc_grouped_gemm");
  return 0;
}

}  // namespace tc
}  // namespace pcg

using namespace pcg;
using namespace pcg::tc;

// Grouped segmented BF16 GEMM, FP32 output (see the top of this file).  a_ptr / b_ptr: up
// to four BF16 operand matrices each ([a_rows[q]][a_ld[q]] K-major, 16-byte aligned rows,
// K a multiple of 64); groups: device array of ngroups GroupDesc records (nseg, amap[4],
// arow[4], bmap[4], brow[4], nkb[4], out) as laid out in this file; element (m, n) of group
// g goes to C[out_g + m*ldm + n*ldn].
extern "C" int pcg_tc_grouped_gemm(int na, const void* const* a_ptr, const long long* a_rows,
                                   const long long* a_ld, int nb, const void* const* b_ptr,
                                   const long long* b_rows, const long long* b_ld,
                                   const void* groups, int ngroups, long long M, long long N,
                                   float* C, long long ldm, long long ldn, int* status,
                                   void* stream) {
  if (na < 1 || na > 4 || nb < 1 || nb > 4 || !groups || ngroups < 1 || M < 1 || N < 1 || !C ||
      !status || ldm < 1 || ldn < 1 || M > 0x7fffffffLL || N > 0x7fffffffLL || !a_ptr ||
      !a_rows || !a_ld || !b_ptr || !b_rows || !b_ld) {
    set_error("pcg_tc_grouped_gemm: bad arguments");
    return -1;
  }
  GMaps maps;
  for (int q = 0; q < 4; ++q) {
    const int qa = q < na ? q : 0, qb = q < nb ? q : 0;
    if (!a_ptr[qa] || !b_ptr[qb] || (a_ld[qa] * 2) % 16 || (b_ld[qb] * 2) % 16) {
      set_error("pcg_tc_grouped_gemm: operand %d not 16-byte aligned", q);
      return -1;
    }
    if (!make_map(&maps.a[q], a_ptr[qa], a_rows[qa], a_ld[qa] * 2, a_ld[qa] * 2, 2, BM)) return -1;
  }
  const int BN = (N <= 64) ? 64 : (N <= 128 ? 128 : (N <= 160 ? 160 : 256));
  for (int q = 0; q < 4; ++q) {
    const int qb = q < nb ? q : 0;
    if (!make_map(&maps.b[q], b_ptr[qb], b_rows[qb], b_ld[qb] * 2, b_ld[qb] * 2, 2, BN)) return -1;
  }
  GArgs a{};
  a.groups = reinterpret_cast<const GroupDesc*>(groups);
  a.ngroups = ngroups;
  a.M = M;
  a.N = N;
  a.ldm = ldm;
  a.ldn = ldn;
  a.mt = (M + BM - 1) / BM;
  a.C = C;
  a.status = status;
  a.wait_ns = wait_limit_ns();
  cudaStream_t st = (cudaStream_t)stream;
  switch (BN) {
    case 64: return glaunch<64>(maps, a, st);
    case 128: return glaunch<128>(maps, a, st);
    case 160: return glaunch<160>(maps, a, st);
    default: return glaunch<256>(maps, a, st);
  }
}

// Size of one GroupDesc record in bytes (for hosts that build the table).
extern "C" int pcg_tc_group_desc_size(void) { return (int)sizeof(GroupDesc); }

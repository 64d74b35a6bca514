// Tensor-core contraction engine of the mixed-precision CCSD path (sm_103a, tcgen05).
//
//   C[m, n] = beta * C[m, n] + alpha * sum_k A[m, k] * B[n, k]        (C in FP64)
//
// * Operands are K-major row matrices in HBM ([rows][ld], K contiguous, ld a multiple of
//   the K block), produced by the pack kernel below from any strided FP64 source
//   (index permutations, the tau / 2t2-t2' combinations and the t1 outer products are
//   folded into the gather, together with the precision conversion).
// * Formats: BF16; split-BF16x3 (A = Ah + Al, B = Bh + Bl, three passes Ah.Bh + Ah.Bl +
//   Al.Bh accumulated in the same TMEM tile), fused (all three products from one stage)
//   and fused with separate accumulators for the small and the leading products;
//   split-BF16x6; FP8 E4M3 with one FP32 scale per row of each operand (applied in the
//   epilogue).
// * Mainloop: one CTA computes a 128 x BN FP32 tile in TMEM.  Warp 0 lane 0 issues TMA
//   (cp.async.bulk.tensor, 128B swizzle) into an S-stage shared-memory ring; warp 1
//   lane 0 issues tcgen05.mma (kind::f16 or kind::f8f6f4) and releases stages with
//   tcgen05.commit; eight epilogue warps (two per TMEM lane quarter, one per column half)
//   drain TMEM (tcgen05.ld 32x32b) and write FP64 with the output permutation folded into
//   per-row / per-column offsets.
// * Every mbarrier wait is bounded (globaltimer); on expiry the CTA records a status code
//   in a caller-provided device word, stops issuing work and releases its TMEM.
#include "tc_common.cuh"
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <algorithm>
#include <cmath>

namespace pcg {
namespace tc {

enum Fmt : int { kBF16 = 0, kBF16x3 = 1, kFP8 = 2, kBF16x6 = 3, kBF16x3F = 4, kBF16x3S = 5 };

// Operand pieces multiplied in each pass (A piece, B piece), smallest products first so
// the FP32 accumulator sums the small corrections before the leading term.
//   BF16x3: v = hi + lo;        Ah.Bh + Ah.Bl + Al.Bh
//   BF16x6: v = hi + mid + lo;  the six products of order <= 2^-16
constexpr int kMaxPass = 6;
struct PassTable {
  int n;
  unsigned char a[kMaxPass], b[kMaxPass];
};

struct Maps {
  CUtensorMap a[3];
  CUtensorMap b[3];
};

struct EpiIdx {
  int n;
  long long ext[kMaxSub];
  long long s[kMaxSub];
};

struct Args {
  long long M, N;
  long long mt, nt;  // output tiles along M and N
  int gm;            // M tiles per raster group (see decode_tile)
  int bs;            // columns per N tile: BN or less, a multiple of 16 (see pcg_tc_gemm)
  int stage_bytes;   // bytes TMA delivers per ring stage: the A tile and bs rows of B
  int splits;        // K splits across CTAs (FP64 atomics in the epilogue when > 1)
  int kb_per_split;  // K blocks of one split
  int nkb_total;     // K blocks of the whole K range
  int kb_chunk;      // K blocks accumulated in TMEM before the FP64 flush
  int npass;         // 1, 3 (split-BF16x3) or 6 (split-BF16x6)
  PassTable pt;
  int fp8;
  EpiIdx em, en;
  double alpha, beta;
  double* C;
  const float* a_scale;
  const float* b_scale;
  unsigned long long wait_ns;  // bound on any single device-side wait
  const long long* col_map;   // optional per-column C offsets (replaces en)
  const double* col_scale;    // optional per-column multipliers
  int atomic_out;
  int red_out;  // one FP64 flush per tile (short K): add into C by reductions when beta is 1
  int* status;
};

// Offset of output row (or column) r: r and the extents are below 2^31 (the host checks
// M, N against the TMA coordinate range), so the decomposition runs in 32-bit integer
// arithmetic instead of the much longer 64-bit division sequence.
__device__ __forceinline__ long long epi_offset(const EpiIdx& d, long long r) {
  long long o = 0;
  unsigned x = (unsigned)r;
  for (int q = d.n - 1; q >= 0; --q) {
    const unsigned e = (unsigned)d.ext[q];
    o += (long long)(x % e) * d.s[q];
    x /= e;
  }
  return o;
}

constexpr int kSmemMax = 232448;  // 227 KB of dynamic shared memory per CTA

// Warp roles: warp 0 issues TMA, warp 1 issues tcgen05.mma, warps 2..9 drain TMEM.  Two
// epilogue warps share each TMEM lane quarter (warp w reads lanes 32 (w % 4) ..), one per
// half of the tile's columns: with one warp per scheduler the FP64 read-modify-write of a
// short-K GEMM is bound by instruction latency, two overlap it.
constexpr int GEMM_EPI_WARPS = 8;
constexpr int GEMM_THREADS = 64 + 32 * GEMM_EPI_WARPS;

// NP operand pieces per stage: 1 (one product per stage; split formats run one pass per
// product), or 2 (split-BF16x3 with both pieces of A and B in the stage, all three products
// issued from it: a third less shared-memory fill traffic per flop).
// SPLIT (fused split-BF16x3 only): the two small products Al.Bh + Ah.Bl accumulate in a
// TMEM accumulator of their own, the leading Ah.Bh in another, and the epilogue adds them
// once.  The small corrections then never meet the leading term's magnitude inside the
// truncating FP32 accumulator (the by-pass format's accuracy, at the fused format's
// traffic).  The small products are about 2^-8 of the leading one, so their accumulator
// runs over the tile's whole K range without the chunked FP64 flushes the leading product
// needs: one BN-column region for them next to the two BN-column leading buffers, which
// limits BN to 160 (480 of the 512 TMEM columns).
template <int BN, int NP = 1, bool SPLIT = false>
struct Smem {
  static constexpr int A_BYTES = BM * KBYTES;
  static constexpr int B_BYTES = BN * KBYTES;
  static constexpr int STAGE = NP * (A_BYTES + B_BYTES);
  // barriers / tmem slot / flags, then per epilogue warp BN/2 column offsets and scales
  static constexpr int TAIL = 512 + GEMM_EPI_WARPS * (BN / 2) * 8;
  static constexpr int FIT = (kSmemMax - 1024 - TAIL) / STAGE;
  static constexpr int STAGES = FIT > 8 ? 8 : FIT;
  static constexpr int TOTAL = 1024 /*align*/ + STAGES * STAGE + TAIL;
  static constexpr int ACC = BN;                        // TMEM columns of one buffer
  static constexpr int SMALL = 2 * BN;                  // SPLIT: small-product region
  static constexpr int USED = SPLIT ? 3 * BN : 2 * BN;
  static constexpr unsigned TMEM_COLS = (USED <= 128) ? 128 : ((USED <= 256) ? 256 : 512);
  static_assert(BN % 32 == 0 && BN >= 64 && BN <= 256, "BN: multiple of 32 in [64, 256]");
  static_assert(USED <= 512 && (!SPLIT || NP == 2), "TMEM holds 512 columns");
  static_assert(STAGES >= 2, "shared-memory ring too shallow");
};

// Tile t -> (split, m tile, n tile).  Tiles are walked in groups of gm M tiles: within a
// group the M tile runs fastest, then the N tile, so the CTAs of one wave (consecutive t)
// cover about gm M tiles x (wave / gm) N tiles and share both operands' row blocks in L2.
// gm = 1 is the N-fastest order.  The host picks gm per launch.
__device__ __forceinline__ void decode_tile(const Args& p, long long t, int& split, long long& m0,
                                            long long& n0) {
  const long long per = p.mt * p.nt;
  split = (int)(t / per);
  const long long r = t % per;
  const long long group = r / ((long long)p.gm * p.nt);
  const long long rg = r % ((long long)p.gm * p.nt);
  const long long gm_here = min((long long)p.gm, p.mt - group * p.gm);
  m0 = (group * p.gm + rg % gm_here) * BM;
  n0 = rg / gm_here;
}

// One batch of W (16 or 32) accumulator columns of this thread's output row: every old C
// value of the batch is loaded before any store (W independent requests in flight per
// thread).  Scales are
// FP32 (powers of two and the terms' small factors) and the widening is integer
// arithmetic, so the only FP64 instruction per element is the accumulate into C.
// Tile column of the jj-th column drained by the epilogue warp of column half h: 32-column
// blocks alternate between the two halves and an odd last block is split 16 / 16, so every
// tcgen05.ld starts at a multiple of its own width (32 or 16 columns).
template <int BN>
__device__ __forceinline__ int epi_col(int h, int jj) {
  constexpr int NB = BN / 32, NFULL = NB / 2;
  if (jj < 32 * NFULL) return 32 * (2 * (jj >> 5) + h) + (jj & 31);
  return 32 * (NB - 1) + 16 * h + (jj - 32 * NFULL);
}

// Column offsets are 32-bit (the host checks that every column offset of C is below 2^31;
// the row offset stays 64-bit), so a batch's offsets stay in registers next to its
// accumulator values and old C values.
template <int W>
__device__ __forceinline__ void epi_batch(uint32_t taddr, const int* co, const float* sc,
                                          bool row_ok, double* crow, float ascale,
                                          double cscale, bool need_old, int atomic_out) {
  uint32_t r[W];
  if constexpr (W == 32) tmem_ld32(taddr, r);
  else tmem_ld16(taddr, r);
  if (!row_ok) return;
  int cj[W];
  double old[W];
#pragma unroll
  for (int j = 0; j < W; ++j) {
    cj[j] = co[j];
    old[j] = (need_old && cj[j] >= 0) ? crow[cj[j]] : 0.0;
  }
#pragma unroll
  for (int j = 0; j < W; ++j) {
    const int c = cj[j];
    if (c < 0) continue;
    const double v = f32_to_f64(__uint_as_float(r[j]) * (ascale * sc[j]));
    if (atomic_out)
      atomicAdd(crow + c, v);
    else if (cscale == 1.0)
      crow[c] = old[j] + v;
    else
      crow[c] = fma(cscale, old[j], v);
  }
}

// Split accumulators, last chunk of a tile: the leading chunk sum + the tile's small-product
// sum (one FP32 rounding) written back over the leading buffer, so that the small
// accumulator is free for the next tile's MMAs before this chunk's FP64 epilogue runs.
template <int W>
__device__ __forceinline__ void tmem_fold(uint32_t lead, uint32_t small) {
  uint32_t r[W], s[W];
  if constexpr (W == 32) {
    tmem_ld32(lead, r);
    tmem_ld32(small, s);
  } else {
    tmem_ld16(lead, r);
    tmem_ld16(small, s);
  }
#pragma unroll
  for (int j = 0; j < W; ++j) r[j] = __float_as_uint(__uint_as_float(r[j]) + __uint_as_float(s[j]));
  if constexpr (W == 32) tmem_st32(lead, r);
  else tmem_st16(lead, r);
}

// Persistent, warp-specialised tcgen05 GEMM.  Each CTA walks the tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ...; each tile's K range is cut into chunks of kb_chunk K blocks
// (all passes of a chunk accumulate into one TMEM buffer), and the epilogue warps add each
// chunk's FP32 sum into the FP64 output while the MMA warp fills the other TMEM buffer.
// Bounding the FP32 accumulation chain keeps the tensor-core accumulator's rounding
// (truncating, so biased for long sums) at the level of a short dot product.
template <int BN, int NP, bool SPLIT = false>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ Maps maps, const Args p) {
  using L = Smem<BN, NP, SPLIT>;
  constexpr int S = L::STAGES;
  constexpr uint32_t TMEM_COLS = L::TMEM_COLS;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint8_t* sA = base;                            // [stage][piece] A tiles
  uint8_t* sB = base + S * NP * L::A_BYTES;      // [stage][piece] B tiles
  uint8_t* tail = base + S * L::STAGE;
  uint64_t* full = reinterpret_cast<uint64_t*>(tail);
  uint64_t* empty = full + S;
  uint64_t* tfull = empty + S;   // [2] accumulator ready (MMA -> epilogue)
  uint64_t* tempty = tfull + 2;  // [2] accumulator drained (epilogue -> MMA)
  uint64_t* sempty = tempty + 2; // SPLIT: small-product region drained (epilogue -> MMA)
  uint64_t* mdone = sempty + 1;  // all MMAs of this CTA retired
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mdone + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  constexpr int HB = BN / 2;  // columns drained by one epilogue warp
  int* colofs_all = reinterpret_cast<int*>(tail + 512);  // [8 warps][HB]
  float* colsc_all = reinterpret_cast<float*>(tail + 512 + GEMM_EPI_WARPS * HB * 4);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long ntiles = p.mt * p.nt * p.splits;
  const int kelem = p.fp8 ? 128 : 64;

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], GEMM_EPI_WARPS);
    }
    mbar_init(sempty, GEMM_EPI_WARPS);
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
      // ---- TMA producer ----
      int it = 0;
      bool stop = false;
      for (long long t = blockIdx.x; t < ntiles && !stop; t += gridDim.x) {
        int split;
        long long m0, nti;
        decode_tile(p, t, split, m0, nti);
        const int n0 = (int)(nti * p.bs);
        const int kb0 = split * p.kb_per_split;
        const int kb1 = min(p.nkb_total, kb0 + p.kb_per_split);
        for (int c0 = kb0; c0 < kb1 && !stop; c0 += p.kb_chunk) {
          const int c1 = min(c0 + p.kb_chunk, kb1);
          const int npass = (NP == 1) ? p.npass : 1;
          for (int pass = 0; pass < npass && !stop; ++pass) {
            for (int kb = c0; kb < c1; ++kb, ++it) {
              const int s = it % S;
              if (it >= S && !mbar_wait(&empty[s], ((it / S) - 1) & 1, p.wait_ns)) {
                atomicExch(p.status, kStatusTimeoutEmpty);
                *abort_flag = 1;
              }
              if (*abort_flag) {
                stop = true;
                break;
              }
              mbar_expect_tx(&full[s], (uint32_t)p.stage_bytes);
#pragma unroll
              for (int q = 0; q < NP; ++q) {
                const CUtensorMap* ta = &maps.a[NP == 1 ? p.pt.a[pass] : q];
                const CUtensorMap* tb = &maps.b[NP == 1 ? p.pt.b[pass] : q];
                tma_load_2d(ta, &full[s], sA + (s * NP + q) * L::A_BYTES, kb * kelem, (int)m0);
                tma_load_2d(tb, &full[s], sB + (s * NP + q) * L::B_BYTES, kb * kelem, n0);
              }
            }
          }
        }
      }
      if (stop) {
        // let the copies already in flight land before the CTA releases its shared memory
        for (int j = max(0, it - S); j < it; ++j)
          mbar_wait(&full[j % S], (j / S) & 1, p.wait_ns);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      uint32_t idesc = (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
      if (!p.fp8) idesc |= (1u << 7) | (1u << 10);  // A, B = BF16 (FP8 E4M3 encodes as 0)
      int it = 0, u = 0, tl = 0;
      bool stop = false;
      const uint32_t tsmall = tmem + (uint32_t)L::SMALL;
      for (long long t = blockIdx.x; t < ntiles && !stop; t += gridDim.x, ++tl) {
        int split;
        long long m0, nti;
        decode_tile(p, t, split, m0, nti);
        const int kb0 = split * p.kb_per_split;
        const int kb1 = min(p.nkb_total, kb0 + p.kb_per_split);
        uint32_t acc_small = 0u;
        if (SPLIT && tl >= 1) {  // the previous tile's small-product sum has been read
          if (!mbar_wait(&sempty[0], (tl - 1) & 1, p.wait_ns)) {
            atomicExch(p.status, kStatusTimeoutEmpty);
            *abort_flag = 1;
          }
          if (*abort_flag) {
            stop = true;
            break;
          }
          tc_fence_after();
        }
        // a tile multiplies its bs columns; the last N tile of a ragged N only its present
        // columns (rounded up to the MMA's multiple of 16).  Accumulator columns beyond are
        // never stored.
        const long long nleft = p.N - nti * p.bs;
        const uint32_t nmma =
            nleft >= p.bs ? (uint32_t)p.bs : (uint32_t)((nleft + 15) & ~15LL);
        const uint32_t idesc_t = (idesc & ~(0x3Fu << 17)) | ((nmma >> 3) << 17);
        for (int c0 = kb0; c0 < kb1 && !stop; c0 += p.kb_chunk, ++u) {
          const int c1 = min(c0 + p.kb_chunk, kb1);
          const int b = u & 1;
          if (u >= 2 && !mbar_wait(&tempty[b], ((u >> 1) - 1) & 1, p.wait_ns)) {
            atomicExch(p.status, kStatusTimeoutEmpty);
            *abort_flag = 1;
          }
          if (*abort_flag) {
            stop = true;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + (uint32_t)(b * L::ACC);
          uint32_t acc = 0u;
          const int npass = (NP == 1) ? p.npass : 1;
          for (int pass = 0; pass < npass && !stop; ++pass) {
            for (int kb = c0; kb < c1; ++kb, ++it) {
              const int s = it % S;
              if (!mbar_wait(&full[s], (it / S) & 1, p.wait_ns)) {
                atomicExch(p.status, kStatusTimeoutFull);
                *abort_flag = 1;
              }
              if (*abort_flag) {
                stop = true;
                break;
              }
              tc_fence_after();
              if constexpr (NP == 1) {
                const uint64_t da = sw128_desc(smem_u32(sA + s * L::A_BYTES));
                const uint64_t db = sw128_desc(smem_u32(sB + s * L::B_BYTES));
#pragma unroll
                for (int k = 0; k < 4; ++k) {  // 4 x 32 bytes of K per 128-byte stage row
                  if (p.fp8)
                    umma_f8(d, da + 2 * k, db + 2 * k, idesc_t, acc);
                  else
                    umma_f16(d, da + 2 * k, db + 2 * k, idesc_t, acc);
                  acc = 1u;
                }
              } else {
                // split-BF16x3 from one stage: Al.Bh, Ah.Bl, then Ah.Bh
                const uint64_t dah = sw128_desc(smem_u32(sA + (s * NP + 0) * L::A_BYTES));
                const uint64_t dal = sw128_desc(smem_u32(sA + (s * NP + 1) * L::A_BYTES));
                const uint64_t dbh = sw128_desc(smem_u32(sB + (s * NP + 0) * L::B_BYTES));
                const uint64_t dbl = sw128_desc(smem_u32(sB + (s * NP + 1) * L::B_BYTES));
                const uint64_t prs[3][2] = {{dal, dbh}, {dah, dbl}, {dah, dbh}};
#pragma unroll
                for (int pr = 0; pr < 3; ++pr)
#pragma unroll
                  for (int k = 0; k < 4; ++k) {
                    if (SPLIT && pr < 2) {  // small products: the tile's own accumulator
                      umma_f16(tsmall, prs[pr][0] + 2 * k, prs[pr][1] + 2 * k, idesc_t,
                               acc_small);
                      acc_small = 1u;
                    } else {
                      umma_f16(d, prs[pr][0] + 2 * k, prs[pr][1] + 2 * k, idesc_t, acc);
                      acc = 1u;
                    }
                  }
              }
              umma_commit(&empty[s]);
            }
          }
          umma_commit(&tfull[b]);
        }
      }
      umma_commit(mdone);
      mbar_wait(mdone, 0, p.wait_ns);  // every MMA of this CTA retired before TMEM is released
    }
    __syncwarp();
  } else {
    // ---- epilogue warps: TMEM -> registers -> FP64 C, one chunk at a time ----
    const int q = warp & 3;         // the TMEM lane quarter this warp may read
    const int h = (warp - 2) >> 2;  // the half of the tile's columns it drains
    int* colofs = colofs_all + (warp - 2) * HB;
    float* colsc = colsc_all + (warp - 2) * HB;
    int u = 0;
    bool stop = false;
    for (long long t = blockIdx.x; t < ntiles && !stop; t += gridDim.x) {
      int split;
      long long m0, nti;
      decode_tile(p, t, split, m0, nti);
      const long long n0 = nti * p.bs;
      const int kb0 = split * p.kb_per_split;
      const int kb1 = min(p.nkb_total, kb0 + p.kb_per_split);
      const long long row = m0 + q * 32 + lane;
      const bool row_ok = row < p.M;
      const long long roff = row_ok ? epi_offset(p.em, row) : 0;
      const float ascale = (p.fp8 && row_ok) ? p.a_scale[row] : 1.0f;
      __syncwarp();  // the previous tile's column offsets are no longer read
      for (int j = lane; j < HB; j += 32) {
        const int cj = epi_col<BN>(h, j);
        const long long c = n0 + cj;
        const bool in = cj < p.bs && c < p.N;
        colofs[j] = in ? (int)(p.col_map ? p.col_map[c] : epi_offset(p.en, c)) : -1;
        double sc = p.alpha;
        if (in && p.fp8) sc *= (double)p.b_scale[c];
        if (in && p.col_scale) sc *= p.col_scale[c];
        colsc[j] = (float)sc;
      }
      __syncwarp();
      bool first = true;
      for (int c0 = kb0; c0 < kb1; c0 += p.kb_chunk, ++u) {
        const int b = u & 1;
        // one lane polls (with back-off), the warp follows
        int okw = 1;
        if (lane == 0) {
          okw = mbar_wait_sleep(&tfull[b], (u >> 1) & 1, p.wait_ns) ? 1 : 0;
          if (!okw) {
            atomicExch(p.status, kStatusTimeoutDone);
            *abort_flag = 1;
          }
          if (*abort_flag) okw = 0;
        }
        // warp-uniform decision: tcgen05.ld below is a .sync.aligned warp instruction
        if (!__shfl_sync(0xffffffffu, okw, 0)) {
          stop = true;
          break;
        }
        tc_fence_after();
        const double cscale = first ? p.beta : 1.0;  // beta applies once per tile
        // adds into C as fire-and-forget reductions (split K, or one flush per tile with C's
        // scale 1: the warp then waits on no load of the old C values)
        const int red = p.atomic_out || (p.red_out && cscale == 1.0);
        const bool need_old = !red && cscale != 0.0;
        double* crow = p.C + roff;
        const uint32_t lanes = (uint32_t)(q * 32) << 16;
        const uint32_t tbase = tmem + lanes + (uint32_t)(b * L::ACC);
        constexpr int NFULL = BN / 64;  // whole 32-column blocks per warp
        if constexpr (SPLIT) {
          if (c0 + p.kb_chunk >= kb1) {  // the tile's last chunk: fold in the small products
            const uint32_t sbase = tmem + lanes + (uint32_t)L::SMALL;
#pragma unroll 1
            for (int fb = 0; fb < NFULL; ++fb)
              tmem_fold<32>(tbase + 32 * (2 * fb + h), sbase + 32 * (2 * fb + h));
            if constexpr (BN % 64 != 0)
              tmem_fold<16>(tbase + (BN - 32) + 16 * h, sbase + (BN - 32) + 16 * h);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&sempty[0]);
          }
        }
#pragma unroll 1
        for (int fb = 0; fb < NFULL; ++fb)
          epi_batch<32>(tbase + 32 * (2 * fb + h), colofs + 32 * fb, colsc + 32 * fb, row_ok,
                        crow, ascale, cscale, need_old, red);
        if constexpr (BN % 64 != 0)  // BN = 96, 160, 224: the last block split 16 / 16
          epi_batch<16>(tbase + (BN - 32) + 16 * h, colofs + 32 * NFULL, colsc + 32 * NFULL,
                        row_ok, crow, ascale, cscale, need_old, red);
        first = false;
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[b]);
      }
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

// ---------------------------------------------------------------------------------------
// Pack: dst[r][k] = w(k) * convert(a*X + b*Y + c*P*Q + d*R*S) at per-source offsets
// rowoff_s(r) + koff_s(k).
// ---------------------------------------------------------------------------------------
constexpr int kPackSrc = 6;  // sources X, Y, P, Q, R, S
struct PackIdx {
  int n;
  long long ext[kMaxSub];
  long long s[kPackSrc][kMaxSub];  // strides of each source
};

// Offsets of flat row (or K) index r in the six sources; r and the extents are below 2^31
// (checked by the host), so the decomposition is 32-bit integer arithmetic.
__device__ __forceinline__ void pack_offsets(const PackIdx& d, long long r,
                                             long long (&o)[kPackSrc]) {
#pragma unroll
  for (int s = 0; s < kPackSrc; ++s) o[s] = 0;
  unsigned rr = (unsigned)r;
  for (int q = d.n - 1; q >= 0; --q) {
    const unsigned e = (unsigned)d.ext[q];
    const long long x = rr % e;
    rr /= e;
#pragma unroll
    for (int s = 0; s < kPackSrc; ++s) o[s] += x * d.s[s][q];
  }
}

struct PackArgs {
  PackIdx r, k;
  long long R, K, Kp;
  double a, b, c, d;
  const double* X;
  const double* Y;
  const double* P;
  const double* Q;
  const double* R2;
  const double* S2;
  void* hi;
  void* lo;
  void* mid;
  float* scale;
  const long long* row_tab;  // optional [6][R] per-source row offsets (replaces r)
  const long long* k_tab;    // optional [6][K] per-source K offsets (replaces k)
  const float* k_w;          // optional [K] multipliers of the K entries
  int fmt;
  // rows walked in an order other than the output's (see pcg_pack_operand): output row of
  // the walked row index = sum over its sub-indices x_q * out_str[q]
  int out_perm;
  long long out_str[kMaxSub];
};

// Tiled pack: a block handles TR rows x TK columns of K.  Row and column offsets of the
// six sources are decomposed (or read from the tables) once per tile into shared memory;
// values are gathered along whichever index is unit-stride in X (kfast) and written out
// along K, so both the FP64 reads and the packed writes are coalesced.  The value type V is
// double for BF16x6 (three pieces carry 24 bits) and float otherwise: FP64 inputs are
// rounded to FP32 in integer arithmetic (f64_to_f32) and combined and split in FP32, which
// keeps the kernel a stream instead of a loop on GB300's FP64 pipe.  A BF16 hi/lo pair
// holds 16 bits, so the FP32 rounding (2^-24 of the operands) is far below the split's own
// error.  The K multipliers are powers of two in practice (exact in FP32).
constexpr int TR = 64, TK = 64, PACK_THREADS = 256;
static_assert((TR * TK) % PACK_THREADS == 0, "pack tile: whole elements per thread");

template <typename V>
struct PackTile {
  long long orow[TR];  // output row of each tile row (the tile row itself unless permuted)
  long long rof[kPackSrc][TR];
  long long kof[kPackSrc][TK];
  V kw[TK];
  V v[TR][TK + 1];
};

template <typename V>
__device__ __forceinline__ V pack_ld(const double* q) {
  if constexpr (sizeof(V) == sizeof(double)) return *q;
  else return f64_to_f32(*q);
}

// PROD: the operand may have the product sources P*Q / R*S (compiled out otherwise, which
// keeps the plain gathers within the register budget of eight resident blocks per SM)
template <typename V, bool KF, bool PROD = true>
__device__ __forceinline__ void pack_tile_load(const PackArgs& p, PackTile<V>& t, long long r0,
                                               long long k0) {
  const int tid = threadIdx.x;
  if (tid < TR) {
    long long o[kPackSrc] = {0, 0, 0, 0, 0, 0};
    long long orow = r0 + tid;
    if (r0 + tid < p.R) {
      if (p.row_tab) {
        for (int s = 0; s < kPackSrc; ++s) o[s] = p.row_tab[s * p.R + r0 + tid];
      } else {
        pack_offsets(p.r, r0 + tid, o);
        if (p.out_perm) {
          orow = 0;
          unsigned rr = (unsigned)(r0 + tid);
          for (int q = p.r.n - 1; q >= 0; --q) {
            const unsigned e = (unsigned)p.r.ext[q];
            orow += (long long)(rr % e) * p.out_str[q];
            rr /= e;
          }
        }
      }
    }
    t.orow[tid] = orow;
    for (int s = 0; s < kPackSrc; ++s) t.rof[s][tid] = o[s];
  } else if (tid >= TR && tid < TR + TK) {
    const int j = tid - TR;
    long long o[kPackSrc] = {0, 0, 0, 0, 0, 0};
    V w = (V)1;
    if (k0 + j < p.K) {
      if (p.k_tab)
        for (int s = 0; s < kPackSrc; ++s) o[s] = p.k_tab[s * p.K + k0 + j];
      else
        pack_offsets(p.k, k0 + j, o);
      if (p.k_w) w = (V)p.k_w[k0 + j];
    }
    for (int s = 0; s < kPackSrc; ++s) t.kof[s][j] = o[s];
    t.kw[j] = w;
  }
  __syncthreads();
  const V a = (V)p.a, b = (V)p.b, c = (V)p.c, d = (V)p.d;
  // Each thread keeps one index of the unit-stride side fixed (a K column when KF, a row
  // otherwise), so consecutive threads read consecutive addresses, and walks the other
  // side; the fixed side's offsets and bound are read once.  All of a thread's gathers
  // are issued before its first shared-memory store.
  constexpr int NF = KF ? TK : TR;
  constexpr int STEP = PACK_THREADS / NF;
  constexpr int PER = (KF ? TR : TK) / STEP;
  const int fx = tid % NF, w0 = tid / NF;
  const bool fx_ok = KF ? (k0 + fx < p.K) : (r0 + fx < p.R);
  const long long wlim = KF ? (p.R - r0) : (p.K - k0);
  long long f[kPackSrc] = {0, 0, 0, 0, 0, 0};
  if (p.X) f[0] = KF ? t.kof[0][fx] : t.rof[0][fx];
  if (p.Y) f[1] = KF ? t.kof[1][fx] : t.rof[1][fx];
  // phase 1: the sources read from DRAM (X, Y), all gathers of the thread in flight
  V vals[PER];
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int wv = w0 + u * STEP;
    V v = 0;
    if (fx_ok && wv < wlim) {
      // each source's walked offset is read inside its (block-uniform) branch, so an
      // operand with X alone reads one offset per element
      auto wof = [&](int src) { return KF ? t.rof[src][wv] : t.kof[src][wv]; };
      if (p.X) v = a * pack_ld<V>(p.X + f[0] + wof(0));
      if (p.Y) v += b * pack_ld<V>(p.Y + f[1] + wof(1));
      if (p.k_w) v *= KF ? t.kw[fx] : t.kw[wv];
    }
    vals[u] = v;
  }
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int wv = w0 + u * STEP;
    if (KF)
      t.v[wv][fx] = vals[u];
    else
      t.v[fx][wv] = vals[u];
  }
  // phase 2: the product sources P*Q and R*S (t1-sized factors, cache-resident), added to
  // the thread's own tile entries; separate from phase 1 so that its gathers from DRAM are
  // not held back by the registers of these.  The K multipliers are powers of two, so
  // applying them to each part gives the same value as to the sum.
  if constexpr (PROD) {
    if (p.P || p.R2) {
      if (p.P) {
        f[2] = KF ? t.kof[2][fx] : t.rof[2][fx];
        f[3] = KF ? t.kof[3][fx] : t.rof[3][fx];
      }
      if (p.R2) {
        f[4] = KF ? t.kof[4][fx] : t.rof[4][fx];
        f[5] = KF ? t.kof[5][fx] : t.rof[5][fx];
      }
#pragma unroll 4
      for (int u = 0; u < PER; ++u) {
        const int wv = w0 + u * STEP;
        if (fx_ok && wv < wlim) {
          auto wof = [&](int src) { return KF ? t.rof[src][wv] : t.kof[src][wv]; };
          V v = 0;
          if (p.P) v = c * pack_ld<V>(p.P + f[2] + wof(2)) * pack_ld<V>(p.Q + f[3] + wof(3));
          if (p.R2) v += d * pack_ld<V>(p.R2 + f[4] + wof(4)) * pack_ld<V>(p.S2 + f[5] + wof(5));
          if (p.k_w) v *= KF ? t.kw[fx] : t.kw[wv];
          if (KF)
            t.v[wv][fx] += v;
          else
            t.v[fx][wv] += v;
        }
      }
    }
  }
  __syncthreads();
}

// BF16 / split-BF16x3 from an FP32 tile: two adjacent K entries per thread, written as one
// bf16x2 word (K offsets are even: Kp and k0 are multiples of 64).
// Eight resident blocks per SM (32 registers), since the pack waits on memory latency and
// the extra blocks hide more of it.  The product sources are added in a second phase of the
// tile load (PROD), which keeps that variant within the same register budget; the plain
// variant compiles the phase out.
template <bool KF, bool PROD>
__global__ void __launch_bounds__(PACK_THREADS, 8) pack_bf16_kernel(const PackArgs p) {
  __shared__ PackTile<float> t;
  const long long r0 = (long long)blockIdx.x * TR, k0 = (long long)blockIdx.y * TK;
  pack_tile_load<float, KF, PROD>(p, t, r0, k0);
  __nv_bfloat162* hi = reinterpret_cast<__nv_bfloat162*>(p.hi);
  __nv_bfloat162* lo = reinterpret_cast<__nv_bfloat162*>(p.lo);
  static_assert(TK == 64, "a warp writes one 64-entry row of the tile");
  const int kk = 2 * (threadIdx.x & 31);
#pragma unroll 4
  for (int rr = threadIdx.x >> 5; rr < TR; rr += PACK_THREADS / 32) {
    if (r0 + rr >= p.R) break;
    const long long at = (t.orow[rr] * p.Kp + k0 + kk) >> 1;
    const float v0 = t.v[rr][kk], v1 = t.v[rr][kk + 1];
    const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
    hi[at] = h;
    if (lo) lo[at] = __floats2bfloat162_rn(v0 - __low2float(h), v1 - __high2float(h));
  }
}

// Split-BF16x6 (hi, mid, lo) from an FP64 tile.
template <bool KF>
__global__ void __launch_bounds__(PACK_THREADS) pack_bf16x6_kernel(const PackArgs p) {
  __shared__ PackTile<double> t;
  const long long r0 = (long long)blockIdx.x * TR, k0 = (long long)blockIdx.y * TK;
  pack_tile_load<double, KF>(p, t, r0, k0);
  __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(p.hi);
  __nv_bfloat16* mid = reinterpret_cast<__nv_bfloat16*>(p.mid);
  __nv_bfloat16* lo = reinterpret_cast<__nv_bfloat16*>(p.lo);
  for (int e = threadIdx.x; e < TR * TK; e += PACK_THREADS) {
    const int rr = e / TK, kk = e % TK;
    if (r0 + rr >= p.R) continue;
    const long long at = t.orow[rr] * p.Kp + k0 + kk;
    const double v = t.v[rr][kk];
    const __nv_bfloat16 h = __double2bfloat16(v);
    hi[at] = h;
    double rest = v - (double)__bfloat162float(h);
    const __nv_bfloat16 m = __double2bfloat16(rest);
    mid[at] = m;
    rest -= (double)__bfloat162float(m);
    lo[at] = __double2bfloat16(rest);
  }
}

// FP8 pass 1: per-row max |v| into rowmax (float bits, zero-initialised; |v| >= 0 so the
// unsigned order of the bits is the float order).
template <bool KF>
__global__ void __launch_bounds__(PACK_THREADS) pack_fp8_max_kernel(const PackArgs p,
                                                                    unsigned* rowmax) {
  __shared__ PackTile<float> t;
  const long long r0 = (long long)blockIdx.x * TR, k0 = (long long)blockIdx.y * TK;
  pack_tile_load<float, KF>(p, t, r0, k0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int rr = warp; rr < TR; rr += PACK_THREADS / 32) {
    float m = fmaxf(fabsf(t.v[rr][lane]), fabsf(t.v[rr][lane + 32]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && r0 + rr < p.R && m > 0.0f)
      atomicMax(rowmax + t.orow[rr], __float_as_uint(m));
  }
}

__device__ __forceinline__ double fp8_scale(unsigned maxbits) {
  // smallest power of two 2^e with max|v| / 2^e <= 448, so dequantisation is exact
  const double m = (double)__uint_as_float(maxbits);
  return (m > 0.0) ? exp2(ceil(log2(m / 448.0))) : 1.0;
}

// FP8 pass 2: replace each row's max bits by its power-of-two scale (once per row).
__global__ void pack_fp8_scale_kernel(long long R, unsigned* rowmax_scale) {
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < R;
       r += (long long)gridDim.x * blockDim.x)
    reinterpret_cast<float*>(rowmax_scale)[r] = (float)fp8_scale(rowmax_scale[r]);
}

// FP8 pass 3: quantise with the row's scale (a power of two, so the FP32 product is exact).
template <bool KF>
__global__ void __launch_bounds__(PACK_THREADS) pack_fp8_kernel(const PackArgs p,
                                                                const float* scale) {
  __shared__ PackTile<float> t;
  const long long r0 = (long long)blockIdx.x * TR, k0 = (long long)blockIdx.y * TK;
  pack_tile_load<float, KF>(p, t, r0, k0);
  __nv_fp8_e4m3* dst = reinterpret_cast<__nv_fp8_e4m3*>(p.hi);
  for (int e = threadIdx.x; e < TR * TK; e += PACK_THREADS) {
    const int rr = e / TK, kk = e % TK;
    if (r0 + rr >= p.R) continue;
    const float inv = 1.0f / scale[t.orow[rr]];
    dst[t.orow[rr] * p.Kp + k0 + kk] = __nv_fp8_e4m3(t.v[rr][kk] * inv);
  }
}

__global__ void scale_epi_kernel(EpiIdx em, EpiIdx en, long long M, long long N, double beta,
                                 double* C) {
  long long total = M * N;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    double* dst = C + epi_offset(em, idx / N) + epi_offset(en, idx % N);
    *dst = (beta == 0.0) ? 0.0 : beta * *dst;
  }
}

// ---- host side --------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)ptr;
  }
  return fn;
}

bool make_map(CUtensorMap* m, const void* base, long long rows, long long ld_bytes,
              long long k_bytes, int elem_bytes, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) {
    set_error("pcg_tc_gemm: cuTensorMapEncodeTiled unavailable");
    return false;
  }
  cuuint64_t dims[2] = {(cuuint64_t)(k_bytes / elem_bytes), (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld_bytes};
  cuuint32_t box[2] = {(cuuint32_t)(KBYTES / elem_bytes), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, elem_bytes == 2 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8,
                  2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("pcg_tc_gemm: cuTensorMapEncodeTiled failed (%d)", (int)r);
    return false;
  }
  return true;
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

template <int BN, int NP = 1, bool SPLIT = false>
int launch(const Maps& maps, Args a, cudaStream_t st) {
  static bool attr = false;
  const int smem = Smem<BN, NP, SPLIT>::TOTAL;
  if (!attr) {
    cudaFuncSetAttribute(tc_gemm_kernel<BN, NP, SPLIT>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  a.nt = (a.N + a.bs - 1) / a.bs;
  const long long ntiles = a.mt * a.nt * a.splits;
  const long long grid = std::min<long long>(ntiles, num_sms());
  tc_gemm_kernel<BN, NP, SPLIT><<<(unsigned)grid, GEMM_THREADS, smem, st>>>(maps, a);
  PCG_CHECK_LAUNCH("pcg_tc_gemm");
  return 0;
}

bool fill_epi(EpiIdx& d, int n, const long long* ext, const long long* s, const char* what) {
  if (n < 0 || n > kMaxSub) {
    set_error("pcg_tc_gemm: %s has %d sub-indices (max %d)", what, n, kMaxSub);
    return false;
  }
  if (n > 0 && (!ext || !s)) {
    set_error("pcg_tc_gemm: %s extents or strides missing", what);
    return false;
  }
  d.n = n ? n : 1;
  if (!n) {
    d.ext[0] = 1;
    d.s[0] = 0;
  }
  for (int q = 0; q < n; ++q) {
    if (ext[q] <= 0 || ext[q] > 0x7fffffffLL) {
      set_error("pcg_tc_gemm: %s extent must be in [1, 2^31)", what);
      return false;
    }
    d.ext[q] = ext[q];
    d.s[q] = s[q];
  }
  return true;
}

bool fill_pack(PackIdx& d, int n, const long long* ext, const long long* str) {
  if (n < 0 || n > kMaxSub) {
    set_error("pcg_pack_operand: %d sub-indices (max %d)", n, kMaxSub);
    return false;
  }
  if (n > 0 && (!ext || !str)) {
    set_error("pcg_pack_operand: extents or strides missing");
    return false;
  }
  d.n = n ? n : 1;
  for (int q = 0; q < kMaxSub; ++q) {
    d.ext[q] = 1;
    for (int s = 0; s < kPackSrc; ++s) d.s[s][q] = 0;
  }
  for (int q = 0; q < n; ++q) {
    if (ext[q] <= 0 || ext[q] > 0x7fffffffLL) {
      set_error("pcg_pack_operand: extent must be in [1, 2^31)");
      return false;
    }
    d.ext[q] = ext[q];
    for (int s = 0; s < kPackSrc; ++s) d.s[s][q] = str[s * kMaxSub + q];
  }
  return true;
}

}  // namespace tc
}  // namespace pcg

using namespace pcg;
using namespace pcg::tc;

extern "C" int pcg_pack_operand(int fmt, int r_n, const long long* r_ext, const long long* r_str,
                                int k_n, const long long* k_ext, const long long* k_str,
                                long long Kp, double a, const double* X, double b,
                                const double* Y, double c, const double* P, const double* Q,
                                double d, const double* R, const double* S, void* hi, void* mid,
                                void* lo, float* row_scale, const long long* row_tab,
                                long long rows, const long long* k_tab, const float* k_w,
                                long long kcount, void* stream) {
  PackArgs p{};
  if (!fill_pack(p.r, r_n, r_ext, r_str) || !fill_pack(p.k, k_n, k_ext, k_str)) return -1;
  p.row_tab = row_tab;
  p.k_tab = k_tab;
  p.k_w = k_w;
  if (fmt == kBF16x3F || fmt == kBF16x3S) fmt = kBF16x3;  // same pieces; the GEMM differs
  if (fmt < 0 || fmt > 3 || (!X && !P && !R) || !hi || ((fmt == kBF16x3 || fmt == kBF16x6) && !lo) ||
      (fmt == kBF16x6 && !mid) || (fmt == kFP8 && !row_scale) || (P && !Q) || (R && !S)) {
    set_error("pcg_pack_operand: bad pointers for format %d", fmt);
    return -1;
  }
  p.R = 1;
  for (int q = 0; q < p.r.n; ++q) p.R *= p.r.ext[q];
  if (row_tab) {
    if (rows <= 0) {
      set_error("pcg_pack_operand: a row table needs rows > 0");
      return -1;
    }
    p.R = rows;
  }
  p.K = 1;
  for (int q = 0; q < p.k.n; ++q) p.K *= p.k.ext[q];
  if (k_tab) {
    if (kcount <= 0) {
      set_error("pcg_pack_operand: a K table needs kcount > 0");
      return -1;
    }
    p.K = kcount;
  } else if (k_w) {
    set_error("pcg_pack_operand: K multipliers need a K table");
    return -1;
  }
  const int kblk = (fmt == kFP8) ? 128 : 64;
  if (Kp < p.K || Kp % kblk != 0) {
    set_error("pcg_pack_operand: Kp=%lld must be >= K=%lld and a multiple of %d", Kp, p.K, kblk);
    return -1;
  }
  p.Kp = Kp;
  p.a = a;
  p.b = b;
  p.c = c;
  p.d = d;
  p.X = X;
  p.Y = Y;
  p.P = P;
  p.Q = Q;
  p.R2 = R;
  p.S2 = S;
  p.hi = hi;
  p.lo = (fmt == kBF16x3 || fmt == kBF16x6) ? lo : nullptr;
  p.mid = (fmt == kBF16x6) ? mid : nullptr;
  p.scale = row_scale;
  p.fmt = fmt;
  // gather along K when X is at least as contiguous along K as along the rows
  // (a table-driven side counts as the gathered side unless the other side is a table too;
  // the caller passes the table's typical step in the unused stride slot then)
  long long ks = 0, rs = 0;
  const int src0 = X ? 0 : (P ? 2 : 4);
  for (int q = 0; q < p.k.n; ++q)
    if (p.k.s[src0][q] != 0)
      ks = (ks == 0) ? llabs(p.k.s[src0][q]) : std::min(ks, llabs(p.k.s[src0][q]));
  for (int q = 0; q < p.r.n; ++q)
    if (p.r.s[src0][q] != 0)
      rs = (rs == 0) ? llabs(p.r.s[src0][q]) : std::min(rs, llabs(p.r.s[src0][q]));
  const int kfast = (rs == 0 || (ks != 0 && ks <= rs)) ? 1 : 0;
  // Rows gathered along their most contiguous sub-index: when that is not the innermost
  // one (rows (b, j) of t2[n][j][f][b]: consecutive rows are a whole (f, b) plane apart),
  // the kernel walks the rows with it moved innermost, so that a warp's consecutive rows
  // are consecutive addresses, and writes each walked row to its own output row.
  p.out_perm = 0;
  if (!kfast && !row_tab && p.r.n >= 2) {
    int qs = -1;
    for (int q = 0; q < p.r.n; ++q)
      if (p.r.s[src0][q] != 0 && (qs < 0 || llabs(p.r.s[src0][q]) < llabs(p.r.s[src0][qs])))
        qs = q;
    if (qs >= 0 && qs != p.r.n - 1) {
      long long ostr[kMaxSub];
      long long run = 1;
      for (int q = p.r.n - 1; q >= 0; --q) {  // output row strides in the given order
        ostr[q] = run;
        run *= p.r.ext[q];
      }
      PackIdx g = p.r;
      int w = 0;
      for (int q = 0; q < p.r.n; ++q) {
        if (q == qs) continue;
        g.ext[w] = p.r.ext[q];
        for (int s = 0; s < kPackSrc; ++s) g.s[s][w] = p.r.s[s][q];
        p.out_str[w] = ostr[q];
        ++w;
      }
      g.ext[w] = p.r.ext[qs];
      for (int s = 0; s < kPackSrc; ++s) g.s[s][w] = p.r.s[s][qs];
      p.out_str[w] = ostr[qs];
      p.r = g;
      p.out_perm = 1;
    }
  }
  const long long gx = (p.R + TR - 1) / TR, gy = Kp / TK;
  if (gy > 65535 || p.R > 0x7fffffffLL - TR) {  // row and K indices stay below 2^31
    set_error("pcg_pack_operand: operand too large (%lld x %lld)", p.R, Kp);
    return -1;
  }
  dim3 grid((unsigned)gx, (unsigned)gy);
  cudaStream_t st = (cudaStream_t)stream;
  if (fmt == kFP8) {
    unsigned* mx = reinterpret_cast<unsigned*>(row_scale);
    cudaMemsetAsync(mx, 0, sizeof(float) * p.R, st);
    if (kfast)
      pack_fp8_max_kernel<true><<<grid, PACK_THREADS, 0, st>>>(p, mx);
    else
      pack_fp8_max_kernel<false><<<grid, PACK_THREADS, 0, st>>>(p, mx);
    PCG_CHECK_LAUNCH("pcg_pack_operand/max");
    pack_fp8_scale_kernel<<<(unsigned)std::min<long long>((p.R + 255) / 256, 4096), 256, 0, st>>>(p.R, mx);
    PCG_CHECK_LAUNCH("pcg_pack_operand/scale");
    if (kfast)
      pack_fp8_kernel<true><<<grid, PACK_THREADS, 0, st>>>(p, row_scale);
    else
      pack_fp8_kernel<false><<<grid, PACK_THREADS, 0, st>>>(p, row_scale);
  } else if (fmt == kBF16x6) {
    if (kfast)
      pack_bf16x6_kernel<true><<<grid, PACK_THREADS, 0, st>>>(p);
    else
      pack_bf16x6_kernel<false><<<grid, PACK_THREADS, 0, st>>>(p);
  } else {
    const bool prod = P || R;
    if (kfast && prod)
      pack_bf16_kernel<true, true><<<grid, PACK_THREADS, 0, st>>>(p);
    else if (kfast)
      pack_bf16_kernel<true, false><<<grid, PACK_THREADS, 0, st>>>(p);
    else if (prod)
      pack_bf16_kernel<false, true><<<grid, PACK_THREADS, 0, st>>>(p);
    else
      pack_bf16_kernel<false, false><<<grid, PACK_THREADS, 0, st>>>(p);
  }
  PCG_CHECK_LAUNCH("pcg_pack_operand");
  return 0;
}

extern "C" int pcg_tc_gemm(int fmt, const void* A_hi, const void* A_mid, const void* A_lo,
                           long long M, long long lda, const void* B_hi, const void* B_mid,
                           const void* B_lo, long long N, long long ldb, long long Kp,
                           const float* a_scale, const float* b_scale, int m_n,
                           const long long* m_ext, const long long* m_sc, int n_n,
                           const long long* n_ext, const long long* n_sc,
                           const long long* col_map, const double* col_scale, double alpha,
                           double beta, double* C, int* status, void* stream) {
  if (fmt < 0 || fmt > 5) {
    set_error("pcg_tc_gemm: unknown format %d", fmt);
    return -1;
  }
  const int eb = (fmt == kFP8) ? 1 : 2;
  const int kblk = KBYTES / eb;
  const bool need_lo =
      (fmt == kBF16x3 || fmt == kBF16x6 || fmt == kBF16x3F || fmt == kBF16x3S);
  if (!A_hi || !B_hi || !C || !status || (need_lo && (!A_lo || !B_lo)) ||
      (fmt == kBF16x6 && (!A_mid || !B_mid)) || (fmt == kFP8 && (!a_scale || !b_scale))) {
    set_error("pcg_tc_gemm: null pointer for format %d", fmt);
    return -1;
  }
  if (M <= 0 || N <= 0 || Kp <= 0 || Kp % kblk != 0 || lda < Kp || ldb < Kp ||
      (lda * eb) % 16 != 0 || (ldb * eb) % 16 != 0) {
    set_error("pcg_tc_gemm: bad sizes M=%lld N=%lld Kp=%lld lda=%lld ldb=%lld", M, N, Kp, lda, ldb);
    return -1;
  }
  const void* ptrs[6] = {A_hi, A_mid, A_lo, B_hi, B_mid, B_lo};
  for (const void* q : ptrs)
    if (q && ((uintptr_t)q % 16) != 0) {
      set_error("pcg_tc_gemm: operand base not 16-byte aligned");
      return -1;
    }
  if (M > 0x7fffffffLL - BM || N > 0x7fffffffLL) {
    set_error("pcg_tc_gemm: M or N exceeds the TMA coordinate range");
    return -1;
  }
  Args a{};
  a.M = M;
  a.N = N;
  a.fp8 = (fmt == kFP8);
  // pieces: 0 = hi, 1 = mid (BF16x6) or lo (BF16x3), 2 = lo (BF16x6)
  static const PassTable t1 = {1, {0}, {0}};
  static const PassTable t3 = {3, {1, 0, 0}, {0, 1, 0}};
  static const PassTable t6 = {6, {2, 1, 0, 1, 0, 0}, {0, 1, 2, 0, 1, 0}};
  a.pt = (fmt == kBF16x3) ? t3 : (fmt == kBF16x6 ? t6 : t1);
  a.npass = a.pt.n;
  if (!fill_epi(a.em, m_n, m_ext, m_sc, "M") || !fill_epi(a.en, n_n, n_ext, n_sc, "N")) return -1;
  if (!col_map) {  // the epilogue keeps column offsets in 32 bits
    long long span = 0;
    for (int q = 0; q < a.en.n; ++q) span += (a.en.ext[q] - 1) * llabs(a.en.s[q]);
    if (span > 0x7fffffffLL) {
      set_error("pcg_tc_gemm: column offsets of C reach %lld (limit 2^31 - 1)", span);
      return -1;
    }
  }
  a.alpha = alpha;
  a.beta = beta;
  a.C = C;
  a.a_scale = a_scale;
  a.b_scale = b_scale;
  a.col_map = col_map;
  a.col_scale = col_scale;
  a.status = status;
  a.wait_ns = wait_limit_ns();
  // Tile width: the least SM time, counting whole waves of the persistent grid (a launch
  // with fewer tiles than SMs is split along K instead) and weighting each tile by its
  // columns plus its fixed A-operand share.
  static const int kBN[] = {64, 96, 128, 160, 192, 224, 256};
  const bool fused = (fmt == kBF16x3F || fmt == kBF16x3S);
  const bool split_acc = (fmt == kBF16x3S);
  const long long sms_all = num_sms();
  int BN = 64;
  long long best = -1;
  for (int bn : kBN) {
    if (split_acc && bn > 160) continue;  // three accumulators in 512 TMEM columns
    // fused split formats hold hi and lo of both operands per stage: above 160 columns only
    // two stages fit in shared memory, and the pipeline then stalls on TMA latency
    // (measured on GB300: 160 columns and three stages issue 1450-1680 TFLOP/s on the
    // ladder and ring shapes, 224 or 256 columns and two stages 1140-1510)
    if (fused && bn > 160) continue;
    const long long tiles = ((M + BM - 1) / BM) * ((N + bn - 1) / bn);
    const long long slots = tiles >= sms_all ? (tiles + sms_all - 1) / sms_all * sms_all : tiles;
    const long long cost = slots * (bn + 48);
    if (best < 0 || cost < best || (cost == best && bn > BN)) {
      best = cost;
      BN = bn;
    }
  }
  long long mt = (M + BM - 1) / BM, nt = (N + BN - 1) / BN;
  if (mt > 0x7fffffffLL || nt > 0x7fffffffLL) {
    set_error("pcg_tc_gemm: too many tiles (M tiles %lld)", mt);
    return -1;
  }
  const int nkb = (int)(Kp / kblk);
  long long tiles = mt * nt;
  int splits = 1;
  const int sms = num_sms();
  // K splits for a launch with fewer tiles than SMs: the count s that minimises the launch's
  // length in tile times, ceil(tiles s / SMs) / s (whole waves of the persistent grid: a
  // count that overfills a wave by one tile doubles the launch, as 3 tiles x 51 splits on
  // 152 SMs did), the smallest s within 3 % of the shortest (fewer FP64 atomics);
  // s <= 4 SMs / tiles, and each split at least 4 K blocks long
  if (tiles < sms && nkb >= 8) {
    const long long smax = std::max(1LL, std::min<long long>(nkb / 4, 4LL * sms / tiles));
    auto len = [&](long long sc) { return (double)((tiles * sc + sms - 1) / sms) / (double)sc; };
    double best = 1e30;
    for (long long sc = 1; sc <= smax; ++sc) best = std::min(best, len(sc));
    for (long long sc = 1; sc <= smax; ++sc)
      if (len(sc) <= best * 1.03) {
        splits = (int)sc;
        break;
      }
  }
  int kps = (nkb + splits - 1) / splits;
  splits = (nkb + kps - 1) / kps;
  a.mt = mt;
  a.nt = nt;
  // N is cut into nt tiles of near-equal width (bs columns, a multiple of 16, the last tile
  // the rest): tiles that take about the same time keep the CTAs that share an A row block
  // in step, so they find it in L2.  A narrow last tile (820 = 5 x 160 + 20 columns) ends
  // early and its CTA runs ahead onto other row blocks (measured on GB300 at 820 columns:
  // the A operand read 2.5 times from DRAM, against 1.05 times at 780 = 4 x 160 + 140).
  // bs <= BN and bs * nt >= N, so the tile count is unchanged.
  {
    const long long units = (N + 15) / 16;
    a.bs = (int)(16 * ((units + nt - 1) / nt));
  }
  // B's tensor map box is bs rows high (a narrower tile loads no rows it does not multiply);
  // the stage's B slot keeps BN rows
  a.stage_bytes = (fmt == kBF16x3F || fmt == kBF16x3S ? 2 : 1) * (BM + a.bs) * KBYTES;
  // raster group: a wave of W CTAs touches gm A row blocks (BM rows) and W / gm B row
  // blocks (BN rows); gm = sqrt(W BN / BM) minimises their sum.  A narrow N (nt <= W / gm)
  // keeps the N-fastest order (gm = 1): the CTAs sharing an A row block are then adjacent
  // and each A block is read once per wave (measured on GB300: the ladder's 6 N tiles run
  // 7-8 % faster this way than in groups of M-fastest tiles; the 12000 x 12000 ring GEMMs
  // 12 % faster in groups than N-fastest).
  {
    const long long W = std::min<long long>(mt * nt * splits, sms_all);
    long long gm = (long long)std::llround(std::sqrt((double)W * BN / BM));
    gm = std::max(1LL, std::min(gm, mt));
    if (nt * gm <= W) gm = 1;
    a.gm = (int)gm;
  }
  a.splits = splits;
  a.nkb_total = nkb;
  a.kb_per_split = kps;
  // FP32 accumulation chain per FP64 flush: 4096 K for split-BF16x3 (fused or by passes),
  // 2048 K for BF16x6, 12288 K for single BF16.
  a.kb_chunk = (fmt == kBF16x3 || fmt == kBF16x3F || fmt == kBF16x3S) ? 64
                                                                      : (fmt == kBF16x6 ? 32 : 192);
  a.atomic_out = splits > 1;
  // a tile whose K fits one flush adds its result into C once: as a reduction the add is
  // done at L2 and the epilogue does not wait a DRAM round trip per tile for the old values
  // (the short-K terms are bound by that wait)
  a.red_out = (splits == 1 && nkb <= a.kb_chunk) ? 1 : 0;
  cudaStream_t st = (cudaStream_t)stream;
  if (a.atomic_out && beta != 1.0) {
    int blocks = (int)std::min<long long>((M * N + 255) / 256, 4096);
    scale_epi_kernel<<<blocks, 256, 0, st>>>(a.em, a.en, M, N, beta, C);
    PCG_CHECK_LAUNCH("pcg_tc_gemm/scale");
  }
  Maps maps;
  const void* pa[3] = {A_hi, fmt == kBF16x6 ? A_mid : A_lo, A_lo};
  const void* pb[3] = {B_hi, fmt == kBF16x6 ? B_mid : B_lo, B_lo};
  for (int q = 0; q < 3; ++q) {
    if (!make_map(&maps.a[q], pa[q] ? pa[q] : A_hi, M, lda * eb, Kp * eb, eb, BM)) return -1;
    if (!make_map(&maps.b[q], pb[q] ? pb[q] : B_hi, N, ldb * eb, Kp * eb, eb, a.bs)) return -1;
  }
  if (split_acc) {
    switch (BN) {
      case 64: return launch<64, 2, true>(maps, a, st);
      case 96: return launch<96, 2, true>(maps, a, st);
      case 128: return launch<128, 2, true>(maps, a, st);
      default: return launch<160, 2, true>(maps, a, st);
    }
  }
  if (fused) {
    switch (BN) {
      case 64: return launch<64, 2>(maps, a, st);
      case 96: return launch<96, 2>(maps, a, st);
      case 128: return launch<128, 2>(maps, a, st);
      case 160: return launch<160, 2>(maps, a, st);
      case 192: return launch<192, 2>(maps, a, st);
      case 224: return launch<224, 2>(maps, a, st);
      default: return launch<256, 2>(maps, a, st);
    }
  }
  switch (BN) {
    case 64: return launch<64>(maps, a, st);
    case 96: return launch<96>(maps, a, st);
    case 128: return launch<128>(maps, a, st);
    case 160: return launch<160>(maps, a, st);
    case 192: return launch<192>(maps, a, st);
    case 224: return launch<224>(maps, a, st);
    default: return launch<256>(maps, a, st);
  }
}

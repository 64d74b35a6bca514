// The particle-particle ladder r_ijab += 1/2 sum_ef tau_ijef <ab|ef> (pycc/ccwfn.py:931) in
// symmetric / antisymmetric pair form: the assembly of its two GEMM results into the half
// residual of r_T2.
//
// With T+-_ij,ef = tau_ijef +- tau_ijfe and V+-_ab,ef = <ab|ef> +- <ab|fe> (V+_ab,ee =
// <ab|ee>), the two GEMMs
//   G+_(ij),(ab) = sum_{e<=f} T+_ij,ef V+_ab,ef      (i <= j, a <= b)
//   G-_(ij),(ab) = sum_{e<f}  T-_ij,ef V-_ab,ef      (i <  j, a <  b)
// give S_ijab = sum_ef tau_ijef <ab|ef> = 1/2 (G+ + s_ab G-), s_ab = sign(b - a): G+ is
// symmetric and G- antisymmetric under i<->j and under a<->b, since tau_jife = tau_ijef and
// <ba|fe> = <ab|ef>.  The GEMMs apply the 1/2 (a power of two) in their epilogue.  Each
// GEMM multiplies about a quarter of the ordered-pair product, so the two together issue
// half of the i <= j pair form's tensor-core work.
//
// The half residual h is only ever read through the symmetrisation r2 = h_ijab + h_jiba
// (pycc/ccwfn.py:790), which doubles the ladder's 1/2 S.  As in the i <= j pair form, the
// pair i < j carries the whole S (h_jiba none of it), and S may be written to either of the
// two places it reaches: for a > b it goes to h_jiba, with b < a.  Every write of the
// assembly then lies in the a <= b triangle of a pair's (a, b) block, and G+ / G- are read
// along their pair index, both unit-stride.  For i = j, h_iiab carries 1/2 S_iiab + 1/2
// S_iiba = S_iiab for a < b and 1/2 S_iiaa on the diagonal.
#include "common.cuh"

namespace pcg {
namespace {

constexpr int LADDER_THREADS = 256;

// Block (x, q): the i <= j pair q (row-major over i) and the virtual rows a0 = x and
// a1 = nv - 1 - x (together nv + 1 elements of the a <= b triangle, so blocks are balanced).
__global__ void __launch_bounds__(LADDER_THREADS)
    ladder_pm_assemble_kernel(const double* __restrict__ Gp, const double* __restrict__ Gm,
                              int no, int nv, double* __restrict__ r) {
  const int q = blockIdx.y;
  int i = 0, rem = q;
  while (rem >= no - i) {
    rem -= no - i;
    ++i;
  }
  const int j = i + rem;
  const long long P = (long long)nv * (nv + 1) / 2, Q = (long long)nv * (nv - 1) / 2;
  const long long qm = (long long)q - (i + 1);  // (i, j) among the i < j pairs (j > i)
  const int a0 = blockIdx.x, a1 = nv - 1 - blockIdx.x;
  const int n0 = nv - a0;
  const int n1 = (a1 > a0) ? nv - a1 : 0;
  const long long vv = (long long)nv * nv;
  double* hij = r + ((long long)i * no + j) * vv;
  double* hji = r + ((long long)j * no + i) * vv;
  const double* gp_q = Gp + (long long)q * P;
  const double* gm_q = (Gm && j > i) ? Gm + qm * Q : nullptr;
  for (int t = threadIdx.x; t < n0 + n1; t += LADDER_THREADS) {
    const int a = t < n0 ? a0 : a1;
    const int b = t < n0 ? a0 + t : a1 + (t - n0);
    const long long p = (long long)a * nv - (long long)a * (a - 1) / 2 + (b - a);
    const long long at = (long long)a * nv + b;
    const double gp = gp_q[p];
    if (j > i) {
      const double gm = (gm_q && b > a) ? gm_q[p - (a + 1)] : 0.0;
      hij[at] += gp + gm;
      if (b > a) hji[at] += gp - gm;
    } else {
      hij[at] += (b > a) ? gp : 0.5 * gp;
    }
  }
}

// Block (x, i): rows r0 = 32 x .. r0 + 31 and the occupied index i; the pairs (i, j >= i)
// in chunks of 32.  G+- are read along the row index (unit-stride) into shared memory, and
// written along j into row i of each row's (i, j) block; the transposed element (j, i) is a
// strided write.  Every element of Z has one writer: (x, y) with y >= x by block x, (x, y)
// with x > y by block y.
__global__ void __launch_bounds__(LADDER_THREADS)
    pair_pm_assemble_kernel(const double* __restrict__ Gp, const double* __restrict__ Gm,
                            int no, long long nrow, double* __restrict__ Z) {
  __shared__ double sp[32][33], sm[32][33];
  const int i = blockIdx.y;
  const long long r0 = (long long)blockIdx.x * 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long pi = (long long)i * no - (long long)i * (i - 1) / 2;        // p(i, i)
  const long long mi = (long long)i * (no - 1) - (long long)i * (i - 1) / 2;  // pm(i, i + 1)
  const long long oo = (long long)no * no;
  for (int jc = i; jc < no; jc += 32) {
    for (int jj = warp; jj < 32; jj += LADDER_THREADS / 32) {
      const int j = jc + jj;
      const long long r = r0 + lane;
      double gp = 0.0, gm = 0.0;
      if (j < no && r < nrow) {
        gp = Gp[(pi + (j - i)) * nrow + r];
        if (j > i && Gm) gm = Gm[(mi + (j - i - 1)) * nrow + r];
      }
      sp[jj][lane] = gp;
      sm[jj][lane] = gm;
    }
    __syncthreads();
    for (int rr = warp; rr < 32; rr += LADDER_THREADS / 32) {
      const long long r = r0 + rr;
      const int j = jc + lane;
      if (r < nrow && j < no) {
        const double gp = sp[lane][rr], gm = sm[lane][rr];
        double* zr = Z + r * oo;
        if (j > i) {
          zr[(long long)i * no + j] += gp + gm;
          zr[(long long)j * no + i] += gp - gm;
        } else {
          zr[(long long)i * no + i] += gp;
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace pcg

using namespace pcg;

// h[i,j,a,b] += the ladder term from G+ ([no(no+1)/2][nv(nv+1)/2]) and G- ([no(no-1)/2]
// [nv(nv-1)/2]), both FP64 and contiguous, as described above.  Gm may be NULL when it is
// empty (no = 1 or nv = 1).  h: the contiguous [no][no][nv][nv] half residual.
extern "C" int pcg_ladder_pm_assemble(const double* Gp, const double* Gm, long long no,
                                      long long nv, double* h, void* stream) {
  if (!Gp || !h || no <= 0 || nv <= 0 || no > 65535 || nv > 65535 ||
      (!Gm && no > 1 && nv > 1)) {
    set_error("pcg_ladder_pm_assemble: bad arguments (no=%lld nv=%lld)", no, nv);
    return -1;
  }
  const long long pairs = no * (no + 1) / 2;
  if (pairs > 65535) {
    set_error("pcg_ladder_pm_assemble: %lld occupied pairs exceed the grid", pairs);
    return -1;
  }
  dim3 grid((unsigned)((nv + 1) / 2), (unsigned)pairs);
  ladder_pm_assemble_kernel<<<grid, LADDER_THREADS, 0, (cudaStream_t)stream>>>(Gp, Gm, (int)no,
                                                                               (int)nv, h);
  PCG_CHECK_LAUNCH("pcg_ladder_pm_assemble");
  return 0;
}

// Z[r][i][j] += Gp + Gm and Z[r][j][i] += Gp - Gm for i < j, Z[r][i][i] += Gp, with Gp
// [no(no+1)/2][nrow] over the i <= j pairs and Gm [no(no-1)/2][nrow] over the i < j pairs
// (row-major over i), both FP64 and contiguous; Z: the contiguous [nrow][no][no] FP64
// array.  Gm may be NULL when it is empty (no = 1).
extern "C" int pcg_pair_pm_assemble(const double* Gp, const double* Gm, long long no,
                                    long long nrow, double* Z, void* stream) {
  if (!Gp || !Z || no <= 0 || nrow <= 0 || no > 65535 || (!Gm && no > 1) ||
      (nrow + 31) / 32 > 0x7fffffffLL) {
    set_error("pcg_pair_pm_assemble: bad arguments (no=%lld nrow=%lld)", no, nrow);
    return -1;
  }
  dim3 grid((unsigned)((nrow + 31) / 32), (unsigned)no);
  pair_pm_assemble_kernel<<<grid, LADDER_THREADS, 0, (cudaStream_t)stream>>>(Gp, Gm, (int)no,
                                                                             nrow, Z);
  PCG_CHECK_LAUNCH("pcg_pair_pm_assemble");
  return 0;
}

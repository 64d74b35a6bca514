// (T) densities and Lambda sources (pycc/cctriples.py:1063-1157, t3_density), FP64: the two
// elementwise kernels of one (i, j, k) triple.  The contractions that follow them run on the
// FP64 DMMA contraction kernel.
//
// pcg_t3_ijk_f64: from the connected partials of the triple (P[3][v][v][v], laid out as in the
// (T) energy: W[a,b,c] = P1[c][a][b] + P2[b][a][c] + P3[a][b][c]) and the integrals, the
// triple's connected and disconnected amplitudes divided by the orbital-energy denominator
// D = e_i + e_j + e_k - e_a - e_b - e_c (t3c_ijk and t3d_ijk with WithDenom):
//   M3[a,b,c] = W[a,b,c] / D
//   N3[a,b,c] = (<ij|ab> t_kc + <ik|ac> t_jb + <jk|bc> t_ia
//                + t2_ijab f_kc + t2_ikac f_jb + t2_jkbc f_ia) / D
//
// pcg_t3_density_terms_f64: the permutation combinations of M3 / N3 the densities contract:
//   sym(X)_abc = 8 X_abc - 4 X_bac - 4 X_acb - 4 X_cba + 2 X_cab + 2 X_bca
//   A  = sym(2 M3 + N3)   (= 2 X3 + Y3 of the reference, sym being linear)
//   S  = sym(M3 + N3)     (= X3 + Y3)
//   Z  = 2 M_abc - 2 M_acb - M_bac + M_bca
//   Ma = M_abc - M_cba,  Mb = 2 M_abc - M_acb - M_cba,  Mc = 2 M_abc - 2 M_bac
// All FP64 (the engine's reference-grade path).
#include "common.cuh"

namespace pcg {
namespace {

constexpr int T3_THREADS = 256;

__global__ void t3_ijk_kernel(const double* __restrict__ P, const double* __restrict__ eps,
                              int i, int j, int k, int no, int nv,
                              const double* __restrict__ Woovv, const double* __restrict__ t1,
                              const double* __restrict__ t2, const double* __restrict__ fov,
                              double* __restrict__ M3, double* __restrict__ N3) {
  const long long v = nv, v2 = v * v, v3 = v2 * v;
  const double* P1 = P;
  const double* P2 = P + v3;
  const double* P3 = P + 2 * v3;
  const double eijk = eps[i] + eps[j] + eps[k];
  const double* ev = eps + no;
  const double* Wij = Woovv + ((long long)i * no + j) * v2;
  const double* Wik = Woovv + ((long long)i * no + k) * v2;
  const double* Wjk = Woovv + ((long long)j * no + k) * v2;
  const double* Tij = t2 + ((long long)i * no + j) * v2;
  const double* Tik = t2 + ((long long)i * no + k) * v2;
  const double* Tjk = t2 + ((long long)j * no + k) * v2;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < v3;
       e += (long long)gridDim.x * blockDim.x) {
    const long long c = e % v, b = (e / v) % v, a = e / v2;
    const double W = P1[(c * v + a) * v + b] + P2[(b * v + a) * v + c] + P3[(a * v + b) * v + c];
    const double D = eijk - ev[a] - ev[b] - ev[c];
    double n = Wij[a * v + b] * t1[k * v + c] + Wik[a * v + c] * t1[j * v + b] +
               Wjk[b * v + c] * t1[i * v + a];
    if (fov)
      n += Tij[a * v + b] * fov[k * v + c] + Tik[a * v + c] * fov[j * v + b] +
           Tjk[b * v + c] * fov[i * v + a];
    M3[e] = W / D;
    N3[e] = n / D;
  }
}

__device__ __forceinline__ double sym6(const double* X, long long v, long long a, long long b,
                                       long long c) {
  const long long v2 = v * v;
  return 8.0 * X[a * v2 + b * v + c] - 4.0 * X[b * v2 + a * v + c] - 4.0 * X[a * v2 + c * v + b] -
         4.0 * X[c * v2 + b * v + a] + 2.0 * X[c * v2 + a * v + b] + 2.0 * X[b * v2 + c * v + a];
}

__global__ void t3_terms_kernel(const double* __restrict__ M, const double* __restrict__ N,
                                int nv, double* __restrict__ A, double* __restrict__ S,
                                double* __restrict__ Z, double* __restrict__ Ma,
                                double* __restrict__ Mb, double* __restrict__ Mc) {
  const long long v = nv, v2 = v * v, v3 = v2 * v;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < v3;
       e += (long long)gridDim.x * blockDim.x) {
    const long long c = e % v, b = (e / v) % v, a = e / v2;
    const double sm = sym6(M, v, a, b, c), sn = sym6(N, v, a, b, c);
    A[e] = 2.0 * sm + sn;
    S[e] = sm + sn;
    const double m = M[e], m_acb = M[a * v2 + c * v + b], m_bac = M[b * v2 + a * v + c];
    const double m_bca = M[b * v2 + c * v + a], m_cba = M[c * v2 + b * v + a];
    Z[e] = 2.0 * m - 2.0 * m_acb - m_bac + m_bca;
    Ma[e] = m - m_cba;
    Mb[e] = 2.0 * m - m_acb - m_cba;
    Mc[e] = 2.0 * m - 2.0 * m_bac;
  }
}

int t3_blocks(long long n) {
  long long b = (n + T3_THREADS - 1) / T3_THREADS;
  return (int)(b < 152LL * 16 ? (b < 1 ? 1 : b) : 152LL * 16);
}

}  // namespace
}  // namespace pcg

using namespace pcg;

// M3 / N3 of the triple (i, j, k) (see top of file).  P: the three connected partials
// [3][nv^3]; eps: nmo orbital energies; Woovv: <ij|ab> [no][no][nv][nv]; t1 [no][nv]; t2
// [no][no][nv][nv]; fov: the occupied-virtual Fock block [no][nv] or NULL when it is zero;
// M3, N3: [nv^3].  All contiguous FP64 device arrays.
extern "C" int pcg_t3_ijk_f64(const double* P, const double* eps, int i, int j, int k, int no,
                              int nv, const double* Woovv, const double* t1, const double* t2,
                              const double* fov, double* M3, double* N3, void* stream) {
  if (!P || !eps || !Woovv || !t1 || !t2 || !M3 || !N3 || no < 1 || nv < 1 || i < 0 ||
      j < 0 || k < 0 || i >= no || j >= no || k >= no) {
    set_error("pcg_t3_ijk_f64: bad arguments");
    return -1;
  }
  const long long n = (long long)nv * nv * nv;
  t3_ijk_kernel<<<t3_blocks(n), T3_THREADS, 0, (cudaStream_t)stream>>>(
      P, eps, i, j, k, no, nv, Woovv, t1, t2, fov, M3, N3);
  PCG_CHECK_LAUNCH("pcg_t3_ijk_f64");
  return 0;
}

// The permutation combinations A, S, Z, Ma, Mb, Mc of M3 and N3 (see top of file), each
// [nv^3] contiguous FP64.
extern "C" int pcg_t3_density_terms_f64(const double* M3, const double* N3, int nv, double* A,
                                        double* S, double* Z, double* Ma, double* Mb,
                                        double* Mc, void* stream) {
  if (!M3 || !N3 || !A || !S || !Z || !Ma || !Mb || !Mc || nv < 1) {
    set_error("pcg_t3_density_terms_f64: bad arguments");
    return -1;
  }
  const long long n = (long long)nv * nv * nv;
  t3_terms_kernel<<<t3_blocks(n), T3_THREADS, 0, (cudaStream_t)stream>>>(M3, N3, nv, A, S, Z,
                                                                         Ma, Mb, Mc);
  PCG_CHECK_LAUNCH("pcg_t3_density_terms_f64");
  return 0;
}

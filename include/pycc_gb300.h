/* pycc_gb300 -- C ABI of the GB300-native RHF-CCSD amplitude engine.
 *
 * Every entry point takes raw device pointers (FP64 unless stated), element counts and
 * element strides, plus a cudaStream_t passed as void* (NULL = legacy default stream).
 * Work is enqueued asynchronously on that stream.  The return value is 0 on success and
 * negative on a host-side argument/launch error; pcg_last_error() then holds the text.
 *
 * The reference (CrawfordGroup/pycc) is pure Python; each entry below names the reference
 * function whose arithmetic it replaces.  The reference-side binding is shown in
 * INTEGRATION.md.
 */
#ifndef PYCC_GB300_H
#define PYCC_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- library ------------------------------------------------------------------------- */
const char* pcg_last_error(void);
int pcg_abi_version(void);
/* Failure detection of the tensor-core kernels (no counterpart in the reference, whose only
 * failure handling is input validation, pycc/exceptions.py:27-50): every device-side wait
 * is bounded.  pcg_set_wait_limit_ns sets the bound (ns) passed to the kernels launched from
 * then on (<= 0: the 4 s default; capped at 600 s) and returns the previous one.
 * pcg_wait_probe launches a self-test that waits on an mbarrier nothing completes, with that
 * bound, and sets *status (device int) to 4 when the wait expires. */
long long pcg_set_wait_limit_ns(long long ns);
int pcg_wait_probe(int* status, void* stream);
/* number of kernels this library has launched since it was loaded */
long long pcg_launch_count(void);
/* compute capability of the current device as major*10+minor (103 on GB300) */
int pcg_device_cc(void);
int pcg_stream_sync(void* stream);

/* ---- FP64 strided contraction ---------------------------------------------------------
 * Replaces ContractionBackend.__call__ (pycc/device.py:64-87), i.e. every pairwise
 * self.contract(...) of the CCSD builders (pycc/ccwfn.py:432-945):
 *   C[m,n] = beta*C[m,n] + alpha * sum_k A[m,k] * B[n,k]
 * m, n, k are flat indices over up to 4 sub-indices each (outer first), given as extents
 * and element strides: M sub-indices carry (stride in A, stride in C), N sub-indices
 * (stride in B, stride in C), K sub-indices (stride in A, stride in B).  An empty group
 * (count 0) is a single index of extent 1 (outer products, full dots). */
int pcg_contract_f64(int m_n, const long long* m_ext, const long long* m_sa,
                     const long long* m_sc, int n_n, const long long* n_ext,
                     const long long* n_sb, const long long* n_sc, int k_n,
                     const long long* k_ext, const long long* k_sa, const long long* k_sb,
                     double alpha, const double* A, const double* B, double beta, double* C,
                     void* stream);

/* Sum of up to four FP64 contractions into one output (written once):
 *   C = beta*C + sum_t alpha[t] * A_t[m,k] B_t[n,k]
 * Common M / N extents and C strides (m_ext, m_sc, n_ext, n_sc); per term t the A strides
 * of the M sub-indices m_sa[t*4+q], the B strides of the N sub-indices n_sb[t*4+q] and its
 * own K group (k_n[t]; k_ext, k_sa, k_sb at [t*4+q]); A, B, alpha: host arrays of nterm.
 * The four t3 terms of one output orientation, t3c_ijk (pycc/cctriples.py:56-67). */
int pcg_contract_multi_f64(int nterm, int m_n, const long long* m_ext, const long long* m_sc,
                           const long long* m_sa, int n_n, const long long* n_ext,
                           const long long* n_sc, const long long* n_sb, const int* k_n,
                           const long long* k_ext, const long long* k_sa, const long long* k_sb,
                           const double* alpha, const double* const* A, const double* const* B,
                           double beta, double* C, void* stream);

/* ---- FP64 elementwise kernels ---------------------------------------------------------- */
/* tau_ijab = f1*t2_ijab + f2*t1_ia*t1_jb; CCwfn.build_tau (pycc/ccwfn.py:432-455) */
int pcg_tau_f64(const double* t1, const double* t2, long long no, long long nv, double f1,
                double f2, double* out, void* stream);

/* out[p] = a*X[p] + b*Y[p] over a 4-index box with per-tensor strides (Y may be NULL);
 * the operand combinations 2*t2 - t2.swapaxes(2,3) etc. (pycc/ccwfn.py:757,933-934) */
int pcg_combine4_f64(const long long* ext4, double a, const double* X, const long long* xs4,
                     double b, const double* Y, const long long* ys4, double* out,
                     const long long* os4, void* stream);

/* out_ijab = h_ijab + h_jiba (out != h); r_T2 symmetrisation (pycc/ccwfn.py:790) */
int pcg_symmetrize_f64(const double* h, long long no, long long nv, double* out, void* stream);

/* t1 += r1/Dia, t2 += r2/Dijab with D from eps[nmo]; *rms2 = sum (r/D)^2 (device scalar).
 * work: >= 1024 doubles of device scratch.  solve_cc update (pycc/ccwfn.py:281-284) */
int pcg_update_amps_f64(double* t1, double* t2, const double* r1, const double* r2,
                        const double* eps, long long no, long long nv, double* work,
                        long long work_len, double* rms2, void* stream);

/* inv1[i,a] = 1/(e_i - e_a), inv2[i,j,a,b] = 1/(e_i + e_j - e_a - e_b) from eps[nmo];
 * the denominators of pycc/ccwfn.py:195-198, computed once per Hamiltonian. */
int pcg_inv_denominators_f64(const double* eps, long long no, long long nv, double* inv1,
                             double* inv2, void* stream);
/* t += r * inv over n elements; *rms2 = sum (r*inv)^2 (device scalar); work >= 1024 doubles.
 * The same update as pcg_update_amps_f64 with the divides replaced by products. */
int pcg_update_inv_f64(double* t, const double* r, const double* inv, long long n, double* work,
                       long long work_len, double* rms2, void* stream);

/* *out = 2 sum f_ia t_ia + sum (t2_ijab + t_ia t_jb) L_ijab (device scalar); f: o x v with
 * strides fs[2], L: oovv with strides ls[4]; work >= 1024 doubles.
 * CCwfn.cc_energy (pycc/ccwfn.py:1122-1162) */
int pcg_energy_f64(const double* fov, const long long* fs2, const double* L,
                   const long long* ls4, const double* t1, const double* t2, long long no,
                   long long nv, double* work, long long work_len, double* out, void* stream);

/* out[j] = <x, ys[j]>, 1 <= k <= 16 (ys: host array of device pointers); work >= 1024*k
 * doubles.  DIIS overlaps, helper_diis.extrapolate (pycc/utils.py:330-339) */
int pcg_dots_f64(const double* x, const double* const* ys, int k, long long n, double* work,
                 long long work_len, double* out, void* stream);

/* Allocation-free pcg_dots_f64 (no counterpart in the reference): out[j] = <x, ys[j]> for
 * 1 <= k <= 8, with the partial sums kept in a fixed 64 KB array inside this library
 * instead of a caller-provided work buffer.  For host programs that own all device memory
 * (or must avoid cudaMalloc's implicit synchronisation) and so cannot hand the library
 * scratch.  The first call on a device looks the array's device address up
 * (cudaGetSymbolAddress); make it before any stream capture.  The address is cached for the
 * process's life: do not use the library across a cudaDeviceReset of that device.  All calls
 * share the array: calls that overlap on the GPU race.  k > 8 is rejected. */
int pcg_dots_f64_noalloc(const double* x, const double* const* ys, int k, long long n,
                         double* out, void* stream);

/* e = x - old (e written; e must not alias x or old) and, in the same pass,
 * out[j] = <e, ys[j]> for j < k-1 and out[k-1] = <e, e>; 1 <= k <= 16 (ys: host array of
 * k-1 device pointers); work >= 1024*k doubles.  helper_diis.add_error_vector and the
 * overlap matrix of helper_diis.extrapolate (pycc/utils.py:284-295, :330-339) */
int pcg_diis_error_f64(const double* x, const double* old, double* e, const double* const* ys,
                       int k, long long n, double* work, long long work_len, double* out,
                       void* stream);

/* pcg_diis_error_f64 with FP32 error vectors, for the mixed-precision solver: e = x - old
 * taken in FP64 and rounded once to FP32; overlaps from FP32 products of four consecutive
 * elements, accumulated in FP64.  x, old, e and ys[j] 16-byte aligned.  The reference's
 * helper_diis keeps its error vectors in the amplitudes' own precision
 * (pycc/utils.py:284-295, :330-339); this is its storage at the precision of the
 * tensor-core residual. */
int pcg_diis_error_f32(const double* x, const double* old, float* e, const float* const* ys,
                       int k, long long n, double* work, long long work_len, double* out,
                       void* stream);

/* out = sum_j c[j]*xs[j], 1 <= k <= 16 (xs, c on the host; out must not alias an input).
 * DIIS extrapolation, helper_diis.extrapolate (pycc/utils.py:351-355) */
int pcg_lincomb_f64(const double* const* xs, const double* c, int k, long long n, double* out,
                    void* stream);
/* pcg_lincomb_f64 in double-float arithmetic, for the mixed-precision solver: every FP64
 * input split into FP32 hi + lo pieces in integer arithmetic, products with their FMA
 * rounding errors, the sum carried as an FP32 pair; about 48 significant bits, one FP64
 * instruction per element instead of k.  Inputs and output 16-byte aligned.  The same DIIS
 * extrapolation (pycc/utils.py:351-355). */
int pcg_lincomb_f64_df(const double* const* xs, const double* c, int k, long long n,
                       double* out, void* stream);

/* ---- (T) ---------------------------------------------------------------------------
 * Lee-Rendell E(T) of the reference's t_tjl (pycc/cctriples.py:177-240) for ntrip triples
 * ijk[t] = (i, j, k), i >= j >= k.  The connected triples of triple t are given as three
 * partial tensors (v^3 each, pstride elements apart between triples), column-major GEMM
 * outputs of the three term orientations:
 *   W[a,b,c] = P1[c][a][b] + P2[b][a][c] + P3[a][b][c]
 * the disconnected triples (t3d_ijk, :108-147) are formed from eoovv = <ij|ab>, t1 and, if
 * fov is not NULL, t2 and f_ov.  fp32 != 0: FP32 partials, eoovv and t2 (16-byte aligned)
 * and FP32 element arithmetic (tiles of the (a, b, c) cube); else all FP64.  eps, t1 and
 * fov are FP64 in both.  Writes pcg_triples_part_len(fp32, nv) FP64 partials per
 * triple at part[t * len ...] (weight (2 - d_ij - d_ik - d_jk) applied); E(T) is their sum. */
int pcg_triples_energy(int fp32, const void* P1, const void* P2, const void* P3,
                       long long pstride, const int* ijk, int ntrip, const double* eps,
                       const void* eoovv, const double* t1, const void* t2,
                       const double* fov, long long no, long long nv, double* part,
                       void* stream);
/* FP64 partials per triple written by pcg_triples_energy: nv (FP64), or the number of
 * 8^3 tile triples A >= B >= C of the virtual range (FP32).  (Sizing helper, no reference
 * counterpart.) */
long long pcg_triples_part_len(int fp32, long long nv);
/* *out += sum(x[0:n]) in FP64 (one block, deterministic). */
int pcg_reduce_sum_f64(const double* x, long long n, double* out, void* stream);

/* ---- tensor-core (tcgen05) contraction engine, mixed-precision path ------------------
 * The GB300 replacement of the low-precision path of the same contractions (pycc/ccwfn.py:
 * 458-945 through pycc/device.py:64-87); the reference's own low-precision mode is plain
 * float32 (pycc/device.py:143-154).
 *
 * pcg_pack_operand: dst[r][k] = convert(w_k * (a*X + b*Y + c*P*Q + d*R*S)), each source
 *   read at rowoff_s(r) + koff_s(k); r (k) is a flat index over r_n (k_n) sub-indices with
 *   extents r_ext[q] and strides r_str[s*4 + q] for source s in (X, Y, P, Q, R, S)
 *   (0 = broadcast; 6 x 4 strides).
 *   Formats: 0 BF16 into hi; 1 BF16 hi + lo = bf16(v - hi); 2 FP8 E4M3 bytes into hi with
 *   row_scale[r] = 2^ceil(log2(max_k |v| / 448)); 3 three BF16 pieces hi = bf16(v),
 *   mid = bf16(v - hi), lo = bf16(v - hi - mid).  Rows are Kp elements long (zero padded);
 *   Kp is a multiple of 64 (BF16) or 128 (FP8).  X, P (with Q) or R (with S) must be
 *   given; Y may be NULL; mid is used by format 3 only.  row_tab (optional, device,
 *   [6][rows]) gives the six sources' row offsets explicitly (e.g. the i <= j pairs of a
 *   symmetric operand); the r sub-indices then only tell the kernel which side is
 *   unit-stride, and `rows` rows are packed.  k_tab (optional, device, [6][kcount]) does the
 *   same for K (e.g. the e <= f pairs), with kcount K entries; k_w (optional, device,
 *   kcount floats, needs k_tab) multiplies each K entry (w_k = 1 without it). */
int pcg_pack_operand(int fmt, int r_n, const long long* r_ext, const long long* r_str, int k_n,
                     const long long* k_ext, const long long* k_str, long long Kp, double a,
                     const double* X, double b, const double* Y, double c, const double* P,
                     const double* Q, double d, const double* R, const double* S, void* hi,
                     void* mid, void* lo, float* row_scale, const long long* row_tab,
                     long long rows, const long long* k_tab, const float* k_w,
                     long long kcount, void* stream);

/* pcg_tc_gemm: C[off_m(m) + off_n(n)] = beta*C + alpha * sum_k A[m][k] B[n][k] (C FP64).
 *   A: M rows of lda elements (K-major, 16-byte aligned rows), B: N rows of ldb elements;
 *   format as above, plus 4 = split-BF16x3 fused (both pieces of A and B loaded per stage,
 *   the three products issued from it; faster, with a slightly larger FP32 truncation bias),
 *   5 = split-BF16x3 fused with the small products and the leading product in separate
 *   FP32 accumulators (the leading one flushed per K chunk, the small one once per tile,
 *   added together before the FP64 accumulate: the accuracy of 1, the traffic of 4; N
 *   tiles of at most 160 columns),
 *   1 = three tcgen05 passes Al.Bh + Ah.Bl + Ah.Bh, 3 = the six piece
 *   products of order <= 2^-16 (smallest first), 2 = FP8 with the row scales applied in the
 *   epilogue.  off_m / off_n: flat index over up to 4 sub-indices (extents, element strides
 *   in C); col_map (optional, device, N entries) replaces off_n and col_scale (optional,
 *   device, N doubles) multiplies each column.  Column offsets (off_n or col_map) lie in
 *   [0, 2^31); row offsets are 64-bit.  status: device int, set non-zero when a
 *   bounded device-side wait expired (the kernel then skips its stores). */
int pcg_tc_gemm(int fmt, const void* A_hi, const void* A_mid, const void* A_lo, long long M,
                long long lda, const void* B_hi, const void* B_mid, const void* B_lo, long long N,
                long long ldb, long long Kp, const float* a_scale, const float* b_scale, int m_n,
                const long long* m_ext, const long long* m_sc, int n_n, const long long* n_ext,
                const long long* n_sc, const long long* col_map, const double* col_scale,
                double alpha, double beta, double* C, int* status, void* stream);

/* pcg_ladder_pm_assemble: the particle-particle ladder 1/2 tau_ijef <ab|ef> (pycc/ccwfn.py:931,
 *   the 'ijef,abef->ijab' contraction of ContractionBackend.__call__, pycc/device.py:64-87) in
 *   symmetric / antisymmetric pair form, added into the half residual h of r_T2.  Gp:
 *   [no(no+1)/2][nv(nv+1)/2] = 1/2 sum_{e<=f} T+_ij,ef V+_ab,ef over the i <= j and a <= b
 *   pairs (row-major), Gm: [no(no-1)/2][nv(nv-1)/2] = 1/2 sum_{e<f} T-_ij,ef V-_ab,ef over the
 *   i < j and a < b pairs, with T+- = tau_ijef +- tau_ijfe and V+- = <ab|ef> +- <ab|fe>
 *   (V+_ab,ee = <ab|ee>), so Gp + sign(b - a) Gm = sum_ef tau_ijef <ab|ef>.  For i < j,
 *   a <= b: h_ijab += Gp + Gm and, for a < b, h_jiab += Gp - Gm (the a > b element of pair
 *   (i, j); h only enters through the symmetrisation r2 = h_ijab + h_jiba, so pair i < j
 *   carries the whole term); for i = j: h_iiab += Gp (a < b) or Gp / 2 (a = b).
 *   Gm may be NULL when it is empty (no = 1 or nv = 1). */
int pcg_ladder_pm_assemble(const double* Gp, const double* Gm, long long no, long long nv,
                           double* h, void* stream);

/* pcg_pair_pm_assemble: the same pair form for the tau_ijef X_r,ef terms of the
 *   intermediates (Zmbij: tau_ijef <mb|ef>, pycc/ccwfn.py:715; Wmnij: tau_ijef <mn|ef>,
 *   pycc/ccwfn.py:603; 'ijef,mbef->mbij' / 'ijef,mnef->mnij' of ContractionBackend.__call__).
 *   Gp: [no(no+1)/2][nrow] = 1/2 sum_{e<=f} T+_ij,ef (X_r,ef + X_r,fe) over the i <= j pairs
 *   (row-major, with 1/2 on e = f), Gm: [no(no-1)/2][nrow] = 1/2 sum_{e<f} T-_ij,ef
 *   (X_r,ef - X_r,fe) over the i < j pairs, so Gp + Gm = sum_ef tau_ijef X_r,ef and
 *   Gp - Gm = sum_ef tau_jief X_r,ef.  Z[r][i][j] += Gp + Gm and Z[r][j][i] += Gp - Gm for
 *   i < j, Z[r][i][i] += Gp.  Z: contiguous [nrow][no][no] FP64; Gm may be NULL when no = 1.
 */
int pcg_pair_pm_assemble(const double* Gp, const double* Gm, long long no, long long nrow,
                         double* Z, void* stream);

/* (T) densities and Lambda sources, FP64 (t3_density, pycc/cctriples.py:1063-1157), the two
 * elementwise steps of one ordered triple (i, j, k):
 * pcg_t3_ijk_f64: M3 = t3c_ijk / D and N3 = t3d_ijk / D (pycc/cctriples.py:27-72, :108-147)
 *   from the connected partials P[3][nv^3] (W[a,b,c] = P1[c][a][b] + P2[b][a][c] +
 *   P3[a][b][c], the (T) energy's layout), eps (nmo), <ij|ab> [no][no][nv][nv], t1, t2 and
 *   the occupied-virtual Fock block fov [no][nv] (NULL when zero); D = e_i + e_j + e_k -
 *   e_a - e_b - e_c.
 * pcg_t3_density_terms_f64: with sym(X)_abc = 8X_abc - 4X_bac - 4X_acb - 4X_cba + 2X_cab +
 *   2X_bca: A = sym(2 M3 + N3), S = sym(M3 + N3), Z = 2M_abc - 2M_acb - M_bac + M_bca,
 *   Ma = M_abc - M_cba, Mb = 2M_abc - M_acb - M_cba, Mc = 2M_abc - 2M_bac.
 * All arrays contiguous FP64 on the device. */
int pcg_t3_ijk_f64(const double* P, const double* eps, int i, int j, int k, int no, int nv,
                   const double* Woovv, const double* t1, const double* t2, const double* fov,
                   double* M3, double* N3, void* stream);
int pcg_t3_density_terms_f64(const double* M3, const double* N3, int nv, double* A, double* S,
                             double* Z, double* Ma, double* Mb, double* Mc, void* stream);

/* Grouped segmented BF16 GEMM with FP32 output, the connected-triples builder of the (T)
 * correction (t3c_ijk, pycc/cctriples.py:56-67, for a batch of triples).  Group g computes
 *   C[out_g + m*ldm + n*ldn] = sum_s A[amap_gs][arow_gs + m, :] . B[bmap_gs][brow_gs + n, :]
 * for m < M, n < N over its nseg <= 4 K segments (nkb_gs K blocks of 64).  a_ptr / b_ptr:
 * host arrays of up to four BF16 K-major operand matrices (a_rows[q] rows of a_ld[q]
 * elements).  groups: device array of ngroups records of pcg_tc_group_desc_size() bytes:
 *   int nseg; int amap[4], arow[4], bmap[4], brow[4], nkb[4]; (pad) long long out. */
int pcg_tc_grouped_gemm(int na, const void* const* a_ptr, const long long* a_rows,
                        const long long* a_ld, int nb, const void* const* b_ptr,
                        const long long* b_rows, const long long* b_ld, const void* groups,
                        int ngroups, long long M, long long N, float* C, long long ldm,
                        long long ldn, int* status, void* stream);
int pcg_tc_group_desc_size(void);

#ifdef __cplusplus
}
#endif
#endif /* PYCC_GB300_H */

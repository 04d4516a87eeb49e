/*
 * apyib_gb300 — C ABI of the GB300 (sm_103a) correlated-wavefunction hot path.
 *
 * Every entry point takes device pointers, sizes and a cudaStream_t passed as
 * void*, returns an agb_status (0 = AGB_OK) and never frees caller memory.
 * Complex data are interleaved (re, im) doubles (numpy complex128 /
 * torch.complex128 layout), row-major, unless stated otherwise.
 * Orbital conventions follow the reference: spin orbitals interleave alpha
 * (even index) and beta (odd index); ERIs are chemist (pq|rs) and
 * <pq||rs> = (pr|qs) - (ps|qr).  No entry point allocates device memory
 * except agb_cisd_plan_create (host memory for the plan object only);
 * device workspace is sized by the library and owned by the caller.
 * Mutable state lives in the caller's plan and workspace; what the library keeps
 * for the whole process is the last error message (one per host thread), an atomic
 * count of kernel launches (agb_launch_count, diagnostics), which kernels' attributes
 * were already set on which device, and the small device array of
 * agb_vec_dots_noalloc (see there).  A plan is used by one caller at a time.
 *
 * Reference cross-walk (apyib project paths):
 *   agb_zgemm / agb_cgemm_tf32x3   opt_einsum contractions of apyib/ci_wfn.py:309-334
 *   agb_zgemm_df64 / agb_zgemm_oz  the same contractions at FP64 accuracy off the FP64 pipe
 *                                  (double-float on the FP32 pipe; Ozaki-split bf16 tensor cores)
 *   agb_compute_f_so               apyib/utils.py:283-313 (compute_F_SO)
 *   agb_compute_eri_so             apyib/utils.py:317-365 (compute_ERI_SO)
 *   agb_cisd_blocks_*              the <pq||rs> block slices formed in apyib/ci_wfn.py:284,309-334
 *   agb_cisd_residual              apyib/ci_wfn.py:309-334 (CISD_SO) and :210-220 (CID_SO)
 *   agb_cisd_update                apyib/ci_wfn.py:336-337
 *   agb_vec_dots                   the DIIS Gram matrix, apyib/utils.py:121
 *   agb_cisd_combine               apyib/utils.py:138 + ci_wfn.py:355,361-365
 *   agb_mp2_so                     apyib/mp2_wfn.py:82-85 (solve_MP2_SO)
 *   agb_ao2mo                      apyib/utils.py:274-277 (compute_ERI_MO)
 *   agb_jk_fock[_sym[64]]          apyib/hf_wfn.py:81 and apyib/utils.py:241,249
 *   agb_ao_one_electron / _eri     psi4 MintsHelper integrals of apyib/hamiltonian.py:32-55
 *                                  (one-electron ones restated in apyib/integrals.py:9-146)
 */
#ifndef APYIB_GB300_H
#define APYIB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int agb_status;
#define AGB_OK 0
#define AGB_ERR_ARG 1          /* bad argument (shape, null pointer, size) */
#define AGB_ERR_CUDA 2         /* a CUDA runtime/driver call failed */
#define AGB_ERR_UNSUPPORTED 3  /* feature not available (e.g. not sm_103a) */
#define AGB_ERR_TIMEOUT 4      /* a bounded device-side wait ran out */
#define AGB_ERR_WORKSPACE 5    /* workspace missing or too small */

#define AGB_PREC_FP64 0        /* FP64 CUDA-core arithmetic */
#define AGB_PREC_TF32X3 1      /* complex FP32 via 3xTF32 tcgen05 MMAs, FP32 accumulate */
#define AGB_PREC_DF64 2        /* double-float (2 x FP32, ~48-bit) GEMMs on the FP32 pipe, FP64 elsewhere */
#define AGB_PREC_OZAKI 3       /* FP64-accurate GEMMs from six 7-bit bf16 slices per operand on the tcgen05
                                  tensor cores (exact FP32 group sums drained into int64), FP64 elsewhere */

/* Library version (major*10000 + minor*100 + patch). */
int agb_version(void);
/* Number of kernels this library has launched in this process (diagnostics;
 * no reference counterpart). */
unsigned long long agb_launch_count(void);
/* Last error message recorded by a failing call on this host thread. */
const char* agb_last_error(void);

/* ---------------------------------------------------------------- GEMMs -- */

/* C[m,n] = alpha * sum_k opA(m,k) * opB(k,n) + beta * C[m,n]
 * opA(m,k) = A[m*sAm + k*sAk] (conjugated if conjA), opB(k,n) = B[k*sBk + n*sBn]
 * (conjugated if conjB); strides in complex elements; C row-major with ldc.
 * Replaces the complex128 opt_einsum/zgemm contractions of apyib/ci_wfn.py:309-334. */
agb_status agb_zgemm(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im,
                     const void* A, int64_t sAm, int64_t sAk, int conjA,
                     const void* B, int64_t sBk, int64_t sBn, int conjB,
                     double beta_re, double beta_im, void* C, int64_t ldc, void* stream);

/* agb_zgemm with scratch for split-K partial sums: an output of fewer tiles than
 * the GPU has SMs (e.g. 24 x 24 from K = 24^3 in the back-transformed density
 * contractions) is computed by up to 256 K-slices whose partials are summed in
 * slice order (deterministic).  agb_zgemm_scratch_bytes(M,N,K) is the size that
 * allows every split the heuristic would choose; less scratch, fewer splits. */
size_t agb_zgemm_scratch_bytes(int64_t M, int64_t N, int64_t K);
agb_status agb_zgemm_ex(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im,
                        const void* A, int64_t sAm, int64_t sAk, int conjA,
                        const void* B, int64_t sBk, int64_t sBn, int conjB,
                        double beta_re, double beta_im, void* C, int64_t ldc,
                        void* scratch, size_t scratch_bytes, void* stream);

/* Same contraction in double-float arithmetic (each FP64 value split into two
 * floats, exact FMA product splitting, two-sum accumulation; ~2^-44 relative)
 * on the FP32 CUDA cores, which GB300 issues far faster than FP64. */
agb_status agb_zgemm_df64(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im,
                          const void* A, int64_t sAm, int64_t sAk, int conjA,
                          const void* B, int64_t sBk, int64_t sBn, int conjB,
                          double beta_re, double beta_im, void* C, int64_t ldc, void* stream);
/* With agb_zgemm_df64_scratch_bytes(M,N,K) bytes of scratch the operands are split
 * once and the complex products use three real products (faster path). */
size_t agb_zgemm_df64_scratch_bytes(int64_t M, int64_t N, int64_t K);
agb_status agb_zgemm_df64_ex(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im,
                             const void* A, int64_t sAm, int64_t sAk, int conjA,
                             const void* B, int64_t sBk, int64_t sBn, int conjB,
                             double beta_re, double beta_im, void* C, int64_t ldc,
                             void* scratch, size_t scratch_bytes, void* stream);
/* C = alpha op(A) op(B) + beta C (agb_zgemm's contract) to ~1e-12 of sum |a||b|:
 * each row of A and column of B is scaled by a power of two and cut into six
 * 7-bit digits stored as bf16 slices; the 21 slice products that carry 42 bits
 * run as tcgen05 kind::f16 MMAs whose low-order group sums stay exact in FP32
 * over K chunks and are drained into int64.  K <= 1024: one pass over Re and Im
 * (four real products sharing one exponent per row, 256-long chunks, C written
 * once); longer K: three real products (3M, 512-long chunks).  scratch:
 * agb_zgemm_oz_scratch_bytes(M, N, K), 256-byte aligned,
 * its first word the kernel's error word (agb_scratch_status).  Exponents of
 * A and B entries must stay within 2^+-500 of one another's row scales. */
size_t agb_zgemm_oz_scratch_bytes(int64_t M, int64_t N, int64_t K);
agb_status agb_zgemm_oz(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im,
                        const void* A, int64_t sAm, int64_t sAk, int conjA,
                        const void* B, int64_t sBk, int64_t sBn, int conjB,
                        double beta_re, double beta_im, void* C, int64_t ldc,
                        void* scratch, size_t scratch_bytes, void* stream);

/* Same contraction computed as complex FP32 with 3xTF32 split products on the
 * tcgen05 tensor cores (FP32 accumulation in TMEM), FP64 in and out.
 * scratch must hold agb_cgemm_tf32x3_scratch_bytes(M,N,K) bytes. */
size_t agb_cgemm_tf32x3_scratch_bytes(int64_t M, int64_t N, int64_t K);
agb_status agb_cgemm_tf32x3(int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im,
                            const void* A, int64_t sAm, int64_t sAk, int conjA,
                            const void* B, int64_t sBk, int64_t sBn, int conjB,
                            double beta_re, double beta_im, void* C, int64_t ldc,
                            void* scratch, size_t scratch_bytes, void* stream);

/* Batched products for the overlap-based AAT terms (apyib/aats.py:120-555 evaluates
 * each as a sum of o x o determinants; here they are a few small products per overlap):
 * C_b = alpha * op(A_b) op(B_b) + beta * C_b for b < batch, with agb_zgemm's strides plus
 * batch strides sAb, sBb, sCb in complex elements (0 broadcasts an operand).  FP64. */
agb_status agb_zgemm_batched(int64_t batch, int64_t M, int64_t N, int64_t K, double alpha_re, double alpha_im,
                             const void* A, int64_t sAm, int64_t sAk, int64_t sAb, int conjA,
                             const void* B, int64_t sBk, int64_t sBn, int64_t sBb, int conjB,
                             double beta_re, double beta_im, void* C, int64_t ldc, int64_t sCb, void* stream);
/* Determinant and inverse of each n x n complex matrix A_b (row-major, leading dimension
 * lda, batch stride sAb; 1 <= n <= 96) by Gauss-Jordan elimination with partial pivoting
 * in FP64: Ainv_b (ldi, sIb), det[b] (complex), info[b] = 0, or k + 1 when the pivot of
 * step k was exactly zero (outputs unspecified).  info may be NULL.  Replaces the
 * np.linalg.det / inv of the occupied overlap blocks (apyib/aats.py:120-131). */
agb_status agb_zdet_inv_batched(int64_t batch, int n, const void* A, int64_t lda, int64_t sAb, void* Ainv,
                                int64_t ldi, int64_t sIb, void* det, int* info, void* stream);


/* Reads and clears the status word a 3xTF32 GEMM keeps in the first bytes of its
 * scratch (zero it once before first use): AGB_ERR_TIMEOUT if a bounded
 * device-side wait ran out.  Synchronises the stream. */
agb_status agb_scratch_status(void* scratch, void* stream);

/* -------------------------------------------------- spin-orbital expansion -- */

/* F_SO[p,q] = F_MO[p/2,q/2] if p%2 == q%2 else 0; F_MO n x n, F_SO 2n x 2n.
 * Replaces apyib/utils.py:283-313 (compute_F_SO). */
agb_status agb_compute_f_so(const void* F_MO, int64_t n, void* F_SO, void* stream);
/* Chemist ERI_SO[p,q,r,s] = ERI_MO[p/2,q/2,r/2,s/2] if p%2==q%2 and r%2==s%2
 * else 0, for an n0 x n1 x n2 x n3 ERI_MO.  Replaces apyib/utils.py:317-365. */
agb_status agb_compute_eri_so(const void* ERI_MO, int64_t n0, int64_t n1, int64_t n2, int64_t n3,
                              void* ERI_SO, void* stream);

/* ------------------------------------------------------------- CISD plan -- */

typedef struct agb_cisd_plan agb_cisd_plan;

#define AGB_PLAN_MIXED 1       /* also keep 3xTF32-prepared operands (AGB_PREC_TF32X3 residuals) */
#define AGB_PLAN_NO_SINGLES 2  /* CID_SO: t1 == 0, no singles blocks */
#define AGB_PLAN_MP2 4         /* MP2_SO only: <ab||ij> and <ij||ab> blocks, no residual */

/* o, v: occupied / virtual spin orbitals (even, >= 2).  Host allocation only. */
agb_status agb_cisd_plan_create(int o, int v, int flags, agb_cisd_plan** plan);
agb_status agb_cisd_plan_destroy(agb_cisd_plan* plan);
/* Device workspace the plan needs; the caller allocates it (any allocator). */
agb_status agb_cisd_plan_workspace_bytes(const agb_cisd_plan* plan, size_t* bytes);
agb_status agb_cisd_plan_set_workspace(agb_cisd_plan* plan, void* workspace, size_t bytes);
/* Sizes of the packed amplitude vector [t1 (o*v) | t2 (o(o-1)/2 * v(v-1)/2)]. */
agb_status agb_cisd_plan_sizes(const agb_cisd_plan* plan, int64_t* n1, int64_t* n2);
/* Benchmark instrumentation kept by the plan (no reference counterpart): while on, each
 * tcgen05 GEMM launch of the plan's residuals is bracketed by CUDA events on its stream.
 * _collect synchronises the recorded events, reports the launch count, summed kernel
 * milliseconds and algorithmic flops (8*M*N*K) of the launches with M*N*K >= min_mnk,
 * and clears the record.  Like every plan call, not for concurrent use on one plan. */
agb_status agb_cisd_plan_gemm_timing(agb_cisd_plan* plan, int on);
agb_status agb_cisd_plan_gemm_timing_collect(agb_cisd_plan* plan, double min_mnk, int* launches, double* ms,
                                             double* flops);

/* Fock matrix (full spin-orbital F_SO, nso x nso) and SO orbital energies
 * eps_so (nso doubles, occupied first) used for the denominators
 * D_ia = e_i - e_a, D_ijab = e_i + e_j - e_a - e_b (apyib/ci_wfn.py:268-271). */
agb_status agb_cisd_set_fock(agb_cisd_plan* plan, const void* F_SO, const double* eps_so, void* stream);
/* (F_SO and eps_so are device pointers.) */

/* Build every antisymmetrised block the residual reads, from
 *  - a spatial-MO chemist tensor ERI_MO (nmo^4, nmo = (o+v)/2), applying the
 *    spin integration of apyib/utils.py:317-365 on the fly;
 *  - a full spin-orbital chemist tensor ERI_SO (nso^4);
 *  - Hermitian factors Bf[L,p,q] (naux x nso x nso): (pq|rs) = sum_L Bf[L,p,q] Bf[L,r,s].
 * 'scratch' (factors variant only) must hold agb_cisd_factor_scratch_bytes bytes. */
agb_status agb_cisd_blocks_from_mo(agb_cisd_plan* plan, const void* ERI_MO, void* stream);
agb_status agb_cisd_blocks_from_so(agb_cisd_plan* plan, const void* ERI_SO, void* stream);
size_t agb_cisd_factor_scratch_bytes(const agb_cisd_plan* plan, int64_t naux);
/* precision: AGB_PREC_FP64, AGB_PREC_DF64 for the factor products in double-float,
 * or AGB_PREC_OZAKI for them on the tensor cores (large products; the rest in
 * double-float).  Status of the tensor-core products: agb_cisd_status. */
agb_status agb_cisd_blocks_from_factors(agb_cisd_plan* plan, const void* Bf, int64_t naux,
                                        void* scratch, size_t scratch_bytes, int precision, void* stream);

#define AGB_RES_CONST 1        /* include the constant terms <ab||ij> and F_ai */
#define AGB_RES_ETERM 2        /* include -E * t */

/* Packed residual of apyib/ci_wfn.py:309-334: t = [t1 | t2p] and r = [r1 | r2p]
 * are packed amplitude vectors (t2p[p(i<j), p(a<b)] = t2[i,j,a,b]).
 * flags selects the constant and -E*t terms (both set for the reference residual;
 * neither for the linear part L(t) used by iterative refinement). */
agb_status agb_cisd_residual(agb_cisd_plan* plan, int precision, const void* t, double E_re, double E_im,
                             int flags, void* r, void* stream);

/* Status of the plan's device-side waits (AGB_ERR_TIMEOUT after a timed-out
 * tcgen05 GEMM); synchronises the stream. */
agb_status agb_cisd_status(agb_cisd_plan* plan, void* stream);

/* t_out = t + r / D (apyib/ci_wfn.py:336-337) on packed vectors. */
agb_status agb_cisd_update(agb_cisd_plan* plan, const void* t, const void* r, void* t_out, void* stream);

/* out[j] = w1 * sum_{k<n1} conj(y_j[k]) x[k] + w2 * sum_{k>=n1} conj(y_j[k]) x[k], j < ny <= 16.
 * (DIIS Gram row, apyib/utils.py:121, with w2 = 4 for packed doubles.)  The first part
 * is summed by a single thread block (it is sized for the singles, n1 = o v): pass a long
 * vector as the second part.  Products and sums run in double-float (~2^-44 relative):
 * entries must satisfy |re|, |im| < 2^128, and an entry at or above it (or inf / NaN)
 * makes the affected results non-finite; parts below 2^-112 in magnitude are dropped. */
agb_status agb_vec_dots(int64_t n1, int64_t n2, double w1, double w2, const void* x,
                        const void* const* ys, int ny, void* out, void* partials, size_t partials_bytes,
                        void* stream);
/* Bytes of the partials buffer agb_vec_dots needs for ny vectors (each of its
 * blocks stores the full slot width of the kernel instance serving ny: 4, 8, 12
 * or 16); agb_cisd_combine needs agb_vec_partials_bytes(3). */
size_t agb_vec_partials_bytes(int ny);

/* agb_vec_dots without the caller-provided partials buffer.  No counterpart in
 * the reference (which has no device code at all); it exists for callers that
 * cannot allocate device memory themselves, e.g. a plugin whose host
 * application owns every device allocation through its own pool and hands out
 * only the vectors, or a latency-bound loop in which an allocation call (and
 * the synchronisation it may imply) is not allowed.
 * The block partial sums live in a fixed array inside the library (155,648
 * bytes on every device that loads it, kept until the process exits), so this
 * entry point allocates nothing and accepts at most ny = 16 vectors; larger ny
 * is rejected with AGB_ERR_ARG.  The array's device address belongs to one CUDA
 * context: the first call in each context (the device's primary context, or a
 * caller's own context made current) looks it up with that context current and
 * caches it under the context's unique id, so a context destroyed and recreated
 * (cudaDeviceReset) gets a fresh lookup; make that first call before any stream
 * capture.  All calls on a device share the one array and
 * each call leaves its partial sums there; calls that overlap on the GPU (for
 * example on two streams at once) race on it, so the caller must keep them
 * from overlapping. */
agb_status agb_vec_dots_noalloc(int64_t n1, int64_t n2, double w1, double w2, const void* x,
                                const void* const* ys, int ny, void* out, void* stream);

/* t_new = sum_j c_j y_j (apyib/utils.py:138; ny <= 16; ny = 1, c = 1 copies),
 * fused with the energy E = sum_ia t1*F_ov + sum_p t2p*<ij||ab>_p (ci_wfn.py:355) and the
 * unconjugated squared norms s1 = sum (t1_old - t1_new)^2, s2 = 4 sum (t2p_old - t2p_new)^2
 * (ci_wfn.py:361-365).  out3 receives (E, s1, s2) as three complex doubles.
 * t_old may alias t_new (read before write per element). */
agb_status agb_cisd_combine(agb_cisd_plan* plan, const void* const* ys, const double* coefs, int ny,
                            const void* t_old, void* t_new, void* out3, void* partials,
                            size_t partials_bytes, void* stream);

/* Unpack a packed amplitude vector into t1[o,v] and the full antisymmetric t2[o,o,v,v]. */
agb_status agb_cisd_unpack(agb_cisd_plan* plan, const void* t, void* t1, void* t2, void* stream);
/* Pack t1[o,v], t2[o,o,v,v] into a packed amplitude vector. */
agb_status agb_cisd_pack(agb_cisd_plan* plan, const void* t1, const void* t2, void* t, void* stream);
/* Initial guesses t1 = F_ai/D_ia, t2p = <ab||ij>/D (apyib/ci_wfn.py:287-290). */
agb_status agb_cisd_guess(agb_cisd_plan* plan, void* t, void* stream);

/* ------------------------------------------------------------------- MP2 -- */

/* MP2_SO from a built plan: t2p = <ab||ij>/D, E = sum_p <ij||ab>_p t2p
 * (apyib/mp2_wfn.py:82-85); t receives the packed vector (t1 part zero).
 * partials: device scratch of at least agb_vec_partials_bytes(1) bytes. */
agb_status agb_mp2_so(agb_cisd_plan* plan, void* t, void* E_out, void* partials, size_t partials_bytes,
                      void* stream);

/* Closed-shell MP2 over complex spatial orbitals (apyib/mp2_wfn.py:42-59):
 * t2[i,j,a,b] = <ab|ij>/D_ijab, E = sum (2<ij|ab> - <ij|ba>) t2, from the active
 * chemist ERI_MO (nmo^4, first no orbitals occupied) and eps (nmo doubles, device).
 * t2 receives no*no*nv*nv complex values; E_out one complex (device). */
agb_status agb_mp2_spatial(const void* ERI_MO, int64_t nmo, int64_t no, const double* eps, void* t2,
                           void* E_out, void* partials, size_t partials_bytes, void* stream);

/* ------------------------------------------------------ AO -> MO, J/K -- */

/* ERI_MO[p,q,r,s] = sum C*[m,p] C[n,q] C*[l,r] C[s',s] (mn|ls') for real AO ERIs
 * (nbf^4 doubles) and complex C (nbf x nmo), four quarter steps
 * (apyib/utils.py:274-277).  precision: AGB_PREC_FP64 (FP64 pipe),
 * AGB_PREC_DF64 (double-float GEMMs, ~1e-13 relative), AGB_PREC_OZAKI (FP64-
 * accurate bf16-slice GEMMs on the tensor cores, ~1e-12 of sum |a||b|) or
 * AGB_PREC_TF32X3 (tensor cores, ~1e-6 relative).  scratch:
 * agb_ao2mo_scratch_bytes for the same precision. */
size_t agb_ao2mo_scratch_bytes(int64_t nbf, int64_t nmo, int precision);
agb_status agb_ao2mo(const double* ERI_AO, int64_t nbf, const void* C, int64_t nmo, void* ERI_MO,
                     void* scratch, size_t scratch_bytes, int precision, void* stream);

/* F = h + scale * sum_ls D[l,s] (2 (mn|ls) - (ml|ns)) with real AO ERIs and
 * complex D, h (may be NULL: zero), F (nbf x nbf).  One pass over the ERIs for
 * J and K, products and sums in double-float arithmetic (~1e-14 relative);
 * deterministic.  apyib/hf_wfn.py:81 (scale 0.5) and apyib/utils.py:241,249
 * (scale 1).  scratch: agb_jk_fock_scratch_bytes(nbf) (the split density). */
size_t agb_jk_fock_scratch_bytes(int64_t nbf);
agb_status agb_jk_fock(const double* ERI_AO, int64_t nbf, const void* D, const void* h, double scale,
                       void* F, void* scratch, size_t scratch_bytes, void* stream);
/* agb_jk_fock for ERIs symmetric in their last index pair, (mn|ls) = (mn|sl), as real
 * AO integrals and their nuclear derivatives are (the caller guarantees it): only
 * l <= s is read, each integral serving J, K[l] and K[s]; same scratch. */
agb_status agb_jk_fock_sym(const double* ERI_AO, int64_t nbf, const void* D, const void* h, double scale,
                           void* F, void* scratch, size_t scratch_bytes, void* stream);
/* agb_jk_fock_sym in FP64 arithmetic (six DFMAs per pair of integrals; the precision
 * of the reference's einsum, for finite differences of energies); same scratch. */
agb_status agb_jk_fock_sym64(const double* ERI_AO, int64_t nbf, const void* D, const void* h, double scale,
                             void* F, void* scratch, size_t scratch_bytes, void* stream);

/* ------------------------------------------------------ AO integrals -- */

/* A contracted Gaussian basis on a molecule.  Every array is device memory.
 * Cartesian functions of a shell of angular momentum l are ordered
 * for i in 0..l, for j in 0..i: x^(l-i) y^(i-j) z^j, and coefs carry the
 * primitive normalisation (apyib/integrals.py:107-119 reads psi4's shells the
 * same way).  Shells have l <= 3 (lmax is checked). */
typedef struct agb_basis {
  int natom;
  int nshell;
  int ncart;                 /* Cartesian functions */
  int lmax;                  /* largest shell angular momentum */
  const double* atom_xyz;    /* [natom][3], bohr */
  const double* atom_charge; /* [natom] nuclear charges */
  const int* shell_l;        /* [nshell] */
  const int* shell_atom;     /* [nshell] centre of each shell */
  const int* shell_nprim;    /* [nshell] */
  const int* shell_prim0;    /* [nshell] first primitive in exps / coefs */
  const int* shell_cart0;    /* [nshell] first Cartesian function */
  const int* bf_shell;       /* [ncart] shell of each Cartesian function */
  const double* exps;        /* primitive exponents */
  const double* coefs;       /* normalised contraction coefficients */
} agb_basis;

#define AGB_OEI_OVERLAP 0    /* S                       1 component  */
#define AGB_OEI_KINETIC 1    /* -1/2 nabla^2            1 component  */
#define AGB_OEI_POTENTIAL 2  /* -sum_C Z_C / |r - C|    1 component  */
#define AGB_OEI_DIPOLE 3     /* -(r - O)                3 components (electron charge included) */
#define AGB_OEI_NABLA 4      /* d/dr acting on the ket  3 components */
#define AGB_OEI_ANGMOM 5     /* -(r - O) x nabla        3 components */
#define AGB_OEI_OVERLAP_HALF 6  /* <d mu / dR | nu>: derivative of the bra function only
                                   (agb_ao_one_electron_deriv only) */

/* One-electron integrals over the Cartesian functions, out[comp][ncart][ncart]
 * (FP64).  origin (host, 3 doubles; NULL = 0) is the origin O of the dipole and
 * angular-momentum operators.  psi4's MintsHelper ao_overlap / ao_kinetic /
 * ao_potential / ao_dipole / ao_nabla / ao_angular_momentum
 * (apyib/hamiltonian.py:32-55), restated by apyib/integrals.py:9-146. */
agb_status agb_ao_one_electron(const agb_basis* basis, int kind, const double* origin, double* out,
                               void* stream);

/* Electron-repulsion integrals (mn|ls) over the Cartesian functions, chemist
 * order, all ncart^4 values (FP64).  psi4's MintsHelper ao_eri
 * (apyib/hamiltonian.py:34). */
agb_status agb_ao_eri(const agb_basis* basis, double* out, void* stream);

/* Nuclear first derivatives over the Cartesian functions, out[atom][x,y,z][ncart][ncart]
 * (zeroed by the call) for kind AGB_OEI_OVERLAP, AGB_OEI_KINETIC, AGB_OEI_POTENTIAL
 * (basis-function centres and the attracting nucleus both move) or
 * AGB_OEI_OVERLAP_HALF; out[atom][x,y,z][component][ncart][ncart] for AGB_OEI_DIPOLE
 * (origin 0).  psi4's MintsHelper ao_oei_deriv1 / ao_overlap_half_deriv1
 * (apyib/analytic_aats.py:96-104). */
agb_status agb_ao_one_electron_deriv(const agb_basis* basis, int kind, double* out, void* stream);

/* Nuclear first derivatives of the ERIs, out[atom][x,y,z][ncart^4] (chemist order,
 * zeroed by the call).  psi4's MintsHelper ao_tei_deriv1 (apyib/analytic_aats.py:100). */
agb_status agb_ao_eri_deriv(const agb_basis* basis, double* out, void* stream);

/* Basis change along one axis: out[a][s][b] = sum_k coef[s][k] in[a][cart0[s] + k][b]
 * for a < pre, s < nout, k < len[s] (<= 16), b < post; in has nin functions on the
 * axis.  Takes Cartesian functions to pure (solid-harmonic) ones. */
agb_status agb_ao_transform_axis(const double* in, int64_t pre, int nin, int64_t post, int nout,
                                 const int* cart0, const int* len, const double* coef, double* out,
                                 void* stream);

#ifdef __cplusplus
}
#endif
#endif /* APYIB_GB300_H */

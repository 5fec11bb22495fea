/*
 * gdfjk.h — C ABI of the GB300 density-fitted J/K engine (libgdfjk.so).
 *
 * The engine replaces the JK half of psi4's in-core DF path: MemDFJK::compute_JK
 * (psi4/src/psi4/libfock/MemDFJK.cc:97-111) -> DFHelper::build_JK / compute_JK /
 * compute_J_symm / compute_K (psi4/src/psi4/lib3index/dfhelper.cc:3015-3377).  The
 * metric-contracted 3-index tensor B[Q][mn] = sum_P J^-1/2_QP (P|mn) is built as
 * DFHelper::prepare_AO_core builds it (dfhelper.cc:514-588), either on the host and uploaded
 * to HBM once, or on the device from its own raw integrals and metric contraction, and
 * every Fock build then runs on the GPU.
 *
 * Conventions: row-major FP64 host/device matrices; every call returns an int status
 * (GDFJK_OK = 0, negative on error) and gdfjk_last_error(h) gives the message (h may be
 * NULL for errors before a handle exists).  One CUDA stream per handle; calls that take
 * host buffers are synchronous, calls with the _device suffix are asynchronous on the
 * handle's stream.  (A build may run its J passes on a second, internal stream beside the
 * tensor-core K; that stream is joined back into the handle's stream before the build's
 * last operation, so the handle's stream still orders everything a caller sees.)  A handle
 * is not re-entrant (like psi4's JK objects, jk.h:232).
 */
#ifndef GDFJK_H
#define GDFJK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gdfjk_s* gdfjk_t;

enum {
    GDFJK_OK = 0,
    GDFJK_ERR_ARG = -1,      /* invalid argument (sizes, null pointers, layout)        */
    GDFJK_ERR_CUDA = -2,     /* CUDA runtime/driver error                              */
    GDFJK_ERR_OOM = -3,      /* device allocation refused                              */
    GDFJK_ERR_STATE = -4,    /* call out of order (e.g. compute before upload_B)       */
    GDFJK_ERR_TIMEOUT = -5,  /* the stream did not finish within the host watchdog     */
    GDFJK_ERR_NUMERIC = -6,  /* non-finite values found in J or K                      */
    GDFJK_ERR_DEVICE = -7    /* a kernel reported an internal error through its flag   */
};

/* B layouts accepted by gdfjk_upload_B */
enum {
    GDFJK_LAYOUT_PQQ = 0,  /* DFHelper in-core pQq: B[big_skips[m] + Q*small_skips[m] + fun_index[m*nbf+n]-1]
                              (dfhelper.cc:1671-1673); needs big_skips/small_skips/fun_index     */
    GDFJK_LAYOUT_QTRI = 1  /* Q-major packed lower triangle: B[Q*nbf(nbf+1)/2 + m(m+1)/2 + n], m >= n */
};

/* compute mode bits */
enum {
    GDFJK_DO_J = 1,
    GDFJK_DO_K = 2,
    GDFJK_MIXED = 4,       /* K as a split-BF16 tensor-core product with FP32 accumulation      */
    GDFJK_INCREMENTAL = 8, /* K += K(dD) against the previous build's density (mixed form only)  */
    GDFJK_RESET = 16,      /* forget the incremental history (next build is a full build)      */
    GDFJK_EMULATED = 32    /* K to FP64 accuracy from BF16 tensor-core products of 7-bit digit
                              slices (Ozaki splitting, exact FP32 level sums, double-float
                              epilogue); lr-symmetric or C_left != C_right, nocc <= 1024;
                              ignored with GDFJK_MIXED                                         */
};

/* gdfjk_create flags */
enum {
    GDFJK_B_HOST = 256  /* keep the FP64 tiles of B in pinned host (Grace) memory mapped into
                           the GPU's address space; the kernels read them over NVLink-C2C.
                           For systems whose B does not fit in HBM (psi4's out-of-core
                           DFHelper, grab_AO, dfhelper.cc:1419-1432); results are identical.
                           The tensor-core forms' derived copies of B stay in HBM (they are
                           streamed with bulk copies); where they do not fit, those forms
                           return GDFJK_ERR_OOM and the native FP64 form still runs       */
};

/* Create an engine on CUDA device `device` for nbf basis functions and naux fitting
 * functions.  pair_mask (nbf*nbf bytes, symmetric, nullable = every pair significant)
 * is DFHelper's Schwarz function mask (schwarz_fun_index_ != 0, dfhelper.cc:375-386).
 * flags: 0 or GDFJK_B_HOST. */
int gdfjk_create(int device, int nbf, int naux, const unsigned char* pair_mask, int flags, gdfjk_t* out);

/* Upload B from host memory, once (MemDFJK::preiterations -> DFHelper::initialize,
 * MemDFJK.cc:71-96).  For GDFJK_LAYOUT_PQQ pass big_skips (nbf+1), small_skips (nbf+1)
 * and fun_index (nbf*nbf) exactly as DFHelper::prepare_sparsity builds them
 * (dfhelper.cc:368-397); for GDFJK_LAYOUT_QTRI pass NULL for all three. */
int gdfjk_upload_B(gdfjk_t h, const double* B, int layout, const int64_t* big_skips, const int64_t* small_skips,
                   const int64_t* fun_index);

/* Same with B already on the device (Q-major packed lower triangle, naux*nbf(nbf+1)/2). */
int gdfjk_upload_B_device(gdfjk_t h, const double* B_qtri_device);

/* Upload B in blocks of aux functions, the way DFHelper builds it block by block
 * (DFHelper::prepare_AO_core -> compute_sparse_pQq_blocking_p over Q-shell blocks,
 * dfhelper.cc:514-588): rows q0 .. q0+nq-1 of the Q-major packed lower triangle
 * (nq * nbf(nbf+1)/2 doubles; screened pairs must be zero, as DFHelper's sparse tensor
 * holds no entry for them).
 * Blocks go in order of q0 starting at 0; the engine is ready for compute once the block
 * that ends at naux has been uploaded.  Neither call keeps the pointer. */
int gdfjk_upload_B_block(gdfjk_t h, const double* B_qtri_rows, int q0, int nq);
int gdfjk_upload_B_device_block(gdfjk_t h, const double* B_qtri_rows_device, int q0, int nq);

/* ---- The raw integrals on the device (DFHelper::prepare_AO_core's integral step,
 * dfhelper.cc:514-588: compute_sparse_pQq_blocking_p_symm, :1284-1347, with libint2's
 * 3-index ERIs; the metric of FittingMetric::form_fitting_metric, fittingmetric.cc:72).
 * McMurchie-Davidson per shell triplet on the FP64 pipes; primary shells up to f, fitting
 * shells up to g; both bases pure (psi4's default for the cc-pVXZ families) or both
 * Cartesian.  Component order and normalisation are those of the host provider (gdfints). */
typedef struct gdfjk_basis_s* gdfjk_basis_t;

/* A basis set copied to CUDA device `device`: nshell shells with angular momentum l[s],
 * nprim[s] primitives exps/coefs[prim_offset[s] ...] (raw contraction coefficients, normalised
 * here as psi4 normalises them), centres xyz[3*s..] in bohr, atom[s] the atom of the shell's
 * centre (nullable; needed by the gradient entries); puream != 0: solid harmonics. */
int gdfjk_basis_create(int device, int nshell, const int* l, const int* nprim, const int* prim_offset,
                       const double* exps, const double* coefs, const double* xyz, const int* atom, int puream,
                       gdfjk_basis_t* out);
void gdfjk_basis_destroy(gdfjk_basis_t b);
int gdfjk_basis_nbf(gdfjk_basis_t b);

/* (P|mn) for fitting functions p0 <= P < p1 and the primary shell pairs M >= N with
 * shell_mask[M*nshell + N] != 0 (host, nullable = every pair; DFHelper's Schwarz shell mask,
 * dfhelper.cc:336-366), written into the device array out, row P - p0 at out + (P - p0)*ldo:
 * column m(m+1)/2 + n (m >= n) when col_map is NULL (ldo >= nbf(nbf+1)/2), else column
 * col_map[m(m+1)/2 + n] (a device array of nbf(nbf+1)/2 entries; < 0 = not stored).  Entries
 * of unlisted pairs are not written (zero the array first).  Runs on `stream` (a
 * cudaStream_t, NULL = the default stream) and returns when the integrals are complete. */
int gdfjk_three_index_device(gdfjk_basis_t aux, gdfjk_basis_t prim, const unsigned char* shell_mask, int p0, int p1,
                             const int64_t* col_map, int64_t ldo, double* out, void* stream);

/* The Coulomb metric (P|Q), rows p0 <= P < p1 at out + (P - p0)*ldo, all naux columns. */
int gdfjk_metric_device(gdfjk_basis_t aux, int p0, int p1, int64_t ldo, double* out, void* stream);

/* The gradient's derivative-integral contractions on the device (DFJKGrad::build_Amn_x_terms,
 * jk_grad.cc:868-1245; MintsHelper::metric_grad, mintshelper.cc:2388), added into the device
 * array grad[natom][3]:
 *   three_index_grad: sum over P and the listed shell pairs of G3[P][col(m,n)] d(P|mn)/dx,
 *       G3 a device array laid out as gdfjk_three_index_device's output (all naux rows,
 *       leading dimension ldg, packed-triangle columns or col_map), off-diagonal mn entries
 *       carrying the weight of both (mn) and (nm);
 *   metric_grad: sum over P, Q of G2[P][Q] d(P|Q)/dx, G2 symmetric, naux x naux, ldg >= naux.
 * Both bases need atom indices.  Summed with atomics (the order of the additions is not
 * fixed; results agree to rounding).  Return when complete. */
int gdfjk_three_index_grad_device(gdfjk_basis_t aux, gdfjk_basis_t prim, const unsigned char* shell_mask,
                                  const double* G3, const int64_t* col_map, int64_t ldg, int natom, double* grad,
                                  void* stream);
int gdfjk_metric_grad_device(gdfjk_basis_t aux, const double* G2, int64_t ldg, int natom, double* grad, void* stream);

/* The nuclear-attraction part of the one-electron gradient (psi4's potential derivative
 * integrals contracted with the density, scf_grad.cc:196-220): grad[natom][3] (device,
 * accumulated) += sum over m >= n of Dp[m(m+1)/2+n] d(V_mn)/dx, V_mn = -sum_C Z_C (m|1/r_C|n),
 * Dp a device packed triangle with the off-diagonal entries doubled (so that the sum is
 * sum_mn D_mn dV_mn for a symmetric D); Z and xyz (bohr) host arrays of natom charges and
 * positions.  The same derivative class kernels with point charges for the fitting shells. */
int gdfjk_potential_grad_device(gdfjk_basis_t prim, const double* Dp, int natom, const double* Z, const double* xyz,
                                double* grad, void* stream);

/* The metric contraction B = J^-1/2 (P|mn) on the tensor cores, to FP64 accuracy (the
 * emulated-FP64 digit products of GDFJK_EMULATED): replaces the naux x naux DGEMM of
 * DFHelper::contract_metric_AO_core_symm (dfhelper.cc:1653-1678) called from
 * DFHelper::prepare_AO_core (dfhelper.cc:514-588).  All device buffers, row-major:
 *   metric  naux x naux (e.g. J^-1/2 from Matrix::power(-0.5, condition), matrix.cc:2370-2415)
 *   Pmn     naux x ncols, leading dimension ldp >= ncols (the raw 3-index integrals; with
 *           ncols = nbf(nbf+1)/2 in GDFJK_LAYOUT_QTRI order, B comes out ready for
 *           gdfjk_upload_B_device)
 *   B       naux x ncols, leading dimension ldb >= ncols: B = metric Pmn, or B += metric Pmn
 *           with accumulate != 0 (B must not overlap Pmn)
 * Runs on the handle's stream with temporary device buffers (the digits of the metric and of
 * one column chunk of Pmn, GDFJK_OZ_GEMM_CHUNK_GB, default 8 GB) and returns when B is
 * complete.  The handle's B is not touched. */
int gdfjk_metric_contract_device(gdfjk_t h, const double* metric, const double* Pmn, int ncols, int64_t ldp, double* B,
                                 int64_t ldb, int accumulate);

/* The same digit product as a general matrix product, for the gradient's contractions with the
 * metric (DFJKGrad's (A|B)^-1/2 applications and the 2-index density, jk_grad.cc:634-832):
 *   C (+)= A op(B),  A M x K (lda), op(B) = B (K x N, ldb) for transb = 0 or B^T (B N x K,
 *   ldb) for transb != 0, C M x N (ldc); all row-major device buffers, C must not overlap A
 *   or B.  Runs on the handle's stream with temporary device buffers (the digits of A and of
 *   one column chunk of op(B)) and returns when C is complete. */
int gdfjk_gemm_device(gdfjk_t h, int transb, int M, int N, int K, const double* A, int64_t lda, const double* B,
                      int64_t ldb, double* C, int64_t ldc, int accumulate);

/* One Fock build, host buffers (JK::compute, jk.cc:595-681, for one density):
 *   C_left  nbf x nocc (row-major, leading dimension ldc >= nocc)
 *   C_right nbf x nocc or NULL (NULL = lr-symmetric: D = C_left C_left^T, jk.cc:597-599)
 *   D_out   nbf x nbf or NULL: receives D = C_left C_right^T (JK::compute_D, jk.cc:314-354)
 *   J, K    nbf x nbf outputs (overwritten, like MemDFJK::compute_JK's zero() + build)
 * nocc = 0 gives K = 0 (dfhelper.cc:3355).  mode: GDFJK_DO_J | GDFJK_DO_K [| GDFJK_MIXED ...] */
int gdfjk_compute(gdfjk_t h, const double* C_left, const double* C_right, int nocc, int ldc, int mode, double* D_out,
                  double* J, double* K);

/* Same with device buffers, asynchronous on the handle's stream. */
int gdfjk_compute_device(gdfjk_t h, const double* C_left, const double* C_right, int nocc, int ldc, int mode,
                         double* D_out, double* J, double* K);

/* Long-range exchange for range-separated functionals (DFHelper::compute_wK, dfhelper.cc:3378-3438,
 * with the tensors of DFHelper::prepare_AO_wK_core, dfhelper.cc:589-699):
 *   wK = sum_Q (L_Q C_left)(R_Q C_right)^T,  L = J^-1 (Q|mn) on h_left, R = (Q|erf(w r)/r|mn) on
 *   h_right (each uploaded into its own handle like B; both handles on one device, same nbf,
 *   naux and pair mask).  C_right = NULL: lr-symmetric, and wK is symmetrised as
 *   MemDFJK::compute_JK does (MemDFJK.cc:103-108).  mode: 0 (native FP64) or GDFJK_EMULATED.
 *   Host buffers; uses h_left's stream and workspaces. */
int gdfjk_compute_wK(gdfjk_t h_left, gdfjk_t h_right, const double* C_left, const double* C_right, int nocc, int ldc,
                     int mode, double* wK);

/* The precision form's incremental build (psi4's INCFOCK idea, DirectJK.cc:138-166, applied
 * to MemDFJK's exchange): J in FP64 from C (as gdfjk_compute), and
 *   K = K_prev + sum_Q B_Q (U+ U+^T - U- U-^T) B_Q
 * as a split-BF16 tensor-core product with FP32 accumulation, where U (nbf x nu, leading
 * dimension ldu) holds npos positive columns then nu - npos negative ones, a signed factor
 * of dD = D - D_prev.  K_prev is the K this handle returned last (kept on the device in
 * FP64); GDFJK_RESET in mode takes K_prev = 0, i.e. a full build from the factor.
 * Without GDFJK_MIXED in mode, K is instead a full FP64 build from C (U is ignored) and
 * becomes the base K_prev of the following increments (an FP64 re-anchor). */
int gdfjk_compute_incremental(gdfjk_t h, const double* C, int nocc, int ldc, const double* U, int nu, int npos, int ldu,
                              int mode, double* J, double* K);

/* Same with device buffers (C, U, J, K), asynchronous on the handle's stream: a caller can
 * enqueue J from the new orbitals first (mode GDFJK_DO_J), form the factor U of dD on the host
 * meanwhile, and then enqueue the K increment (mode GDFJK_DO_K | GDFJK_MIXED). */
int gdfjk_compute_incremental_device(gdfjk_t h, const double* C, int nocc, int ldc, const double* U, int nu, int npos,
                                     int ldu, int mode, double* J, double* K);

/* Reverse-mode derivative of one lr-symmetric build (the differentiation form):
 * given upstream gradients gJ = dE/dJ and gK = dE/dK (nbf x nbf, device or host per
 * `on_device`), returns
 *   dC     (nbf x nocc)  dE/dC_left through D = C C^T (J) and K = sum_Q (B_Q C)(B_Q C)^T,
 *   Gamma  (naux x nbf(nbf+1)/2, Q-major packed, off-diagonal entries carry both (mn),(nm))
 *          dE/dB_Q,mn, the 3-index density contracted later with derivative integrals.
 * Either output may be NULL.  (Q|mi) is recomputed, not stored. */
/* Gamma = dE/dB of gdfjk_backward alone, for systems whose full-size backward workspaces do
 * not fit (the C100H202 gradient): device C, gJ, gK; the aux functions are taken in batches of
 * batch_q (0: as many as fit GDFJK_BW_BATCH_GB, default 16 GB, of X_b and Y_b), X_b = B_b C
 * recomputed per batch ((Q|mi) never stored whole), Y_b = gK X_b and Y_Q C^T (the dense part of
 * Gamma, GDFJK_BW_GAMMA_GB, default 8 GB, of it at a time) on the tensor cores to FP64
 * accuracy (the digit product of gdfjk_gemm_device), and Gamma written into the device array
 * Gamma (naux rows, leading dimension ldg; packed-triangle columns, or col_map[m(m+1)/2+n],
 * < 0 = not stored; cleared first).  Returns when complete. */
int gdfjk_backward_gamma_device(gdfjk_t h, const double* C, int nocc, int ldc, const double* gJ, const double* gK,
                                const int64_t* col_map, int64_t ldg, double* Gamma, int batch_q);

int gdfjk_backward(gdfjk_t h, const double* C, int nocc, int ldc, const double* gJ, const double* gK, double* dC,
                   double* Gamma, int on_device);

/* Release the derived copies of B that the tensor-core forms keep (split BF16 slices, int8
 * digits) and their X buffers; they are rebuilt on the next build that needs them.  No
 * counterpart in the reference (psi4's JK keeps no such copies): for callers that need the
 * device memory back between phases. */
int gdfjk_trim(gdfjk_t h);

/* Device bytes the engine needs for these sizes (feeds JK::memory_estimate, jk.h:398);
 * flags: mode bits of the forms in use, plus GDFJK_B_HOST (B then not counted). */
int gdfjk_query_memory(int nbf, int naux, int max_nocc, int flags, size_t* bytes);

/* Timing of the last build in milliseconds (J passes, K half-transform, K contraction).  When
 * the J passes ran on the internal second stream beside K, j_ms is their span there, which
 * then covers most of K's time rather than J's own. */
int gdfjk_last_timings(gdfjk_t h, double* j_ms, double* k_transform_ms, double* k_contract_ms);

/* Host watchdog: wait for the stream at most timeout_s seconds (GDFJK_ERR_TIMEOUT after). */
int gdfjk_synchronize(gdfjk_t h, double timeout_s);

/* The CUDA stream of the handle (cudaStream_t as void*). */
void* gdfjk_stream(gdfjk_t h);

/* Coulomb build that allocates nothing (no counterpart in the reference: psi4's JK objects
 * always own their buffers).  For callers that cannot call cudaMalloc — code running under
 * another framework's memory pool or allocator hooks, hosts that forbid allocation after
 * start-up, drivers that fix their buffers once.  Runs on the calling thread's current
 * device, asynchronously on `stream` (a cudaStream_t, NULL = legacy default stream):
 *   B  device, Q-major packed lower triangle, naux x nbf(nbf+1)/2 (GDFJK_LAYOUT_QTRI)
 *   D  device, nbf x nbf density (symmetrised internally)
 *   J  device, nbf x nbf output, overwritten with J_mn = sum_Q B_Q,mn sum_ls B_Q,ls D_ls
 * The fitted density d_Q is kept in a fixed file-scope device array of
 * GDFJK_NOALLOC_MAX_NAUX doubles (512 KB) that every GPU loading the library holds until
 * exit; naux above that limit is rejected with GDFJK_ERR_ARG.  Every call looks up the
 * array's device address in the calling thread's current CUDA context (cudaGetSymbolAddress,
 * which allocates nothing); the first call in a context may load the module, so make that
 * first call before any stream capture.  All calls share the array and each overwrites it
 * completely before reading it; calls whose work overlaps on the GPU race on it.
 * Errors: gdfjk_last_error(NULL). */
#define GDFJK_NOALLOC_MAX_NAUX 65536
int gdfjk_coulomb_noalloc(int nbf, int naux, const double* B, const double* D, double* J, void* stream);

/* Host-side fault injection for the failure tests (no counterpart in the reference, whose
 * failures are PSIEXCEPTIONs from the allocator and the integral code):
 *   gdfjk_debug_refuse_allocations(after, count)  of the device (and pinned host)
 *       allocations the engine makes from now on, the first `after` go through and the next
 *       `count` are refused as out of memory, exactly as a full device refuses them, so the
 *       GDFJK_ERR_OOM paths (release the other form's copy of B and retry once) run;
 *       count = 0 ends the injection.  Process-wide.  Returns the number of refusals of
 *       the previous setting that were still pending (>= 0), or GDFJK_ERR_ARG.
 *   gdfjk_debug_wait_probe(h, limit_s)  runs the tensor-core kernels' bounded mbarrier wait on
 *       a barrier that nothing arrives on, with the limit limit_s (0 < limit_s <= 10) instead
 *       of the production 2 s: the kernel gives up, raises its wait error bit and returns, and
 *       the call returns GDFJK_ERR_DEVICE; the handle stays usable. */
int gdfjk_debug_refuse_allocations(int after, int count);
int gdfjk_debug_wait_probe(gdfjk_t h, double limit_s);

int gdfjk_destroy(gdfjk_t h);
const char* gdfjk_last_error(gdfjk_t h);

#ifdef __cplusplus
}
#endif
#endif

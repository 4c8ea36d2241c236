/*
 * fasterlmm_gb300 -- C ABI of the GB300 (sm_103a) batched LMM association scan.
 *
 * Every entry point takes caller-owned DEVICE pointers, plain sizes and leading dimensions, a CUDA stream passed as
 * `void*` (NULL = legacy default stream), and returns an int status (FLMM_OK = 0).  Launches are asynchronous on
 * that stream unless stated otherwise; an entry point never synchronises the device.  Scratch memory is passed in
 * by the caller (`work`, `work_bytes`), sized by the matching *_workspace_bytes query.  No entry point allocates
 * except flmm_context_create.
 *
 * Matrix layouts (row-major, element (i, j) at ptr[i * ld + j]):
 *   Zt    (M, N)     standardised variants, variant-major: row m = one variant's N samples
 *   Yt    (P, N)     phenotype columns, column-major in the reference's terms: row p = one column's N samples
 *   Ut    (Neff, N)  kept eigenvectors, one per row (the transpose of the reference's U_eff)
 *   UYt   (P, Neff)  rotated phenotypes (transpose of the reference's UY)
 *   USt   (Mc, Neff) rotated variants of one chromosome (transpose of the reference's US)
 *   out   (M, B)     per-variant detail of the B real columns, variant-major like the reference's ScanResult
 *
 * The interface replaces the Python functions of the reference's scan path (paths inside the reference project);
 * each declaration cites the function whose work it does.
 */
#ifndef FASTERLMM_GB300_H
#define FASTERLMM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ----------------------------------------------------------------------------------------- */
#define FLMM_OK 0
#define FLMM_ERR_ARG 1          /* null pointer, bad size, bad leading dimension or misalignment */
#define FLMM_ERR_CUDA 2         /* a CUDA runtime call or kernel launch failed */
#define FLMM_ERR_SOLVER 3       /* cuSOLVER returned an error */
#define FLMM_ERR_WORKSPACE 4    /* work_bytes smaller than the *_workspace_bytes query */
#define FLMM_ERR_DEVICE 5       /* the device is not an sm_103 (GB300) part */
#define FLMM_ERR_TIMEOUT 6      /* a bounded device-side wait gave up; the kernel returned without its result */
#define FLMM_ERR_IO 7           /* an output file could not be opened or written */

typedef struct flmm_context flmm_context;

/* Version of this ABI (major * 10000 + minor * 100 + patch). */
int flmm_version(void);
/* Static string for a status code. */
const char* flmm_status_string(int status);
/* Text of the last CUDA / cuSOLVER error seen on this thread (empty if none). */
const char* flmm_last_error(void);

/* Number of kernels this library has launched in this process (library calls such as cuSOLVER not counted). */
uint64_t flmm_kernel_launches(void);

/* Create / destroy a per-device context (cuSOLVER handle, device properties).  Allocates host memory and library
 * handles; the only allocating entry point.  `device` must be an sm_103 GPU. */
int flmm_context_create(int device, flmm_context** out);
int flmm_context_destroy(flmm_context* ctx);

/* ---- input preparation ------------------------------------------------------------------------------------ */

/* Unit standardiser (fasterlmm/io.py:223-246, torch branch): NaN-aware column mean and population std (ddof = 0),
 * std == 0 -> inf, (z - mean) / std, NaN -> 0.  Input Z (N, M) sample-major FP64 with NaN for missing calls, leading
 * dimension ldz >= M; output Zt (M, N) variant-major, leading dimension ldzt >= N. */
int flmm_standardise_f64(const double* Z, int64_t ldz, int N, int M, double* Zt, int64_t ldzt, void* stream);

/* Same standardiser from int8 dosages Gt (M, N) variant-major (0/1/2, negative = missing).  Statistics are exact
 * integer sums, so mean and std are exact to one rounding. */
int flmm_standardise_dosage(const int8_t* Gt, int64_t ldg, int N, int M, double* Zt, int64_t ldzt, void* stream);

/* Out-of-place FP64 transpose: At (cols, rows) = A (rows, cols)^T; moves the reference's sample-major (N, M)
 * layouts into the variant-major layout of this library. */
int flmm_transpose_f64(const double* A, int64_t lda, int rows, int cols, double* At, int64_t ldat, void* stream);

/* ---- kinship ---------------------------------------------------------------------------------------------- */

/* Gram of a variant block, the GRM numerator (fasterlmm/io.py:257-265): Gc (N, N) = sum over rows m of
 * Zt[m]^T Zt[m], FP64; beta = 0 overwrites Gc, beta = 1 accumulates.  Used per chromosome so that every LOCO
 * kinship is (total - own chromosome) / M_loco (hoisting fasterlmm/core.py:711 out of the chromosome loop). */
int flmm_gram_f64(const double* Zt, int64_t ldzt, int M, int N, double beta, double* Gc, int64_t ldg, void* stream);

/* K (N, N) = (Gtot - Gc) / m_loco.  Gc may be NULL (single-K: K = Gtot / m_loco). */
int flmm_loco_kinship(const double* Gtot, const double* Gc, int64_t ld, int N, double m_loco, double* K, void* stream);

/* ---- compat rotation (fasterlmm/core.py:487-519) ------------------------------------------------------------ */

/* Covariate basis: thin SVD of X (N, D) row-major in FP64 on the device (cuSOLVER gesvd), rank by the same
 * relative cut as torch.linalg.pinv (sigma > eps * max(N, D) * sigma_max).  Outputs Qx (D, N): the first `rank`
 * rows are an orthonormal basis of range(X), the rest zero; Xpinv (D, N) = pinv(X); rank on the device. */
int flmm_covariate_basis_workspace_bytes(flmm_context* ctx, int N, int D, size_t* bytes);
int flmm_covariate_basis(flmm_context* ctx, const double* X, int N, int D, double* Qx, double* Xpinv,
                         int32_t* rank_dev, void* work, size_t work_bytes, void* stream);

/* Kp (N, N) = (I - PX)(K + I)(I - PX) with PX = Qx^T Qx (fasterlmm/core.py:499-506), formed as a rank-2D update
 * of K + I (no N^3 products); rows of Qx beyond the rank are zero and drop out.  Workspace: 2 N D + D D doubles. */
int flmm_project_kinship_workspace_bytes(int N, int D, size_t* bytes);
int flmm_project_kinship(const double* K, int64_t ldk, const double* Qx, int N, int D, double* Kp, int64_t ldkp,
                         void* work, size_t work_bytes, void* stream);

/* Symmetric eigendecomposition in FP64 (cuSOLVER syevd; fasterlmm/core.py:54-77).  A (N, N) is overwritten by
 * the eigenvectors, stored one per row (ascending eigenvalue order), so rows D.. are Ut.  evals (N,) ascending. */
int flmm_eigh_workspace_bytes(flmm_context* ctx, int N, size_t* bytes);
int flmm_eigh(flmm_context* ctx, double* A, int N, double* evals, void* work, size_t work_bytes, void* stream);

/* The same for `batch` independent matrices A (batch, N, N) contiguous, evals (batch, N): every LOCO kinship of a
 * scan at once.  mode 1 = cusolverDnXsyevBatched on the context's main solver handle (slot = -1) or on worker handle
 * `slot` (0..7, so that batches on different streams never share a handle); mode 2 = syevd calls run side by side on
 * the context's worker streams, forked from and joined back into `stream`.  Workspace per mode from the query. */
int flmm_eigh_batched_workspace_bytes(flmm_context* ctx, int N, int batch, int mode, size_t* bytes);
int flmm_eigh_batched(flmm_context* ctx, double* A, int N, int batch, double* evals, int mode, int slot, void* work,
                      size_t work_bytes, void* stream);

/* FP32 twin of flmm_eigh_batched (mode 1, main handle) for the split-precision form, whose eigenbasis is used at
 * ~2^-22 relative precision: an FP32 eigendecomposition's backward error (~1e-7 of the projected kinship) is below
 * that.  Same layout: eigenvectors one per row of each A[b], evals ascending.  Below N = 2,500 the library's own
 * batched solver runs (FLMM_EIGH_F32=cusolver selects cuSOLVER's batched call instead); from there on batches of up to
 * 4 matrices go one at a time through cusolverDnSsyevd and larger ones through the batched call. */
int flmm_eigh_batched_f32_workspace_bytes(flmm_context* ctx, int N, int batch, size_t* bytes);
int flmm_eigh_batched_f32(flmm_context* ctx, float* A, int N, int batch, float* evals, void* work, size_t work_bytes,
                          void* stream);


/* One Ogita-Aishima refinement step for the FP32 decomposition of FP64 symmetric A (batch, N, N): U (batch, N, N)
 * FP32 eigenvector rows in, U_out refined rows out (U_out != U), evals (batch, N) FP64 Rayleigh quotients out.  A U
 * is formed FP64-accurately (flmm_refine_product, tensor-core form unless FLMM_REFINE_PRODUCT=df32 is set in the
 * environment); the corrections in FP32.  No counterpart in the reference (its eigh is FP64,
 * fasterlmm/core.py:54-77); it brings the FP32 eigenbasis to the accuracy the fast form's delta fit needs. */
int flmm_eigh_refine_workspace_bytes(int N, int batch, size_t* bytes);
int flmm_eigh_refine_f32(const double* A, float* U, float* U_out, double* evals, int N, int batch, void* work,
                         size_t work_bytes, void* stream);

/* The refinement's product W (batch, N, N) FP64 = U~ A^T for FP32 U and FP64 symmetric A (batch, N, N).  form 0:
 * FP16 tensor cores on exact digit planes (Ozaki splitting; U~ is U rounded to 28 bits below each row's largest
 * element, A to 48 bits; ~2^-46 relative); form 1: double-FP32 arithmetic on the FP32 pipe (U~ = U; ~2^-44).  U~
 * is written to Ut.  Workspace from flmm_refine_product_workspace_bytes. */
int flmm_refine_product_workspace_bytes(int N, int batch, size_t* bytes);
int flmm_refine_product(const float* U, const double* A, int N, int batch, int form, float* Ut, double* W, void* work,
                        size_t work_bytes, void* stream);

/* Kept spectrum: s (Neff,) = max(evals[D + i] - 1, 0) (fasterlmm/core.py:514); the _f32 form reads FP32 evals. */
int flmm_compat_spectrum(const double* evals, int N, int D, double* s, void* stream);
int flmm_compat_spectrum_f32(const float* evals, int N, int D, double* s, void* stream);

/* OLS regress-out of the covariates, row-wise: R[i] = A[i] - X (Xpinv A[i]^T) for rows of A (rows, N)
 * (fasterlmm/core.py:517 for phenotypes, :628 for variants).  R may alias A. */
int flmm_regress_out(const double* A, int64_t lda, int rows, int N, const double* X, int D, const double* Xpinv,
                     double* R, int64_t ldr, void* stream);

/* FP64 C (Mr, Nr) = alpha * A (Mr, K) * B (Nr, K)^T, both operands K-contiguous (the rotations UY = U_eff^T Y_r
 * and US = U_eff^T S_r, fasterlmm/core.py:518, :629, computed transposed). */
int flmm_gemm_nt_f64(const double* A, int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc, int Mr,
                     int Nr, int K, double alpha, void* stream);

/* ---- null-model delta fit (fasterlmm/core.py:525-595) --------------------------------------------------------- */

/* Grid node values exactly as torch.linspace(lo, hi, n_grid) in FP64. */
int flmm_delta_grid_nodes(double lo, double hi, int n_grid, double* grid, void* stream);

/* Plain FP64 form: (G, P) grid loss, first argmin, then the reference's 50-step golden-section search on
 * [grid[i-1], grid[i+1]] with its update order, result clamped to [lo, hi]; refine = 0 returns the grid node.
 * Outputs log_delta (P,) and grid_idx (P,).  Workspace holds the (G, Neff) weights. */
int flmm_fit_delta_f64_workspace_bytes(int Neff, int n_grid, size_t* bytes);
int flmm_fit_delta_f64(const double* s, int Neff, const double* UYt, int64_t ldu, int P, int n_grid, double lo,
                       double hi, int refine, double* log_delta, int32_t* grid_idx, void* work, size_t work_bytes,
                       void* stream);

/* ---- Wald scan (fasterlmm/core.py:601-671) -------------------------------------------------------------------- */

/* Plain FP64 form: for every column p < P and variant m < Mc: sWy = sum_n w UY US, sWs = sum_n w US^2 with
 * w = 1 / (s + exp(log_delta[p])), then beta, var_beta (df Neff - 1), F with the reference's clamps; max_F[p] is
 * raised to the column max (int64 atomic max on the FP64 bit pattern, F >= 0).  Real columns p < n_real write
 * f / beta / se / sfve at out[rows[m] * ldo + p].  Workspace holds w and w * UY (2 P Neff doubles). */
int flmm_wald_f64_workspace_bytes(int P, int Neff, size_t* bytes);
int flmm_wald_f64(const double* s, int Neff, const double* UYt, int64_t ldu, const double* log_delta, int P,
                  int n_real, const double* USt, int64_t ldus, int Mc, const int64_t* rows, double* f, double* beta,
                  double* se, double* sfve, int64_t ldo, double* max_F, void* work, size_t work_bytes, void* stream);

/* y[i] += alpha * x[i], FP64 (sums the per-chromosome Grams into the all-variant Gram). */
int flmm_axpy_f64(int64_t n, double alpha, const double* x, double* y, void* stream);

/* Permutation row orders (fasterlmm/perms.py:51-55), bit-identical to the reference's numpy draw: for each of the B
 * columns, PCG64 seeded by numpy's SeedSequence([seed, seed_cols[b]]), n_perm rows of N uniforms, argsort of each
 * row.  orders (B, n_perm, N) int32, orders[(b n_perm + j) N + i] = row landing at position i.  N <= 16384. */
int flmm_perm_orders(const int64_t* seed_cols, int B, uint64_t seed, int n_perm, int N, int32_t* orders,
                     void* stream);

/* Permutation packing (fasterlmm/perms.py:56-59): Yt_all (B + B n_perm, N) gets the B real columns Yt_real (B, N)
 * as its first rows, then for each real column b its n_perm shuffles, pheno-major: row B + b n_perm + j holds
 * Yt_real[b, orders[(b n_perm + j) N + n]] at sample n.  orders are 0-based row indices < N. */
int flmm_pack_perm_columns(const double* Yt_real, int64_t ldy, int B, int N, const int32_t* orders, int n_perm,
                           double* Yt_all, int64_t lda, void* stream);

/* nullh2 = 1 / (1 + exp(log_delta[p])) for p < n_real at out[rows[m] * ldo + p] (fasterlmm/core.py:669-670). */
int flmm_fill_nullh2(const double* log_delta, int n_real, const int64_t* rows, int Mc, double* nullh2, int64_t ldo,
                     void* stream);

/* Fill x[0..n) with a constant (max_F starts at -inf, fasterlmm/core.py:706). */
int flmm_fill_f64(double* x, int64_t n, double value, void* stream);

/* ---- post-scan statistics (fasterlmm/cli.py:405-406) ----------------------------------------------------------- */

/* out[i] = -log10 P(F(1, df2) > F[i]) in FP64, from the regularized incomplete beta I_{df2/(df2+F)}(df2/2, 1/2)
 * evaluated in log space by the modified Lentz continued fraction, so large F gives a finite value where
 * scipy.stats.f.sf underflows to 0. */
int flmm_neglog10_pvalue(const double* F, int64_t n, int df2, double* out, void* stream);

/* ---- split-precision tensor-core form --------------------------------------------------------------------------
 * Operands are FP16 pairs with one power-of-two exponent per row: x ~= (hi[k] + lo[k]) * scale[row].  Products of
 * two split operands are hi*hi + hi*lo + lo*hi on the tensor cores (tcgen05.mma kind::f16) with FP32 accumulation.
 * Split operands need 16-byte aligned base pointers and a row pitch (in elements) that is a multiple of 8.  These
 * kernels use bounded device-side waits; flmm_context_check reports a wait that gave up. */

/* Synchronise `stream` and return FLMM_ERR_TIMEOUT (clearing the flag) if a kernel of this context gave up a
 * bounded wait since the last check. */
int flmm_context_check(flmm_context* ctx, void* stream);

/* Split rows of X (rows, K) -- FP64 when x_is_f64, else FP32 -- into hi / lo FP16 (rows, ldo) and scale (rows,). */
int flmm_split_rows_f16(const void* X, int x_is_f64, int64_t ldx, int rows, int K, void* hi, void* lo, int64_t ldo,
                        float* scale, void* stream);

/* C (Mr, Nr) FP32 = sa[i] sb[j] sum_k (Ah + Al)[i, k] (Bh + Bl)[j, k]  (+ C when accumulate): the eigenbasis
 * rotations UY = U_eff^T Y_r and US = U_eff^T S_r (fasterlmm/core.py:518, :629) and the per-chromosome Gram of the
 * kinship (fasterlmm/io.py:264), all computed as row-major "rows x rows" products. */
int flmm_gemm_split_f16(flmm_context* ctx, const void* Ah, const void* Al, const float* sa, int64_t lda, int Mr,
                        const void* Bh, const void* Bl, const float* sb, int64_t ldb, int Nr, int K, float* C,
                        int64_t ldc, int accumulate, void* stream);

/* Kernel form and tile order of the split products (flmm_gemm_split_f16, flmm_wald_split_f16); no counterpart in the
 * reference.  mode 0: defaults (CTA pairs where the device runs them, A-major tile order); mode 1 (the initial mode,
 * unless FLMM_AUTOTUNE=0 is set in the environment): the first launch of each product shape times every candidate
 * (pair or single CTA x tile-order groups 1, 2, 4, 8) on the caller's operands and stream, synchronising the calling
 * thread once, and keeps the fastest for the process; not while the stream is being captured, and not for a GEMM
 * that accumulates into C; mode 2: force `pair` (0/1) and `group` (>= 1).  All choices give bit-identical results.
 * flmm_autotune_report writes one line per tuned shape into buf (host memory): "NG rows cols K K2 pair group ms
 * default_ms", and the number of shapes into *n_records. */
int flmm_tc_config(int mode, int pair, int group);
int flmm_autotune_report(char* buf, size_t len, int* n_records);

/* Fast delta fit (fasterlmm/core.py:561-595): FP32 grid argmin, then the stationary point of the loss in the
 * reference's bracket [grid[i-1], grid[i+1]] by a sign-safeguarded Newton iteration on d loss / d log delta with
 * compensated sums.  UYt is FP32.  Outputs as flmm_fit_delta_f64. */
int flmm_fit_delta_fast_workspace_bytes(int Neff, int n_grid, size_t* bytes);
int flmm_fit_delta_fast(const double* s, int Neff, const float* UYt, int64_t ldu, int P, int n_grid, double lo,
                        double hi, int refine, double* log_delta, int32_t* grid_idx, void* work, size_t work_bytes,
                        void* stream);

/* flmm_fit_delta_fast without caller workspace.  No counterpart in the reference: it exists for callers that cannot
 * give this library device memory -- a host whose device memory is all owned by another pool, or a latency-critical
 * loop that may not call cudaMalloc (it can synchronise the device).  The scratch is a fixed 4 MiB device array in
 * the library (held by every GPU that loads it until exit).  A call fits when flmm_fit_delta_fast_workspace_bytes
 * (Neff, n_grid) <= 4 MiB, i.e. 4 (n_grid Neff + n_grid + 2 Neff + 4) + 8 n_grid + 512 <= 4,194,304 bytes (n_grid * Neff
 * a little under 1,048,576); larger requests fail with FLMM_ERR_WORKSPACE.  The array's device address is looked up
 * (cudaGetSymbolAddress) on the first call in each driver context and kept with that context, so a call after
 * cudaDeviceReset or from another context looks it up again: make the first call of a context before any stream
 * capture.  All calls share the array: calls whose kernels overlap on the GPU race and must be serialised by the
 * caller.  Allocates nothing. */
int flmm_fit_delta_fast_noalloc(const double* s, int Neff, const float* UYt, int64_t ldu, int P, int n_grid,
                                double lo, double hi, int refine, double* log_delta, int32_t* grid_idx, void* stream);

/* Wald operands (fasterlmm/core.py:639-650).  All Wald outputs are unchanged when a column's weights w = 1/(s + delta)
 * are scaled by a constant; the fast form uses w~ = (shat + delta) / (s + delta) with shat the mean eigenvalue
 * (flmm_mean_f32).  Column side: A1 = w~ o UY split per column, rWr[p] = max(sum w~ UY^2, 1e-300), and the 10-point
 * Lagrange weights L (R entries per column, split) of x = log_delta[p] on the nodes x0 + r h (r < R).  Node side:
 * W~ (R, Neff) FP64 = (shat + e^{x_r}) / (s + e^{x_r}), to be split and multiplied into F = (US o US) W~^T, the node
 * values of sWs~; rWr0 receives the same sum with the unscaled weights.  Variant side: B1 = US and B2 = US o US split
 * per variant.  Column log deltas must lie in
 * [x0 + 4h, x0 + (R - 6) h]. */
int flmm_mean_f32(const double* x, int n, float* out, void* stream);
int flmm_wald_interp_nodes(const double* s, int Neff, const float* shat, double x0, double h, int R, double* W,
                           void* stream);
int flmm_wald_split_prep_columns(const float* s32, int Neff, const float* UYt, int64_t ldu, const double* log_delta,
                                 int P, const float* shat, double x0, double h, int R, void* A1h, void* A1l,
                                 int64_t lda, void* Lh, void* Ll, int64_t ldl, float* sa1, float* sl, float* rWr,
                                 float* rWr0, void* stream);
int flmm_wald_split_prep_variants(const float* USt, int64_t ldus, int Mc, int Neff, void* B1h, void* B1l, void* B2h,
                                  void* B2l, int64_t ldb, float* sb1, float* sb2, void* stream);

/* Fused split-precision Wald scan (fasterlmm/core.py:601-671): sWy = A1 B1^T (K = Neff) and sWs~ = L F^T (K = R) on
 * the tensor cores, then in the epilogue beta, var_beta (df Neff - 1), F, SE, SFVE with the reference's clamps (a
 * variant with sWs = 0 gets the FP64 1e-300 clamp); real columns p < n_real write out[rows[m] * ldo + p]; max_F[p]
 * is raised to the column max.  Strong real tests: with flag_count != NULL, every real test whose F exceeds f_refine
 * is left out of max_F and listed as (variant index m in [0, Mc), column p) int32 pairs in flags (room for flag_cap
 * pairs; *flag_count is reset by this call and receives the number of such tests, which may exceed flag_cap), for
 * flmm_wald_refine_f32 to recompute before the operands are overwritten.  flag_count == NULL: no list, every test
 * counts into max_F. */
int flmm_wald_split_f16(flmm_context* ctx, const void* A1h, const void* A1l, int64_t lda, const float* sa1,
                        const void* Lh, const void* Ll, int64_t ldl, const float* sl, const float* rWr,
                        const float* rWr0, int P, int n_real, const void* B1h, const void* B1l, int64_t ldb, const float* sb1, const void* Fh,
                        const void* Fl, int64_t ldf, const float* sf, int Mc, int Neff, int R, const int64_t* rows,
                        double* f, double* beta, double* se, double* sfve, int64_t ldo, double* max_F, float f_refine,
                        int32_t* flag_count, int32_t* flags, int flag_cap, void* stream);
/* The same scan with the F test's degrees of freedom given (var_df > 0) instead of Neff - 1: the low-rank form runs
 * its first product over K = k + N while the residual degrees of freedom stay N - D - 1 (fasterlmm/lowrank.py:270). */
int flmm_wald_split_f16_df(flmm_context* ctx, const void* A1h, const void* A1l, int64_t lda, const float* sa1,
                           const void* Lh, const void* Ll, int64_t ldl, const float* sl, const float* rWr,
                           const float* rWr0, int P, int n_real, const void* B1h, const void* B1l, int64_t ldb,
                           const float* sb1, const void* Fh, const void* Fl, int64_t ldf, const float* sf, int Mc,
                           int Neff, int R, const int64_t* rows, double* f, double* beta, double* se, double* sfve,
                           int64_t ldo, double* max_F, float f_refine, int32_t* flag_count, int32_t* flags,
                           int flag_cap, int var_df, void* stream);

/* ---- split-precision low-rank Wald (fasterlmm/lowrank.py:239-316) ----------------------------------------------
 *
 * With w~_i = (shat + delta) / (s_i + delta), c = (shat + delta) / delta (shat = mean s) and the off-rank residuals
 * UUY = Y_r - U_eff UY, UUS = S_r - U_eff US (lowrank.py:110, 289), the low-rank sWy is one product over K = k + N of
 * the column row [w~ o UY | c UUY] and the variant row [US | UUS], and sWs the interpolated product of
 * [US^2 | ||UUS||^2] with node weights [w~(x_r) | c(x_r)]; flmm_wald_split_f16_df then runs the fused scan with
 * K = k + N and var_df = N - D - 1.
 *
 * flmm_lr_residual: R = Y - C (rows, N) FP64 from Y FP64 and a product C FP32, and the row sums of squares ss.
 * flmm_lr_prep_columns: UYt (P, ldu) FP32 on-rank rotations, UUYt (P, ldy) FP64 off-rank residuals, yy_off (P,) FP64
 * = ||UUY||^2, s32 (k,) FP32, shat (device scalar, flmm_mean_f32 of s), column log deltas -> A1 (P, lda >= k + N)
 * split, the Lagrange weights L (P, ldl) split, rWr = sum w~ UY^2 + c yy_off, rWr0 = rWr / (shat + delta).
 * flmm_lr_prep_variants: USt (Mc, ldus) FP32 on-rank rotations of the standardised variants Zt (Mc, ldz) FP64, Ct =
 * U_eff US (Mc, ldc) FP32, orthonormal covariate basis rows Qt (D, ldq), D <= 16 -> UUS = Zt - Qt^T Qt Zt - Ct formed
 * in FP32, B1 = [US | UUS] (Mc, ldb >= k + N) and B2 = [US^2 | ||UUS||^2] (Mc, ldb2 >= k + 1), each split with its row
 * scales.  flmm_lr_interp_nodes: node weights W (R, ldw >= k + 1) FP64 at x_r = x0 + r h. */
int flmm_lr_residual(const double* Y, int64_t ldy, const float* C, int64_t ldc, int rows, int N, double* R,
                     int64_t ldr, double* ss, void* stream);
int flmm_lr_prep_columns(const float* s32, int k, const float* UYt, int64_t ldu, const double* UUYt, int64_t ldy,
                         int N, const double* yy_off, const double* log_delta, int P, const float* shat, double x0,
                         double h, int R, void* A1h, void* A1l, int64_t lda, void* Lh, void* Ll, int64_t ldl,
                         float* sa1, float* sl, float* rWr, float* rWr0, void* stream);
int flmm_lr_prep_variants(const float* USt, int64_t ldus, const double* Zt, int64_t ldz, const float* Ct, int64_t ldc,
                          int Mc, int k, int N, const double* Qt, int64_t ldq, int D, void* B1h, void* B1l,
                          int64_t ldb, float* sb1, void* B2h, void* B2l, int64_t ldb2, float* sb2, void* stream);
int flmm_lr_interp_nodes(const double* s, int k, const float* shat, double x0, double h, int R, double* W, int64_t ldw,
                         void* stream);
/* The strong real tests listed by flmm_wald_split_f16_df for a low-rank block (as flmm_wald_refine_f32 for the full
 * rank): each recomputed over the on-rank part (USt, UYt, s32) and the off-rank residuals (UUS = Sr - Ct, UUYt) with
 * no cancelling subtraction, on var_df degrees of freedom; outputs overwritten in place, max_F raised. */
int flmm_lr_wald_refine(const int32_t* flags, const int32_t* flag_count, int flag_cap, float f_refine, const float* USt,
                        int64_t ldus, const float* UYt, int64_t lduy, const double* Sr, int64_t ldz, const float* Ct,
                        int64_t ldc, const double* UUYt, int64_t lduu, const float* s32, const double* log_delta,
                        int k, int N, int Mc, int n_real, int var_df, const int64_t* rows, double* f, double* beta,
                        double* se, double* sfve, int64_t ldo, double* max_F, void* stream);

/* Re-evaluation of the strong real tests listed by flmm_wald_split_f16 (the reference's Wald formulas,
 * fasterlmm/core.py:649-667, without the cancelling subtraction rss = rWr - sWy^2 / sWs): from the FP32 rotated
 * operands USt (Mc, ldus) and UYt (P, lduy) of the same chromosome, the FP32 spectrum s32 and the column log deltas,
 * each listed test's residual sum of squares is formed around the scan's beta as a sum of positive terms
 * (compensated FP32 per lane, FP64 across the warp), and f, beta, se, sfve are overwritten in place and max_F[p]
 * raised to the new F.  When *flag_count > flag_cap every real test of the chromosome whose stored F exceeds f_refine
 * is recomputed instead.  No counterpart in the reference (which computes in FP64 throughout). */
int flmm_wald_refine_f32(flmm_context* ctx, const int32_t* flags, const int32_t* flag_count, int flag_cap,
                         float f_refine, const float* USt, int64_t ldus, const float* UYt, int64_t lduy,
                         const float* s32, const double* log_delta, int Neff, int Mc, int n_real, const int64_t* rows,
                         double* f, double* beta, double* se, double* sfve, int64_t ldo, double* max_F, void* stream);

/* Small conversions of the fast form: y[i] = (float)x[i]; y[i] += x[i] (FP32 into FP64); the LOCO kinship from an FP64
 * total and an FP32 chromosome Gram, K = (Gtot - Gc) / m_loco. */
int flmm_convert_f64_f32(int64_t n, const double* x, float* y, void* stream);
int flmm_accumulate_f32_f64(int64_t n, const float* x, double* y, void* stream);
int flmm_loco_kinship_f32(const double* Gtot, const float* Gc, int N, double m_loco, double* K, void* stream);

/* ---- scan-level entry points (fasterlmm/perms.py:21-68 -> fasterlmm/core.py:677-726) -----------------------------
 *
 * The whole fast-form LOCO scan behind a handful of calls, for callers that bind the library directly (the reference
 * binds the Python functions by name; these are what an FFI binding of that path would call).  A scan object is
 * bound to one device and owns its working buffers; inputs and outputs are caller-owned device pointers, every call
 * takes a stream (0 = the legacy default stream) and returns a status.  Order: create, group_prepare (once per
 * sample group: covariates and kinship panel), rotate_phenos (once per batch of scan columns), then either run (every
 * chromosome, pipelined) or fit_delta(k) followed by wald(k) per chromosome; destroy.
 *
 * flmm_scan_opts: delta grid (n_grid points on [log_delta_min, log_delta_max], refine != 0: exact refinement of the
 * grid argmin; fasterlmm/core.py:561-595), eigh_refine_steps (0: 2 up to N = 1,024, 3 above), f_refine (real tests
 * with F above it are recomputed without the FP32 cancellation; <= 0: off), pipeline (!= 0: the column side of
 * chromosome k + 1 runs on a second stream beside the variant side of chromosome k). */
typedef struct flmm_scan flmm_scan;
typedef struct flmm_scan_opts {
    int n_grid;
    double log_delta_min;
    double log_delta_max;
    int refine;
    int eigh_refine_steps;
    double f_refine;
    int pipeline;
} flmm_scan_opts;
int flmm_scan_opts_default(flmm_scan_opts* opts);
int flmm_scan_create(int device, int N, int D, const flmm_scan_opts* opts, flmm_scan** out);
int flmm_scan_destroy(flmm_scan* scan);
/* Covariates X (N, D) row-major and the kinship panel Zt_kin (M_kin, ldz) standardised, variant-major, with host
 * chromosome labels chrom_kin (M_kin,); loco_chroms (host, n_units) lists the chromosomes to scan, each with the
 * kinship of the panel without that chromosome (fasterlmm/core.py:707-713); n_units = 0 prepares one unit with the
 * whole panel's kinship (single-K, fasterlmm/core.py:729-740).  Forms the covariate basis, the per-chromosome Grams,
 * the projected LOCO kinships and their refined eigendecompositions; returns after the device work is done. */
int flmm_scan_group_prepare(flmm_scan* scan, const double* X, const double* Zt_kin, int64_t ldz, int M_kin,
                            const int32_t* chrom_kin, const int32_t* loco_chroms, int n_units, void* stream);
/* Scan columns Yt (P, ldy) row-major (the real phenotypes first, then their permutations; fasterlmm/perms.py:56-59),
 * regressed off the covariates and split for the tensor cores.  Returns after the device work is done. */
int flmm_scan_rotate_phenos(flmm_scan* scan, const double* Yt, int64_t ldy, int P, void* stream);
/* Column side of unit k (the k-th prepared chromosome): UY = U_eff^T Y_r and the fast delta fit; log_delta_out (P,)
 * device, may be NULL.  Must precede flmm_scan_wald(k); units k and k + 2 share buffers. */
int flmm_scan_fit_delta(flmm_scan* scan, int unit, double* log_delta_out, void* stream);
/* Variant side of unit k: the chromosome's standardised variants Zt_c (Mc, ldz), their output rows rows (Mc,) int64
 * device; fused Wald scan into f, beta, se, sfve, nullh2 (nullh2 may be NULL) at out[rows[m] * ldo + p] for the
 * n_real real columns, max_F (P,) raised to the column maxima (fasterlmm/core.py:601-671). */
int flmm_scan_wald(flmm_scan* scan, int unit, const double* Zt_c, int64_t ldz, int Mc, const int64_t* rows,
                   int n_real, double* f, double* beta, double* se, double* sfve, double* nullh2, int64_t ldo,
                   double* max_F, void* stream);
/* Every unit: tested variants Zt (M, ldz) standardised, variant-major, with host chromosome labels chrom (M,); unit k
 * scans the variants of its chromosome (all variants for a single-K unit); outputs (M, n_real) at ldo, max_F (P,)
 * (set to -inf first), log_delta_out (n_units, P) device or NULL.  The column side of unit k + 1 runs on the scan's
 * second stream while the variant side of unit k runs on `stream` (opts.pipeline).  Returns after the device work
 * is done, FLMM_ERR_TIMEOUT if a bounded device wait gave up. */
int flmm_scan_run(flmm_scan* scan, const double* Zt, int64_t ldz, int M, const int32_t* chrom, int n_real,
                  double* f, double* beta, double* se, double* sfve, double* nullh2, int64_t ldo, double* max_F,
                  double* log_delta_out, void* stream);

/* ---- PLINK .bed input (fasterlmm/io.py:54-67, fasterlmm/io_stream.py:60-71) ------------------------------------
 *
 * Decode n_variants SNP-major .bed records (each bytes_per_variant = ceil(n_fam / 4) bytes, header stripped) into
 * int8 dosages G (n_variants, ldg): kept sample i is .fam row rows[i] (rows NULL: the first n_keep rows); A1 allele
 * counts with count_a1 != 0 (the reference's default), else A2 counts; missing calls and rows outside [0, n_fam)
 * give -1.  flmm_standardise_dosage then produces the standardised variant-major block. */
int flmm_bed_decode(const uint8_t* bed, int64_t bytes_per_variant, int n_variants, int n_fam, const int32_t* rows,
                    int n_keep, int count_a1, int8_t* G, int64_t ldg, void* stream);

/* ---- learned delta proposal (no counterpart in the reference) ---------------------------------------------------
 *
 * Features of each rotated column, feats (P, 65): log energy fractions of UY^2 over 32 equal-count bins of the
 * ascending spectrum s (Neff >= 32), log mean eigenvalue per bin, log(Neff) / 10.  The MLP 65 -> 128 -> 128 -> 1
 * (tanh-GELU; W1 (128, 65), W2 (128, 128) row-major, w3 (128,)) maps them to a proposed log delta, clamped to
 * [lo, hi]. */
int flmm_delta_features_f32(const double* s, int Neff, const float* UYt, int64_t ldu, int P, float* feats,
                            void* stream);
int flmm_delta_mlp_f32(const float* feats, int P, const float* W1, const float* b1, const float* W2, const float* b2,
                       const float* w3, float b3, double lo, double hi, double* x_out, void* stream);

/* The fast delta fit (flmm_fit_delta_fast; fasterlmm/core.py:561-595) with the grid search collapsed to a narrow
 * bracket around the MLP's proposal: each column evaluates the FP32 grid loss at the 2 half_width + 1 nodes nearest
 * its proposal.  A column whose window argmin is on the window's edge falls back to the full grid; every
 * audit_stride-th column (0 = none) also evaluates the full grid, and if a node outside its window is lower, every
 * column falls back.  The exact Newton refinement then runs from the chosen node, so results equal the grid path's
 * wherever the loss has one minimum near the grid argmin.  stats (device int32[4], zeroed by the call): columns that
 * fell back, audited columns, audits lost, grid nodes evaluated by the window and audit pass (the full-grid fallback
 * adds n_grid per fallback column).  Workspace: flmm_fit_delta_learned_workspace_bytes. */
int flmm_fit_delta_learned_workspace_bytes(int Neff, int n_grid, int P, size_t* bytes);
int flmm_fit_delta_learned(const double* s, int Neff, const float* UYt, int64_t ldu, int P, int n_grid, double lo,
                           double hi, int refine, const float* W1, const float* b1, const float* W2, const float* b2,
                           const float* w3, float b3, int half_width, int audit_stride, double* log_delta,
                           int32_t* grid_idx, int32_t* stats, void* work, size_t work_bytes, void* stream);

/* Training of the proposal MLP on the device (no counterpart in the reference).  The FP32 master parameters are one
 * flat array of FLMM_MLP_PARAMS floats: W1 (128, 65) | b1 (128) | W2 (128, 128) | b2 (128) | w3 (128) | b3.
 *
 * flmm_mlp_grad: grad = d/dparams of the mean smooth-L1 loss (huber_beta) of the network's output against y[rows[r]]
 * for the feature rows X[rows[r], :65], r < batch, of a feature matrix X (n_x, ldx) and labels y (n_x,); an index
 * outside [0, n_x) contributes nothing.  bf16 != 0 rounds every matrix operand to BF16 (inputs, weights,
 * activations, back-propagated gradients) with FP32 accumulation; bf16 == 0 keeps FP32 operands.  *loss (device
 * float, may be NULL) receives the minibatch loss.  Deterministic: per-CTA partial gradients are added in a fixed
 * order.  Workspace: flmm_mlp_grad_workspace_bytes(batch).
 * flmm_mlp_adamw: one AdamW step (decoupled weight decay, bias correction for step >= 1) on the master parameters
 * with moment arrays m, v (FLMM_MLP_PARAMS floats each, zero before step 1). */
#define FLMM_MLP_PARAMS 25089
int flmm_mlp_grad_workspace_bytes(int batch, size_t* bytes);
int flmm_mlp_grad(const float* params, const float* X, int64_t ldx, int n_x, const float* y, const int32_t* rows,
                  int batch, float huber_beta, int bf16, float* grad, float* loss, void* work, size_t work_bytes,
                  void* stream);
int flmm_mlp_adamw(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1, float beta2,
                   float eps, float weight_decay, void* stream);

/* ---- low-rank path (fasterlmm/lowrank.py): kinship factor G (N, k), k < N --------------------------------------
 *
 * s (k,) kept eigenvalues, UYt (P, k) on-rank rotated columns, UUYt (P, N) off-rank residuals, USt / UUSt the same
 * for a variant block; Neff = N - D (not k). */

/* fit_delta_grid_lowrank (fasterlmm/lowrank.py:172-208): grid + golden section on the low-rank ML loss, with the
 * off-rank sum of squares yy_off (P,) (see flmm_row_sumsq_f64) and (Neff - k) log(delta) in log det V.  Workspace
 * as flmm_fit_delta_f64_workspace_bytes(k, n_grid). */
int flmm_fit_delta_lowrank_f64(const double* s, int k, const double* UYt, int64_t ldu, const double* yy_off, int Neff,
                               int P, int n_grid, double lo, double hi, int refine, double* log_delta,
                               int32_t* grid_idx, void* work, size_t work_bytes, void* stream);

/* snp_wald_scan_lowrank (fasterlmm/lowrank.py:239-316): on-rank forms weighted by 1 / (s + delta), off-rank ones
 * by 1 / delta, df = Neff - 1; outputs as flmm_wald_f64. */
int flmm_wald_lowrank_f64_workspace_bytes(int k, int N, int P, int Mc, size_t* bytes);
int flmm_wald_lowrank_f64(const double* s, int k, const double* UYt, int64_t ldu, const double* UUYt, int64_t lduu,
                          int N, int Neff, const double* log_delta, int P, int n_real, const double* USt, int64_t ldus,
                          const double* UUSt, int64_t lduus, int Mc, const int64_t* rows, double* f, double* beta,
                          double* se, double* sfve, int64_t ldo, double* max_F, void* work, size_t work_bytes,
                          void* stream);

/* out[r] = sum_c A[r, c]^2 (off-rank residual sums of squares). */
int flmm_row_sumsq_f64(const double* A, int64_t lda, int rows, int cols, double* out, void* stream);

/* ---- plain GLS path (fasterlmm/core.py:89-451): covariates kept in the model ------------------------------------
 *
 * Layouts as in the compat path: Xrt (C, N) the rotated covariates U^T X one column per row, Yrt (P, N) the rotated
 * phenotype columns, Srt (M, N) rotated variants, s (N,) the spectrum.  1 <= C <= 30. */

/* eigendecompose's jitter and clamp (fasterlmm/core.py:89-102): A[i, i] += value; y = max(x, 0). */
int flmm_shift_diagonal_f64(double* A, int N, int64_t lda, double value, void* stream);
int flmm_clamp_nonneg_f64(const double* x, int64_t n, double* y, void* stream);

/* GLS -2 log L (fasterlmm/core.py:148-224): per_column = 0 evaluates the (n_ld, P) grid loss[g, p] at the n_ld
 * values log_delta (workspace from the query); per_column = 1 evaluates loss[p] at log_delta[p] (n_ld == P, no
 * workspace).  reml = 1 divides by N - C and adds log det(X~^T W X~).  A failed Cholesky gives +inf. */
int flmm_gls_loss_workspace_bytes(int N, int C, int P, int n_ld, size_t* bytes);
int flmm_gls_loss_f64(const double* s, int N, const double* Xrt, int64_t ldx, int C, const double* Yrt, int64_t ldy,
                      int P, const double* log_delta, int n_ld, int per_column, int reml, double* loss, void* work,
                      size_t work_bytes, void* stream);

/* fit_delta_grid (fasterlmm/core.py:227-264): grid argmin then 50 golden-section steps per column, ML or REML. */
int flmm_fit_delta_gls_workspace_bytes(int N, int C, int P, int n_grid, size_t* bytes);
int flmm_fit_delta_gls_f64(const double* s, int N, const double* Xrt, int64_t ldx, int C, const double* Yrt,
                           int64_t ldy, int P, int n_grid, double lo, double hi, int refine, int reml,
                           double* log_delta, int32_t* grid_idx, void* work, size_t work_bytes, void* stream);

/* snp_wald_scan (fasterlmm/core.py:295-375): GLS Wald of every (variant, column) with the covariates in the model;
 * detail rows[m] * ldo + p for p < n_real, running max into max_F (P,) (initialise to -inf). */
int flmm_wald_gls_workspace_bytes(int N, int C, int P, size_t* bytes);
int flmm_wald_gls_f64(const double* s, int N, const double* Xrt, int64_t ldx, int C, const double* Yrt, int64_t ldy,
                      const double* log_delta, int P, int n_real, const double* Srt, int64_t lds, int M,
                      const int64_t* rows, double* f, double* beta, double* se, double* sfve, int64_t ldo,
                      double* max_F, void* work, size_t work_bytes, void* stream);

/* chi2.isf(P(F(1, df2) > F), 1) for every element (the genomic inflation factor's input,
 * fasterlmm/inflation.py:19-29): 2 erfcinv(p)^2; NaN stays NaN, p below the FP64 range gives +inf. */
int flmm_chisq1_from_f(const double* F, int64_t n, int df2, double* out, void* stream);

/* Genome-wide permutation threshold per phenotype (fasterlmm/cli.py:128, :406): thresh[b] = numpy.quantile(p, q) with
 * linear interpolation, p = P(F(1, df2) > perm_max_F[b, :]) over the row's n_perm permutation maxima (B, n_perm). */
int flmm_perm_threshold_p(const double* perm_max_F, int B, int n_perm, int df2, double q, double* thresh,
                          void* stream);

/* P(F(1, df2) > F) for every element, the CLI's PValue column (fasterlmm/cli.py:405, scipy.stats.f.sf(F, 1, df2)):
 * F <= 0 gives 1, +inf gives 0, NaN stays NaN. */
int flmm_f_pvalue(const double* F, int64_t n, int df2, double* out, void* stream);

/* Per-phenotype setup of the batched epistasis Wald for one anchor and a chunk of Pc phenotypes
 * (lux/src/fasterlmm_lux/epi/_kernel.py:21-150, the FP64 block before the test-column loop), all FP64: with
 * w_p = 1 / (s + exp(log_delta[p])) (N,), A_p = X^T W_p X = L_p L_p^T, beta_x = A_p^-1 X^T W_p y_p and
 * r_p = y_p - X beta_x, it writes R1 (Pc (C + 1), N; phenotype p's C rows Q_p = L_p^-1 X^T W_p, then w_p o r_p),
 * W (Pc, N) = w_p, rWr (Pc,) = max(sum w r^2, 1e-300) and L (Pc C (C + 1) / 2 doubles, caller-allocated scratch:
 * each L_p's packed lower triangle, row by row).  X is (N, C) with row stride ldx, y_p = Y[n * ldy + p].  When a
 * pivot of some A_p is not positive (A_p not positive definite) *info is set to 1 (it is never cleared) and that
 * phenotype's outputs are NaN; the reference's batched Cholesky raises for the batch.  1 <= C <= 200. */
int flmm_epi_setup_f64(const double* s, int N, const double* X, int64_t ldx, int C, const double* Y, int64_t ldy,
                       const double* log_delta, int Pc, double* R1, double* W, double* rWr, double* L, int* info,
                       void* stream);

/* Batched epistasis Wald, per anchor and phenotype chunk (lux/src/fasterlmm_lux/epi/_kernel.py:21-150): from
 * G1 (Pc (C + 1), Mc) FP32 = [Q_p; (w_p o r_p)] S (Q_p = L_p^-1 X^T W_p, C rows per phenotype), G2 (Pc, Mc) FP32 =
 * W (S o S) and rWr (Pc,): quad = ||Q_p s_m||^2, denom = max(sWs - quad, 1e-300), beta, SE, F (F = 0 where
 * sWs - quad < floor_rel sWs); detail at (m0 + m) * ldo + p0 + p for p0 + p < n_real; running maximum F and its
 * first column into max_f / argmax (P,) (a chunk replaces them only when strictly greater, never when its maximum
 * is NaN).  var_df = N - C - 1. */
int flmm_epi_wald_f32(const float* G1, int64_t ldg1, const float* G2, int64_t ldg2, const double* rWr, int Pc, int C,
                      int Mc, int m0, int p0, int n_real, double var_df, double floor_rel, double* beta, double* se,
                      double* F, int64_t ldo, double* max_f, int64_t* argmax, void* stream);

/* ---- output files (host code; fasterlmm/cli.py:100-161) ---------------------------------------------------------
 * Numbers are written as the reference's pyarrow CSV writer writes them: shortest round-trip digits, fixed notation
 * for decimal exponents -6 .. 9, d.ddde+X otherwise, nan / inf / -inf.  Each call writes one file and holds no
 * lock, so phenotypes can be written from parallel threads.  Errors: FLMM_ERR_ARG, FLMM_ERR_IO. */

/* The text of v[0..n) back to back in buf (buf_bytes; 40 bytes per value always suffice), value i at
 * [offsets[i], offsets[i + 1]) (offsets holds n + 1 entries). */
int flmm_format_f64(const double* v, int64_t n, char* buf, int64_t buf_bytes, int64_t* offsets);

/* One phenotype's gwas.tsv (fasterlmm/cli.py:150-153): header plus M rows sid_index, SNP, Chr, GenDist (null),
 * ChrPos, PValue, SnpWeight, SnpWeightSE, EffectSize = beta^2 g_var / p_var, SnpFractVarExpl, Mixing (0), Nullh2,
 * Pheno, PhenoCount, in the row order order[i * ld_order] (variant indices; NULL = variant order).  Per-variant
 * columns chrom, pos, g_var have stride 1; result columns pvalue .. nullh2 have stride ld (e.g. B for an (M, B)
 * variant-major table).  SNP ids are snp_ids[snp_offsets[v] .. snp_offsets[v + 1]). */
int flmm_write_gwas_tsv(const char* path, int64_t M, const char* snp_ids, const int64_t* snp_offsets,
                        const double* chrom, const double* pos, const double* g_var, double p_var,
                        const double* pvalue, const double* beta, const double* se, const double* sfve,
                        const double* nullh2, int64_t ld, const int64_t* order, int64_t ld_order,
                        const char* pheno_name, int64_t pheno_count);

/* A one-column table (e.g. perms.tsv, fasterlmm/cli.py:154): the header line, then one value per line. */
int flmm_write_column_tsv(const char* path, const char* header, const double* v, int64_t n);

/* Host memory: dst[r * ld + j] = vec[j] for r < rows, j < n, on up to `threads` host threads.  The streamed result
 * path fills each chromosome's nullh2 rows this way from one (B,) vector instead of copying repeats from the
 * device.  No counterpart in the reference, which keeps its results on one device. */
int flmm_fill_rows_host_f64(double* dst, int64_t ld, int64_t rows, const double* vec, int64_t n, int threads);

/* Page-locked host memory mapped into the device's address space (cudaHostAllocMapped): *host_ptr for the host,
 * *dev_ptr for kernels, which then write it over the host link without the copy engines (whose queue the scan's
 * result copies occupy).  The streamed result path has each chromosome's nullh2 vector written there.  Free with
 * flmm_host_free_mapped. */
int flmm_host_alloc_mapped(size_t bytes, void** host_ptr, void** dev_ptr);
int flmm_host_free_mapped(void* host_ptr);

#ifdef __cplusplus
}
#endif

#endif /* FASTERLMM_GB300_H */

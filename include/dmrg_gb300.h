/*
 * dmrg_gb300.h -- C ABI of the GB300 two-site DMRG/TDVP sweep library.
 *
 * Every entry point takes plain device pointers, sizes and a cudaStream_t
 * (passed as void*), allocates nothing itself (scratch comes from a
 * caller-provided workspace whose size the matching *_workspace_bytes()
 * reports), and returns an int status (DMRG_OK = 0).  No entry point
 * traps, aborts or waits without a bound.
 *
 * Array layouts (row-major, element type double or interleaved complex
 * double as selected by `dtype`):
 *   MPS site tensor A      (chi_left, d, chi_right)
 *   MPO site tensor W      (w_left, d_in, d_out, w_right)   d_in = ket leg
 *   left environment L     (chi_bra, w, chi_ket)
 *   right environment R    (chi_bra, w, chi_ket)
 *   two-site centre theta  (chi_left, d1, d2, chi_right)
 *
 * The functions replace the numerical kernels of dmrgpy's pure-Python
 * backend (src/dmrgpy/pyitensor); each declaration cites the reference
 * function it stands in for.
 */
#ifndef DMRG_GB300_H
#define DMRG_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define DMRG_OK              0
#define DMRG_ERR_ARG         1  /* bad shape, null pointer or unsupported combination */
#define DMRG_ERR_WORKSPACE   2  /* caller workspace smaller than *_workspace_bytes() */
#define DMRG_ERR_CUDA        3  /* a CUDA runtime call or kernel launch failed */
#define DMRG_ERR_NAN         4  /* a non-finite value reached a reduction */
#define DMRG_ERR_NOCONV      5  /* an iterative eigensolver hit its sweep limit */
#define DMRG_ERR_TIMEOUT     6  /* a bounded device-side wait gave up */
#define DMRG_ERR_UNSUPPORTED 7  /* combination not built (e.g. complex + TF32x3) */
#define DMRG_ERR_PRECISION   8  /* a split-TF32 estimate cannot decide what was asked
                                   (callers repeat the step in FP64) */

/* ---- element types and contraction precisions ------------------------ */
#define DMRG_REAL64      0
#define DMRG_COMPLEX128  1
#define DMRG_PREC_FP64   0  /* all contractions in FP64 */
#define DMRG_PREC_TF32X3 1  /* bulk contractions as split-TF32 (3 products,
                               FP32 accumulation) on tcgen05; vectors and
                               reductions stay FP64 */

/* Effective-Hamiltonian operator of one bond/site.
 *   kind 2: y = L . W1 . W2 . R . theta  over theta (chil, d1, d2, chir)
 *           (pyitensor/dmrg.py:224-248 two_site_heff, the plan of
 *            pyitensor/kernels.py:298-410)
 *   kind 1: y = L . W1 . R . A            over A (chil, d1, chir)
 *           (pyitensor/dmrg.py:251-275 one_site_heff)
 *   kind 0: y = L . R . C                 over C (chil, chir)
 *           (pyitensor/dmrg.py:278-299 zero_site_heff)
 * MPO bonds: W1 is (wl, d1, d1, wm), W2 is (wm, d2, d2, wr); for kind 1
 * W1 is (wl, d1, d1, wr); for kind 0, wl == wr and W1/W2 are unused.
 * L is (chil, wl, chil), R is (chir, wr, chir). */
typedef struct dmrg_heff_t {
  int kind;
  int dtype;
  int precision;
  int chil, d1, d2, chir;
  int wl, wm, wr;
  const void* L;
  const void* W1;
  const void* W2;
  const void* R;
} dmrg_heff_t;

/* Library version (major*10000 + minor*100 + patch). */
int dmrg_version(void);
/* Static description of a status code. */
const char* dmrg_status_string(int status);
/* Number of CUDA kernels this library has launched in this process (all
 * devices, all streams); a monotonic counter for instrumentation. */
unsigned long long dmrg_kernel_launches(void);

/* ---- effective-Hamiltonian matvec ------------------------------------- */
/* Workspace for dmrg_heff_apply (also covers the operand preparation). */
size_t dmrg_heff_workspace_bytes(const dmrg_heff_t* op);
/* y = H_eff x.  Replaces the matvec closure of pyitensor/kernels.py:353-410
 * (_make_matvec_planned) built by pyitensor/dmrg.py:224-299.  x and y must
 * not alias. */
int dmrg_heff_apply(const dmrg_heff_t* op, const void* x, void* y,
                    void* work, size_t work_bytes, void* stream);

/* The same matvec split in two, for callers that drive their own Krylov
 * loop: dmrg_heff_prepare() does the per-operator work once (split-TF32:
 * splitting L, R and the two-site MPO into the workspace; FP64: nothing),
 * dmrg_heff_apply_prepared() applies H_eff for each new vector with the same
 * op and workspace (the plan-once / replay-per-iteration structure of
 * pyitensor/kernels.py:353-410).  dmrg_heff_status() synchronises the stream
 * and reports a bounded-wait timeout recorded by the tensor-core kernels
 * since the last prepare. */
int dmrg_heff_prepare(const dmrg_heff_t* op, void* work, size_t work_bytes, void* stream);
int dmrg_heff_apply_prepared(const dmrg_heff_t* op, const void* x, void* y,
                             void* work, size_t work_bytes, void* stream);
int dmrg_heff_status(const dmrg_heff_t* op, void* work, size_t work_bytes, void* stream);

/* Allocation-free FP64 matvec: y = H_eff x like dmrg_heff_apply, with the
 * scratch taken from one fixed device array inside the library instead of a
 * caller workspace; the call allocates nothing.  It has no counterpart in the
 * reference (whose matvec allocates its NumPy intermediates on every call).
 * For callers that cannot allocate device memory per call (no device
 * allocator of their own, or a memory budget fixed at start-up).
 * precision must be DMRG_PREC_FP64 (else DMRG_ERR_UNSUPPORTED); an operator
 * whose dmrg_heff_workspace_bytes() exceeds DMRG_NOALLOC_SCRATCH_BYTES is
 * rejected with DMRG_ERR_WORKSPACE.  The first call on a device sets up the
 * array's address and should come before any stream capture; the address is
 * cached per device number, so the library assumes the device's primary
 * context (the CUDA runtime's) and no cudaDeviceReset between calls.  All
 * calls share the array: calls that may execute at the same time race and
 * must be serialised by the caller (e.g. one stream); nothing in it needs to
 * start at zero.  The array is part of the library's device image: every
 * device that loads the library holds its 64 MiB until the process exits,
 * whether or not this entry point is called. */
#define DMRG_NOALLOC_SCRATCH_BYTES (64u << 20)
int dmrg_heff_apply_noalloc(const dmrg_heff_t* op, const void* x, void* y, void* stream);

/* ---- environments ----------------------------------------------------- */
size_t dmrg_env_workspace_bytes(int dtype, int precision, int chil, int d, int chir, int wl, int wr);
/* Lnew (chir, wr, chir) = L (chil, wl, chil) . conj(A) . W . A with
 * A (chil, d, chir), W (wl, d, d, wr).  Replaces pyitensor/dmrg.py:170-191
 * (_extend_left). */
int dmrg_env_extend_left(int dtype, int precision, int chil, int d, int chir, int wl, int wr,
                         const void* L, const void* W, const void* A, void* Lnew,
                         void* work, size_t work_bytes, void* stream);
/* Rnew (chil, wl, chil) = R (chir, wr, chir) . conj(B) . W . B with
 * B (chil, d, chir).  Replaces pyitensor/dmrg.py:194-201 (_extend_right). */
int dmrg_env_extend_right(int dtype, int precision, int chil, int d, int chir, int wl, int wr,
                          const void* R, const void* W, const void* B, void* Rnew,
                          void* work, size_t work_bytes, void* stream);

/* ---- adjoint of the environment chain (FP64) ----------------------------- */
size_t dmrg_env_gradient_workspace_bytes(int dtype, int chil, int d, int chir, int wl, int wr);
/* G (wl, d, d, wr) = d<psi|H|psi>/dW_i = L (chil, wl, chil) . A . conj(A) .
 * R (chir, wr, chir) with A (chil, d, chir) the site tensor, L/R the
 * environments of the sites left/right of it.  No reference function: the
 * reference has no derivative features; the result is checked against
 * finite differences of its energies and against <dH/dlambda> evaluated with
 * its expectation value (pyitensor/chain.py:277-287). */
int dmrg_env_gradient(int dtype, int chil, int d, int chir, int wl, int wr,
                      const void* L, const void* A, const void* R, void* G,
                      void* work, size_t work_bytes, void* stream);

/* Transition forms for <chi|H|psi> with two different MPS: bra B (clb, d,
 * crb), ket A (clk, d, crk), environments (chi_bra, w, chi_ket).
 * side 0: Lnew (crb, wr, crk) = L (clb, wl, clk) . conj(B) . W . A;
 * side 1: Rnew (clb, wl, clk) = R (crb, wr, crk) . conj(B) . W . A.
 * Used by the adjoint of real-time evolution (costate bra, state ket); the
 * reference's counterpart is its transition element overlap_aMb
 * (pyitensor/chain.py:289-293), evaluated there on the host. */
size_t dmrg_env_mixed_workspace_bytes(int side, int dtype, int clb, int crb, int clk, int crk, int d, int wl, int wr);
int dmrg_env_extend_mixed(int side, int dtype, int clb, int crb, int clk, int crk, int d, int wl, int wr,
                          const void* E, const void* W, const void* B, const void* A, void* Enew,
                          void* work, size_t work_bytes, void* stream);
/* G (wl, d, d, wr) = d<chi|H|psi>/dW_i with the bra/ket site tensors B, A and
 * the transition environments L (clb, wl, clk), R (crb, wr, crk).  No
 * reference counterpart (no derivative features in the reference). */
size_t dmrg_env_gradient_mixed_workspace_bytes(int dtype, int clb, int crb, int clk, int crk, int d, int wl, int wr);
int dmrg_env_gradient_mixed(int dtype, int clb, int crb, int clk, int crk, int d, int wl, int wr,
                            const void* L, const void* B, const void* A, const void* R, void* G,
                            void* work, size_t work_bytes, void* stream);

/* ---- Krylov solvers ------------------------------------------------------ */
size_t dmrg_lanczos_workspace_bytes(const dmrg_heff_t* op, int niter);
/* Lowest eigenpair of H_eff by Lanczos with full reorthogonalisation; stops
 * when the lowest Ritz value moves by less than tol*max(1,|E|), when the
 * residual norm drops below tol, or after niter matvecs.  x holds the start
 * vector on entry and the normalised eigenvector on exit.  Replaces
 * pyitensor/dmrg.py:95-142 (_lanczos_ground_state) as driven by
 * pyitensor/dmrg.py:302-333 (_local_ground_state). */
int dmrg_lanczos_ground(const dmrg_heff_t* op, void* x, int niter, double tol,
                        double* energy, int* iters,
                        void* work, size_t work_bytes, void* stream);
size_t dmrg_expm_workspace_bytes(const dmrg_heff_t* op, int niter);
/* x <- exp(coeff * H_eff) x by a Krylov subspace of dimension <= niter with
 * Saad's a-posteriori stop (beta0*beta_k*|e_k^T exp(coeff T) e_1| < errgoal).
 * Complex dtype only.  Replaces pyitensor/tdvp.py:82-172
 * (_lanczos_expm_multiply). */
int dmrg_krylov_expm(const dmrg_heff_t* op, void* x, double coeff_re, double coeff_im,
                     int niter, double tol, double errgoal, int* iters,
                     void* work, size_t work_bytes, void* stream);

/* ---- truncated factorisation --------------------------------------------- */
size_t dmrg_svd_workspace_bytes(int dtype, int m, int n);
/* Truncated SVD of the row-major m x n matrix M followed by the
 * cutoff/maxdim/mindim rule of pyitensor/svd.py:32-68, in FP64.  Two routes,
 * chosen like the reference's (pyitensor/svd.py:108-151):
 *  - real M with min(m,n) >= 16 (and a kept side of at most 2 min(m,n) and
 *    4096): the Gram-matrix route -- the FP64 Gram matrix of the side the
 *    caller keeps orthonormal (M M^T for absorb 0, M^T M for absorb 1, the
 *    smaller side for absorb 2), its eigendecomposition by blocked Jacobi
 *    (dmrg_syev), singular values as square roots of the eigenvalues, the
 *    kept eigenvectors as the orthonormal factor and one FP64 product for
 *    the other (absorb 2 divides by S and, like svd.py:139, falls back to
 *    the exact SVD when the smallest kept value is below 1e-7 of the
 *    largest);
 *  - otherwise one-sided (Hestenes) Jacobi on the min(m,n) columns of M^H
 *    or M (the reference's np.linalg.svd cases), which keeps small singular
 *    values to high relative accuracy.
 * Replaces pyitensor/svd.py:108-195 (_svd_truncated, svd) as used by
 * pyitensor/dmrg.py:336-352.
 *   absorb = 0: left_out = U (m x keep), right_out = S.Vh (keep x n)
 *   absorb = 1: left_out = U.S (m x keep), right_out = Vh (keep x n)
 *   absorb = 2: left_out = U, right_out = Vh (S only in svals)
 * maxdim <= 0 means no cap; cutoff < 0 keeps every value (lossless split).
 * svals (host, min(m,n) doubles, descending), keep and discarded (host)
 * receive the spectrum.  left_out/right_out must hold min(m,n,maxdim)
 * columns/rows. */
int dmrg_svd_truncate(int dtype, int m, int n, const void* M,
                      double cutoff, int maxdim, int mindim, int absorb,
                      void* left_out, void* right_out,
                      double* svals, int* keep, double* discarded,
                      void* work, size_t work_bytes, void* stream);

/* Fixed-rank truncation for the split-TF32 sweep when maxdim binds
 * (cutoff <= 0): keeps k = maxdim vectors found by warm-started subspace
 * iteration (products with theta split-TF32 on tcgen05), polar
 * (Newton-Schulz) orthonormalisation on FP16-split tcgen05 GEMMs, and one
 * correction of the kept basis from a near-FP64 Gram matrix (dmrg_gram's
 * digit method), instead of a full SVD.  Real dtype.  A basis the polar
 * iteration cannot orthonormalise (a direction below its 1e-8 floor, or a
 * non-finite value) returns DMRG_ERR_NOCONV: the caller falls back to
 * dmrg_svd_truncate.
 *   absorb 0: left_out (m x k) orthonormal columns, right_out = left^T theta
 *             (k x n); start = the current RIGHT tensor as kstart x n
 *             (orthonormal rows in a right-canonical MPS)
 *   absorb 1: right_out (k x n) orthonormal rows, left_out = theta right^T
 *             (m x k); start = the current LEFT tensor as m x kstart
 *             (ld kstart, orthonormal columns in a left-canonical MPS)
 * A start that is not orthonormal is orthonormalised first; start vectors
 * beyond kstart are random.  iters (1..8): products with theta per side
 * (1 = kept basis from theta . start).  *discarded receives the weight of
 * theta outside the kept space over |theta|^2.  Stands in for the
 * maxdim-bound case of pyitensor/svd.py:154-195 as used by
 * pyitensor/dmrg.py:336-352 (singular values are not formed). */
size_t dmrg_subspace_workspace_bytes(int m, int n, int k);
int dmrg_subspace_truncate(int m, int n, int k, const void* theta, const void* start, int kstart, int absorb,
                           int iters, void* left_out, void* right_out, double* discarded,
                           void* work, size_t work_bytes, void* stream);

/* Truncation of a large two-site tensor to at most k vectors by subspace
 * iteration plus Rayleigh-Ritz with the cutoff/mindim rule of
 * pyitensor/svd.py:32-68 (maxdim = k): the maxdim-bound case of
 * pyitensor/svd.py:108-151 (Gram route) at bond dimensions where the full
 * eigenproblem of the min(m,n)-sized Gram matrix is not needed.
 * start/kstart/absorb/iters as dmrg_subspace_truncate.
 *   DMRG_PREC_FP64:   every product FP64: Z = theta W from the start basis,
 *                     Ritz pairs of theta^T theta on span(W) from the k x k
 *                     FP64 Gram Z^T Z (dmrg_syev), kept basis
 *                     U = Z E Lambda^(-1/2) made orthonormal to 1e-13 (weak
 *                     directions below a cutoff-dependent fraction of the
 *                     largest Ritz value replaced by an orthonormal
 *                     completion), C = U^T theta; the rule runs on the
 *                     weights |C_j|^2 with the rest of |theta|^2 as forced
 *                     drops; where it keeps fewer than k, or that weight is
 *                     below 10 cutoff + 1e-11, the subspace gets up to two
 *                     more iterations, and a count below k comes from the
 *                     Ritz values of theta theta^T on the kept space.  svals (host, k) receives the
 *                     singular-value estimates.
 *   DMRG_PREC_TF32X3: the basis of dmrg_subspace_truncate keeping k.  With
 *                     cutoff > 0 the weight outside it is |theta - lo ro|^2;
 *                     unless it exceeds the cutoff by more than its error
 *                     (1e-12 + 2e-6 sqrt(weight), relative to |theta|^2) and
 *                     is above 10 cutoff + 1e-11 (the subspace may miss the
 *                     optimal one by a few 1e-12) the call returns
 *                     DMRG_ERR_PRECISION and the caller repeats the bond in
 *                     FP64.  svals (may be NULL) receives the
 *                     FP32-accurate Ritz values of the kept problem (digit
 *                     Gram, FP32 Jacobi).
 * keep receives the kept count (<= k); left_out is written as m x keep,
 * right_out as keep x n (capacity m*k and k*n).  A basis that cannot be
 * made orthonormal returns DMRG_ERR_NOCONV (callers fall back to
 * dmrg_svd_truncate). */
size_t dmrg_subspace_truncate_ex_workspace_bytes(int precision, int m, int n, int k);
int dmrg_subspace_truncate_ex(int precision, int m, int n, int k, const void* theta, const void* start, int kstart,
                              int absorb, int iters, double cutoff, int mindim, void* left_out, void* right_out,
                              double* svals, int* keep, double* discarded, void* work, size_t work_bytes,
                              void* stream);

/* ---- symmetric eigendecomposition ----------------------------------------
 * A (n x n, row-major, ld lda, symmetric) = V diag(w) V^T in FP64 by the
 * parallel cyclic block-Jacobi method: 16-wide blocks, one CTA per block
 * pair running a Jacobi sweep over the 32 x 32 subproblem in shared memory,
 * the rotations applied to A and V as corrections by a second kernel per
 * round; at most 40 sweeps.  w (host, n) receives the eigenvalues in
 * descending order; V (device, n x n, ld ldv; may be NULL) the matching
 * eigenvectors as columns.  Stands in for np.linalg.eigh in
 * pyitensor/svd.py:131-133 and eigh_truncate (pyitensor/svd.py:71-88).
 * DMRG_ERR_NOCONV if the last sweep still rotated.  Synchronises the
 * stream. */
size_t dmrg_syev_workspace_bytes(int n);
int dmrg_syev(int n, const void* A, long long lda, double* w, void* V, long long ldv, int* sweeps, void* work,
              size_t work_bytes, void* stream);

/* ---- tile autotuner of the split-TF32 GEMM ------------------------------
 * The tensor-core GEMM uses 128 x 128 or 128 x 64 output tiles and walks
 * them in groups of `group` M-tiles per N-tile; on the first overwrite-mode
 * call of each shape (M, N, K) on a device the library times both widths in
 * plain order and in groups of 16 and 8 and keeps the fastest.  The shapes
 * of a sweep are functions of (chi_left, chi_right, d, w), so the decisions
 * are effectively keyed on those.  Results do not depend on the choice
 * (every output element sums the same K slices in the same order).  No
 * reference counterpart (the reference's contraction order is chosen per
 * call in Python, pyitensor/kernels.py:298-334). */
/* Turn tuning of new shapes on (1, the default) or off; returns the previous setting. */
int dmrg_autotune_enable(int enable);
/* Copies up to max_entries decisions as 7 ints each (M, N, K, tile width,
 * 1 if the two B splits are issued as one MMA, group, best time in
 * microseconds) into out (may be NULL); returns the number held. */
int dmrg_autotune_entries(int* out, int max_entries);

/* ---- many independent chains at once (FP64 / complex FP64) ----------------
 * Batched forms of the bond-update steps for lock-step sweeps of nprob
 * chains with different bond dimensions (one grouped launch per step).
 * Per-problem shapes come as host arrays of length nprob and device
 * pointers as host arrays of device addresses.  No reference counterpart:
 * the reference sweeps one chain at a time; each batched step computes, per
 * problem, what its single-chain entry point above computes. */
size_t dmrg_batch_gemm_workspace_bytes(int nprob);
/* C_p (m_p x n_p) = A_p (m_p x k_p) . B_p (k_p x n_p): the two-site merges. */
int dmrg_batch_gemm(int dtype, int nprob, const int* m, const int* k, const int* n,
                    const void* const* A, const void* const* B, void* const* C,
                    void* work, size_t work_bytes, void* stream);
/* side 0: Enew_p = dmrg_env_extend_left(E_p, W_p, A_p); side 1: right. */
size_t dmrg_batch_env_workspace_bytes(int side, int dtype, int nprob, const int* chil, const int* d,
                                      const int* chir, const int* wl, const int* wr);
int dmrg_batch_env_extend(int side, int dtype, int nprob, const int* chil, const int* d, const int* chir,
                          const int* wl, const int* wr, const void* const* E, const void* const* W,
                          const void* const* A, void* const* Enew, void* work, size_t work_bytes, void* stream);
/* dmrg_lanczos_ground for every ops[p] (kind 2, FP64 precision, one dtype),
 * x[p] in/out; the recurrence runs in lock step, blocks of steps replayed
 * from captured CUDA graphs when use_graph != 0 (cached per shape and
 * workspace address); each problem stops by the single-chain rule, at most
 * niter steps. */
size_t dmrg_batch_lanczos_workspace_bytes(int nprob, const dmrg_heff_t* ops, int niter);
int dmrg_batch_lanczos_ground(int nprob, const dmrg_heff_t* ops, void* const* x, int niter, double tol,
                              int use_graph, double* energies, int* iters,
                              void* work, size_t work_bytes, void* stream);
/* dmrg_svd_truncate for every M_p (m_p x n_p) in two phases: factor (one CTA
 * per problem) returns keep[p] by the truncation rule of
 * pyitensor/svd.py:32-68 with maxdim[p]; the caller then allocates the
 * outputs (m_p x keep_p, keep_p x n_p) and calls output with the same
 * workspace and the same absorb. */
size_t dmrg_batch_svd_workspace_bytes(int dtype, int nprob, const int* m, const int* n);
int dmrg_batch_svd_factor(int dtype, int nprob, const int* m, const int* n, const void* const* M, double cutoff,
                          const int* maxdim, int mindim, int absorb, int* keep, double* discarded, double* svals,
                          int ld_svals, void* work, size_t work_bytes, void* stream);
int dmrg_batch_svd_output(int dtype, int nprob, const int* m, const int* n, const int* keep, int absorb,
                          void* const* left, void* const* right, void* work, size_t work_bytes, void* stream);

/* ---- Gram matrix ------------------------------------------------------------
 * No counterpart in the reference (its truncation is an SVD,
 * pyitensor/svd.py:32-68): G (k x k, row-major) = X^T X for a real FP64
 * block X (m x k, row-major, leading dimension ld >= k), the orthonormality
 * check of the subspace truncation.  method DMRG_GRAM_FP64: FP64 on the
 * CUDA cores (no workspace); DMRG_GRAM_DIGITS: exact digit products on the
 * tensor cores (columns scaled by powers of two, three 8-bit integer digits
 * multiplied and summed exactly, the 2^-24 tail in FP32), error ~1e-13
 * relative to |x_a| |x_b|, m <= 32768 (DMRG_ERR_ARG beyond).  G is exactly
 * symmetric.  A non-finite entry of X gives DMRG_ERR_NAN (digit method).
 * Synchronises the stream. */
#define DMRG_GRAM_FP64 0
#define DMRG_GRAM_DIGITS 1
size_t dmrg_gram_workspace_bytes(int method, int m, int k);
int dmrg_gram(int method, int m, int k, const void* X, long long ld, void* G, void* work, size_t work_bytes,
              void* stream);

/* ---- bounded-wait probe ----------------------------------------------------
 * No reference counterpart: launches one kernel whose mbarrier wait nothing
 * completes, with the bounded wait of the tcgen05 kernels (~2 s), and
 * returns the status it recorded, DMRG_ERR_TIMEOUT; the device stays
 * usable.  Exercises the timeout path without a fault.  work: >= 256 bytes
 * of device memory.  Synchronises the stream. */
int dmrg_wait_timeout_probe(void* work, size_t work_bytes, void* stream);

/* ---- dense contraction ---------------------------------------------------- */
size_t dmrg_gemm_workspace_bytes(int dtype, int precision, int m, int k, int n);
/* C (m x n) = A (m x k) . B (k x n), all row-major.  Used for the two-site
 * merge theta = A_i . A_{i+1} (pyitensor/dmrg.py:233, Ti * Tj) and for the
 * bond-matrix absorption of one-site TDVP (pyitensor/tdvp.py:300-313). */
int dmrg_gemm(int dtype, int precision, int m, int k, int n, const void* A, const void* B, void* C,
              void* work, size_t work_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DMRG_GB300_H */

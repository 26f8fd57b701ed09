// Truncation of a two-site tensor through the eigendecomposition of a Gram
// matrix, the route pyitensor/svd.py:108-151 takes for min(m, n) >= 16:
// diagonalise M M^T (or M^T M), take the singular values as square roots of
// its eigenvalues, apply the cutoff/maxdim/mindim rule of svd.py:32-68, and
// form the other factor with one product.  The eigensolver is the blocked
// Jacobi of syev.cu.
//
// Three forms:
//   gram_truncate   full route, FP64.  The Gram matrix is taken on the side
//                   the caller keeps orthonormal (rows for absorb 0, columns
//                   for absorb 1), so the kept factor is an eigenvector block
//                   (orthonormal to rounding) and the other factor a plain
//                   product with no division by small singular values;
//                   absorb 2 uses the smaller side like the reference and
//                   divides, falling back (GRAM_FALLBACK) when the smallest
//                   kept value is below 1e-7 of the largest, as svd.py:139.
//   rr_truncate     Rayleigh-Ritz subspace route in FP64 for bonds too large
//                   for the full eigenproblem: Z = theta W from a start basis
//                   W (the orthonormal tensor across the bond), Ritz pairs of
//                   theta^T theta on span(W) from the k x k Gram Z^T Z, kept
//                   basis U = Z E Lambda^(-1/2) corrected to orthonormality,
//                   C = U^T theta, the rule on the weights |C_j|^2.
//   subspace_ritz   the Ritz values of the kept problem after the split-TF32
//                   subspace basis (subspace.cu), for spectra on request.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "heff.cuh"
#include "tf32x3.cuh"

namespace dmrg {

namespace {

inline int grid1(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  return (int)(g < 1 ? 1 : g);
}

// dst (cols x rows, ld ldd) = src^T, src rows x cols (ld lds)
__global__ void gt_transpose_kernel(const double* __restrict__ src, long long lds, int rows, int cols,
                                    double* __restrict__ dst, long long ldd) {
  __shared__ double t[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + j, c = c0 + tx;
    if (r < rows && c < cols) t[j][tx] = src[(long long)r * lds + c];
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int c = c0 + j, r = r0 + tx;
    if (c < cols && r < rows) dst[(long long)c * ldd + r] = t[tx][j];
  }
}

int gt_transpose(const double* src, long long lds, int rows, int cols, double* dst, long long ldd, cudaStream_t s) {
  const dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  if (grid.y > 65535) return DMRG_ERR_ARG;
  gt_transpose_kernel<<<grid, 256, 0, s>>>(src, lds, rows, cols, dst, ldd);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

// X[r * ld + c] *= f[c] (cols) or f[r] (rows)
__global__ void gt_scale_kernel(double* __restrict__ X, long long ld, int rows, int cols,
                                const double* __restrict__ f, int by_row) {
  const long long total = (long long)rows * cols;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / cols), c = (int)(e - (long long)r * cols);
    X[(long long)r * ld + c] *= by_row ? f[r] : f[c];
  }
}

int gt_scale(double* X, long long ld, int rows, int cols, const double* f, int by_row, cudaStream_t s) {
  gt_scale_kernel<<<grid1((long long)rows * cols), 256, 0, s>>>(X, ld, rows, cols, f, by_row);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

__global__ void gt_copy2d_kernel(const double* __restrict__ src, long long lds, double* __restrict__ dst,
                                 long long ldd, int rows, int cols) {
  const long long total = (long long)rows * cols;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / cols), c = (int)(e - (long long)r * cols);
    dst[(long long)r * ldd + c] = src[(long long)r * lds + c];
  }
}

int gt_copy2d(const double* src, long long lds, double* dst, long long ldd, int rows, int cols, cudaStream_t s) {
  gt_copy2d_kernel<<<grid1((long long)rows * cols), 256, 0, s>>>(src, lds, dst, ldd, rows, cols);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

// columns c0..c1-1 of Z (rows x ld) <- uniform(-0.5, 0.5) from a counter hash
__global__ void gt_random_kernel(double* __restrict__ Z, long long ld, int rows, int c0, int c1,
                                 unsigned long long seed) {
  const int w = c1 - c0;
  const long long total = (long long)rows * w;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / w), c = c0 + (int)(e - (long long)r * w);
    unsigned long long z = seed ^ (0x9e3779b97f4a7c15ull * (unsigned long long)((long long)r * 1000003LL + c + 1));
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    Z[(long long)r * ld + c] = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  }
}

// out[r] = sum_c X[r * ld + c]^2, one warp per row
__global__ void gt_rowsq_kernel(const double* __restrict__ X, long long ld, int rows, int cols,
                                double* __restrict__ out) {
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  double acc = 0.0;
  for (int c = lane; c < cols; c += 32) {
    const double v = X[(long long)r * ld + c];
    acc = fma(v, v, acc);
  }
  acc = warp_sum(acc);
  if (lane == 0) out[r] = acc;
}

__global__ void gt_sumsq_kernel(const double* __restrict__ x, long long n, double* __restrict__ out) {
  __shared__ double sh[32];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    s = fma(x[i], x[i], s);
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    s = warp_sum(s);
    if (threadIdx.x == 0) atomicAdd(out, s);
  }
}

// From the Gram matrix G = X^T X (k x k): B = I - (G - I)/2, the
// Newton-Schulz factor of X <- X B, and *dev = max|G - I| (ordered bits)
__global__ void gt_half_dev_kernel(const double* __restrict__ G, int k, double* __restrict__ B,
                                   unsigned long long* __restrict__ dev) {
  const long long total = (long long)k * k;
  unsigned long long mx = 0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / k), c = (int)(e - (long long)r * k);
    const double d = G[e] - (r == c ? 1.0 : 0.0);
    B[e] = (r == c ? 1.0 : 0.0) - 0.5 * d;
    double a = fabs(d);
    if (!(a == a)) a = INFINITY;
    unsigned long long b;
    memcpy(&b, &a, sizeof(b));
    if (b > mx) mx = b;
  }
  if (mx) atomicMax(dev, mx);
}

// C (m x n) = op(A) op(B) in FP64 (tgemm with strides); A is m x k (ld lda)
// or, transposed, k x m; B is k x n (ldb) or, transposed, n x k
int gemm64(int tA, int tB, int m, int n, int k, const double* A, long long lda, const double* B, long long ldb,
           double* C, long long ldc, cudaStream_t s) {
  TGemm g{};
  g.B = ax(1); g.M = ax(m); g.K = ax(k); g.N = ax(n);
  if (!tA) { g.a_m = st(lda); g.a_k = st(1); } else { g.a_m = st(1); g.a_k = st(lda); }
  if (!tB) { g.b_k = st(ldb); g.b_n = st(1); } else { g.b_k = st(1); g.b_n = st(ldb); }
  g.c_m = st(ldc); g.c_n = st(1);
  return tgemm<double>(g, 1.0, A, B, 0.0, C, s);
}

// C <- C - A B (FP64; A rows x k (ld lda), B k x cols (ld ldb))
int gemm64_sub(int rows, int cols, int k, const double* A, long long lda, const double* B, long long ldb, double* C,
               long long ldc, cudaStream_t s) {
  TGemm g{};
  g.B = ax(1); g.M = ax(rows); g.K = ax(k); g.N = ax(cols);
  g.a_m = st(lda); g.a_k = st(1);
  g.b_k = st(ldb); g.b_n = st(1);
  g.c_m = st(ldc); g.c_n = st(1);
  return tgemm<double>(g, -1.0, A, B, 1.0, C, s);
}

}  // namespace

// *out = sum of squares of x (n doubles), on the stream
int sumsq_dev(const double* x, long long n, double* out, cudaStream_t s) {
  DMRG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double), s));
  gt_sumsq_kernel<<<grid1(n), 256, 0, s>>>(x, n, out);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

// ---------------------------------------------------------------- full route
// Workspace: transposed copy (rows route), Gram, Jacobi state, scale vector.
size_t gram_truncate_workspace_bytes(int m, int n, int absorb) {
  const int rows = absorb == 0 || (absorb == 2 && m <= n);
  const size_t c = rows ? m : n;
  const size_t d = sizeof(double);
  return align_up(d * (size_t)m * n) + align_up(d * c * c) + syev_jacobi_workspace_bytes((int)c) +
         align_up(d * c) + 256;
}

// The Gram route of pyitensor/svd.py:108-151 with the keep rule of
// svd.py:32-68.  Returns GRAM_FALLBACK (absorb 2 only) when the smallest kept
// singular value is below 1e-7 of the largest: the caller then uses the
// exact SVD, as the reference does.
int gram_truncate(int m, int n, const double* M, double cutoff, int maxdim, int mindim, int absorb, double* lo,
                  double* ro, double* svals, int* keep, double* disc, int* sweeps, void* work, size_t work_bytes,
                  cudaStream_t s) {
  if (m <= 0 || n <= 0 || !M || !lo || !ro || absorb < 0 || absorb > 2) return DMRG_ERR_ARG;
  if (!work || gram_truncate_workspace_bytes(m, n, absorb) > work_bytes) return DMRG_ERR_WORKSPACE;
  const int rows = absorb == 0 || (absorb == 2 && m <= n);
  const int c = rows ? m : n;        // Gram size (kept side)
  const int r = rows ? n : m;        // contracted dimension
  const int cmin = std::min(m, n);
  const size_t d = sizeof(double);
  char* p = static_cast<char*>(work);
  double* T = reinterpret_cast<double*>(p); p += align_up(d * (size_t)m * n);
  double* G = reinterpret_cast<double*>(p); p += align_up(d * (size_t)c * c);
  void* sw = p; p += syev_jacobi_workspace_bytes(c);
  double* fdev = reinterpret_cast<double*>(p);
  const size_t sw_bytes = syev_jacobi_workspace_bytes(c);
  // G = X^T X with X = M^T (rows route) or M
  if (rows) {
    DMRG_TRY(gt_transpose(M, n, m, n, T, m, s));   // T = M^T (n x m)
    DMRG_TRY(tgemm_gram(T, m, r, c, G, s));
  } else {
    DMRG_TRY(tgemm_gram(M, n, r, c, G, s));
  }
  std::vector<double> w(c);
  DMRG_TRY(syev_jacobi(c, G, c, w.data(), 40, sweeps, sw, sw_bytes, s));
  std::vector<double> sv(cmin);
  for (int i = 0; i < cmin; ++i) sv[i] = std::sqrt(std::max(w[i], 0.0));
  int kp;
  double dc;
  keep_rule(sv.data(), cmin, cutoff, maxdim, std::max(1, mindim), &kp, &dc);
  if (kp > cmin) kp = cmin;
  if (absorb == 2 && !(sv[0] > 0.0 && sv[kp - 1] >= 1e-7 * sv[0])) return GRAM_FALLBACK;
  std::vector<double> f(kp);
  for (int i = 0; i < kp; ++i) f[i] = sv[i] > 0.0 ? 1.0 / sv[i] : 0.0;
  if (rows) {
    // U = E[:, :keep] (m x keep), right = U^T M (keep x n)
    DMRG_TRY(syev_vectors(c, kp, lo, kp, 0, sw, s));
    DMRG_TRY(gemm64(1, 0, kp, n, m, lo, kp, M, n, ro, n, s));
    if (absorb == 2) {
      DMRG_CUDA_TRY(cudaMemcpyAsync(fdev, f.data(), d * kp, cudaMemcpyHostToDevice, s));
      DMRG_TRY(gt_scale(ro, n, kp, n, fdev, 1, s));
    }
  } else {
    // V^T = E[:, :keep]^T (keep x n), left = M V (m x keep)
    DMRG_TRY(syev_vectors(c, kp, ro, n, 1, sw, s));
    DMRG_TRY(gemm64(0, 1, m, kp, n, M, n, ro, n, lo, kp, s));
    if (absorb == 2) {
      DMRG_CUDA_TRY(cudaMemcpyAsync(fdev, f.data(), d * kp, cudaMemcpyHostToDevice, s));
      DMRG_TRY(gt_scale(lo, kp, m, kp, fdev, 0, s));
    }
  }
  // f must outlive its copy
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  if (svals) std::memcpy(svals, sv.data(), d * cmin);
  if (keep) *keep = kp;
  if (disc) *disc = dc;
  return DMRG_OK;
}

// ---------------------------------------------------------------- keep rule on a partial spectrum
// The rule of pyitensor/svd.py:32-68 when only the k largest of c squared
// singular values are known (lam, descending) together with their total:
// the unknown c - k values are the smallest, so with hi = min(maxdim, c) <= k
// they are all forced drops and only their sum enters the rule.  rem: the
// weight fraction outside the k known values when the caller has a better
// estimate than 1 - sum(lam)/total (negative: use that difference).
void keep_rule_partial(const double* lam, int k, int c, double total, double cutoff, int maxdim, int mindim,
                       double rem, int* keep, double* disc) {
  if (!(total > 0.0)) {
    *keep = std::max(1, mindim);
    *disc = 0.0;
    return;
  }
  const int hi = maxdim > 0 ? std::min(maxdim, c) : c;
  const int kk = std::min(k, hi);
  double known = 0.0;
  for (int i = 0; i < k; ++i) known += lam[i] / total;
  // weight of everything beyond the first hi values (forced drops)
  double forced = rem >= 0.0 ? rem : std::max(0.0, 1.0 - known);
  for (int i = kk; i < k; ++i) forced += lam[i] / total;
  const int lo_keep = std::max(1, std::min(mindim, kk));
  int kp = kk;
  double run = forced;
  // drop from the smallest kept upward while the discarded weight stays
  // within the cutoff (never below mindim)
  while (kp > lo_keep && run + lam[kp - 1] / total <= cutoff) {
    run += lam[kp - 1] / total;
    --kp;
  }
  *keep = kp;
  *disc = run;
}

// ---------------------------------------------------------------- Rayleigh-Ritz route (FP64)
namespace {

struct RRWs {
  double *Tt, *W, *Z, *Z2, *E, *G, *B, *f, *acc;
  unsigned long long* dev;
  void* sw;
  size_t sw_bytes;
};

size_t rr_layout(int m, int n, int k, RRWs* w, void* base) {
  const size_t big = (size_t)std::max(m, n);
  const size_t d = sizeof(double);
  char* p = static_cast<char*>(base);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    void* q = p ? p + off : nullptr;
    off += align_up(bytes);
    return q;
  };
  RRWs r;
  r.Tt = static_cast<double*>(take(d * (size_t)m * n));
  r.W = static_cast<double*>(take(d * big * k));
  r.Z = static_cast<double*>(take(d * big * k));
  r.Z2 = static_cast<double*>(take(d * big * k));
  r.E = static_cast<double*>(take(d * (size_t)k * k));
  r.G = static_cast<double*>(take(d * (size_t)k * k));
  r.B = static_cast<double*>(take(d * (size_t)k * k));
  r.f = static_cast<double*>(take(d * k));
  r.acc = static_cast<double*>(take(64));
  r.dev = reinterpret_cast<unsigned long long*>(r.acc + 4);
  r.sw_bytes = syev_jacobi_workspace_bytes(k);
  r.sw = take(r.sw_bytes);
  if (w) *w = r;
  return off;
}

// Directions whose Ritz value is below a fraction `null` of the largest
// carry no weight the truncation can use: Z e_j / sqrt(lambda_j) is
// orthonormal only to ~eps lambda_max / lambda_j, so they are replaced by an
// orthonormal completion (the reference's exact-SVD fallback keeps such
// directions too, with singular values ~0).  With a positive cutoff the
// fraction sits three decades below it (a direction of weight 1e-3 cutoff
// cannot change the kept count unless ~1000 of them pile up), at most 1e-13
// and at least 1e-16, where the orthonormalisation below still converges.
double null_fraction(double cutoff) {
  if (!(cutoff > 0.0)) return 1e-13;
  return std::max(1e-16, std::min(1e-13, 1e-3 * cutoff));
}

int count_nonnull(const std::vector<double>& lam, int k, double null = 1e-13) {
  if (k < 1 || !(lam[0] > 0.0)) return 0;
  int c = 0;
  while (c < k && lam[c] > null * lam[0]) ++c;
  return c;
}

// Gram of Z (rows x kz, ld) and its eigenpairs (host lam, descending; the
// vectors stay in the Jacobi workspace)
int rr_ritz(const double* Z, long long ld, int rows, int kz, RRWs& w, std::vector<double>& lam, cudaStream_t s) {
  DMRG_TRY(tgemm_gram(Z, ld, rows, kz, w.G, s));
  lam.assign(kz, 0.0);
  return syev_jacobi(kz, w.G, kz, lam.data(), 40, nullptr, w.sw, w.sw_bytes, s);
}

// out = Z E[:, :nc] Lambda^(-1/2), then X <- X (I - (X^T X - I)/2) until
// max|X^T X - I| < 1e-13; a basis still far from orthonormal after the
// scaling (weak directions) first gets a second Gram-eigen scaling, whose
// Gram matrix is then well conditioned (as Cholesky-QR run twice).  out and
// tmp: rows x ld buffers; *result is the buffer that holds the basis.
int rr_basis(const double* Z, long long ld, int rows, int kz, int nc, const std::vector<double>& lam, double* out,
             double* tmp, RRWs& w, double** result, cudaStream_t s) {
  DMRG_TRY(syev_vectors(kz, nc, w.E, nc, 0, w.sw, s));
  DMRG_TRY(gemm64(0, 0, rows, nc, kz, Z, ld, w.E, nc, out, ld, s));
  std::vector<double> f(nc);
  for (int j = 0; j < nc; ++j) f[j] = 1.0 / std::sqrt(lam[j]);
  DMRG_CUDA_TRY(cudaMemcpyAsync(w.f, f.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, s));
  DMRG_TRY(gt_scale(out, ld, rows, nc, w.f, 0, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));   // f must outlive its copy
  double* X = out;
  double* Y = tmp;
  double dev = 1.0;
  bool second = false;
  for (int it = 0; it < 6; ++it) {
    DMRG_TRY(tgemm_gram(X, ld, rows, nc, w.G, s));
    DMRG_CUDA_TRY(cudaMemsetAsync(w.dev, 0, sizeof(unsigned long long), s));
    gt_half_dev_kernel<<<grid1((long long)nc * nc), 256, 0, s>>>(w.G, nc, w.B, w.dev);
    DMRG_CHECK_LAUNCH();
    unsigned long long h = 0;
    DMRG_CUDA_TRY(cudaMemcpyAsync(&h, w.dev, sizeof(h), cudaMemcpyDeviceToHost, s));
    DMRG_CUDA_TRY(cudaStreamSynchronize(s));
    std::memcpy(&dev, &h, sizeof(dev));
    if (dev < 1e-13 || it == 5) break;
    if (dev > 0.1 && !second) {
      second = true;
      std::vector<double> l2(nc);
      DMRG_TRY(syev_jacobi(nc, w.G, nc, l2.data(), 40, nullptr, w.sw, w.sw_bytes, s));
      if (!(l2[nc - 1] > 1e-8)) return DMRG_ERR_NOCONV;
      DMRG_TRY(syev_vectors(nc, nc, w.E, nc, 0, w.sw, s));
      DMRG_TRY(gemm64(0, 0, rows, nc, nc, X, ld, w.E, nc, Y, ld, s));
      for (int j = 0; j < nc; ++j) f[j] = 1.0 / std::sqrt(l2[j]);
      DMRG_CUDA_TRY(cudaMemcpyAsync(w.f, f.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, s));
      DMRG_TRY(gt_scale(Y, ld, rows, nc, w.f, 0, s));
      DMRG_CUDA_TRY(cudaStreamSynchronize(s));
      std::swap(X, Y);
      continue;
    }
    DMRG_TRY(gemm64(0, 0, rows, nc, nc, X, ld, w.B, nc, Y, ld, s));
    std::swap(X, Y);
  }
  *result = X;
  return dev < 1e-11 ? DMRG_OK : DMRG_ERR_NOCONV;
}

// Columns nz..nc-1 of the basis U (rows x ld, columns 0..nz-1 orthonormal)
// become an orthonormal completion: random vectors, projected out of U
// twice, orthonormalised by their own Gram matrix (well conditioned).
// spare and spare2 (rows x ld) are scratch.
int rr_complete(double* U, long long ld, int rows, int nz, int nc, double* spare, double* spare2, RRWs& w,
                cudaStream_t s) {
  const int r = nc - nz;
  if (r <= 0) return DMRG_OK;
  double* R = U + nz;
  gt_random_kernel<<<grid1((long long)rows * r), 256, 0, s>>>(U, ld, rows, nz, nc, 0xc0ffee5eedULL + rows);
  DMRG_CHECK_LAUNCH();
  for (int pass = 0; pass < 2 && nz > 0; ++pass) {
    DMRG_TRY(gemm64(1, 0, nz, r, rows, U, ld, R, ld, w.B, r, s));         // T = U^T R  (nz x r)
    DMRG_TRY(gemm64_sub(rows, r, nz, U, ld, w.B, r, R, ld, s));          // R -= U T
  }
  std::vector<double> lam;
  DMRG_TRY(rr_ritz(R, ld, rows, r, w, lam, s));
  if (count_nonnull(lam, r) < r) return DMRG_ERR_NOCONV;
  double* res = nullptr;
  DMRG_TRY(rr_basis(R, ld, rows, r, r, lam, spare, spare2, w, &res, s));
  return gt_copy2d(res, ld, R, ld, rows, r, s);
}

}  // namespace

size_t rr_truncate_workspace_bytes(int m, int n, int k) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  return rr_layout(m, n, k, nullptr, nullptr);
}

// theta (m x n).  absorb 0 keeps an orthonormal LEFT basis, X = the right
// tensor across the bond (kx x n, orthonormal rows); absorb 1 keeps a RIGHT
// basis, X = the left tensor (m x kx, ld kx, orthonormal columns).  Start
// vectors beyond kx are random.  Keeps at most k vectors by the rule of
// pyitensor/svd.py:32-68; svals (host, >= k) receives the singular-value
// estimates of the kept space (nvals of them).
int rr_truncate(int m, int n, int k, const double* theta, const double* X, int kx, int absorb, int iters,
                double cutoff, int mindim, double* lo, double* ro, double* svals, int* nvals, int* keep, double* disc,
                void* work, size_t work_bytes, cudaStream_t s) {
  if (m <= 0 || n <= 0 || k <= 0 || k > std::min(m, n) || kx < 0 || kx > k || (kx > 0 && !X) || iters < 1 ||
      iters > 8 || !theta || !lo || !ro || (absorb != 0 && absorb != 1))
    return DMRG_ERR_ARG;
  if (!work || rr_truncate_workspace_bytes(m, n, k) > work_bytes) return DMRG_ERR_WORKSPACE;
  RRWs w;
  rr_layout(m, n, k, &w, work);
  const double nul = null_fraction(cutoff);
  const double* Th = theta;
  int M = m, N = n;
  if (absorb == 1) {
    DMRG_TRY(gt_transpose(theta, n, m, n, w.Tt, m, s));
    Th = w.Tt; M = n; N = m;
    if (kx > 0) DMRG_TRY(gt_copy2d(X, kx, w.W, k, N, kx, s));
  } else if (kx > 0) {
    DMRG_TRY(gt_transpose(X, n, kx, n, w.W, k, s));
  }
  DMRG_CUDA_TRY(cudaMemsetAsync(w.acc, 0, 64, s));
  gt_sumsq_kernel<<<grid1((long long)m * n), 256, 0, s>>>(theta, (long long)m * n, w.acc);
  DMRG_CHECK_LAUNCH();
  int kw = k;
  std::vector<double> lam;
  double* res = nullptr;
  if (kx < k) {
    gt_random_kernel<<<grid1((long long)N * (k - kx)), 256, 0, s>>>(w.W, k, N, kx, k, 0x7a11ce5eedULL + N);
    DMRG_CHECK_LAUNCH();
    // an orthonormal basis of the start block
    DMRG_TRY(rr_ritz(w.W, k, N, k, w, lam, s));
    kw = count_nonnull(lam, k);
    if (kw < 1) return DMRG_ERR_NOCONV;
    DMRG_TRY(rr_basis(w.W, k, N, k, kw, lam, w.Z, w.Z2, w, &res, s));
    if (res != w.W) DMRG_TRY(gt_copy2d(res, k, w.W, k, N, kw, s));
  }
  double hacc = 0.0;
  DMRG_CUDA_TRY(cudaMemcpyAsync(&hacc, w.acc, sizeof(double), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  if (!(hacc == hacc)) return DMRG_ERR_NAN;
  // Where the cutoff binds (fewer than k kept) or the weight beyond the
  // subspace is within reach of it, the rule's forced drops are that weight,
  // so a subspace short of the optimal one by ~cutoff weight shifts the kept
  // count along a flat spectrum; up to two more iterations
  // (W = orth(Th^T U), then again) close that gap.
  double* C = nullptr;
  std::vector<double> wt;
  int kp = 0;
  for (int round = 0;; ++round) {
    for (int it = 0;; ++it) {
      DMRG_TRY(gemm64(0, 0, M, kw, N, Th, N, w.W, k, w.Z, k, s));   // Z = Th W
      DMRG_TRY(rr_ritz(w.Z, k, M, kw, w, lam, s));
      const int nz = count_nonnull(lam, kw, nul);
      if (nz < 1) return DMRG_ERR_NOCONV;
      if (it + 1 >= (round == 0 ? iters : 1)) break;
      // W = orth(Th^T orth(Z))
      DMRG_TRY(rr_basis(w.Z, k, M, kw, nz, lam, w.Z2, w.W, w, &res, s));
      DMRG_TRY(gemm64(1, 0, N, nz, M, Th, N, res, k, w.Z, k, s));
      DMRG_TRY(rr_ritz(w.Z, k, N, nz, w, lam, s));
      kw = count_nonnull(lam, nz, nul);
      if (kw < 1) return DMRG_ERR_NOCONV;
      DMRG_TRY(rr_basis(w.Z, k, N, nz, kw, lam, w.W, w.Z2, w, &res, s));
      if (res != w.W) DMRG_TRY(gt_copy2d(res, k, w.W, k, N, kw, s));
    }
    const int nz = count_nonnull(lam, kw, nul);
    // U (M x kw, ld k): Ritz basis of the resolved directions, an
    // orthonormal completion for the rest; C = U^T Th
    DMRG_TRY(rr_basis(w.Z, k, M, kw, nz, lam, w.Z2, w.W, w, &res, s));
    double* other = res == w.Z2 ? w.W : w.Z2;
    if (kw > nz) DMRG_TRY(rr_complete(res, k, M, nz, kw, w.Z, other, w, s));
    C = other;
    DMRG_TRY(gemm64(1, 0, kw, N, M, res, k, Th, N, C, N, s));              // C = U^T Th (kw x N)
    // the weight of theta along each kept direction, |C_j|^2 = u_j^T theta
    // theta^T u_j (one power beyond the Ritz value, and exactly what the
    // truncation keeps); the rule of pyitensor/svd.py:32-68 runs on these,
    // the rest of |theta|^2 being the forced drops
    gt_rowsq_kernel<<<(kw + 7) / 8, 256, 0, s>>>(C, N, kw, N, w.f);
    DMRG_CHECK_LAUNCH();
    wt.assign(kw, 0.0);
    DMRG_CUDA_TRY(cudaMemcpyAsync(wt.data(), w.f, sizeof(double) * kw, cudaMemcpyDeviceToHost, s));
    DMRG_CUDA_TRY(cudaStreamSynchronize(s));
    double dc;
    keep_rule_partial(wt.data(), kw, std::min(m, n), hacc, cutoff, k, std::max(1, mindim), -1.0, &kp, &dc);
    double kept_all = 0.0;
    for (int j = 0; j < kw; ++j) kept_all += wt[j];
    const double rem = hacc > 0.0 ? std::max(0.0, 1.0 - kept_all / hacc) : 0.0;
    // one product with the previous basis leaves the subspace a few 1e-12
    // (of the total weight) short of the optimal one: within that of the
    // cutoff the rule's answer is not settled yet
    const bool near = rem < 10.0 * cutoff + 1e-11;
    if (!(cutoff > 0.0 && (kp < kw || near) && round < 2)) break;
    // W = orth(Th^T U), then the next round from it
    DMRG_TRY(gemm64(1, 0, N, kw, M, Th, N, res, k, w.Z, k, s));
    const int kz = kw;
    DMRG_TRY(rr_ritz(w.Z, k, N, kz, w, lam, s));
    kw = count_nonnull(lam, kz, nul);
    if (kw < 1) return DMRG_ERR_NOCONV;
    DMRG_TRY(rr_basis(w.Z, k, N, kz, kw, lam, w.W, w.Z2, w, &res, s));
    if (res != w.W) DMRG_TRY(gt_copy2d(res, k, w.W, k, N, kw, s));
  }
  double* U = res;
  if (cutoff > 0.0 && kp < kw) {
    // the cutoff binds: the rule needs the singular values of theta within
    // the kept space, not the weights of a basis only approximately aligned
    // with them -- Ritz pairs of theta theta^T on span(U) from C C^T (FP64)
    DMRG_TRY(gemm64(0, 1, kw, kw, N, C, N, C, N, w.G, kw, s));
    std::vector<double> l2(kw);
    DMRG_TRY(syev_jacobi(kw, w.G, kw, l2.data(), 40, nullptr, w.sw, w.sw_bytes, s));
    double dc;
    keep_rule_partial(l2.data(), kw, std::min(m, n), hacc, cutoff, k, std::max(1, mindim), -1.0, &kp, &dc);
    DMRG_TRY(syev_vectors(kw, kp, w.E, kp, 0, w.sw, s));
    DMRG_TRY(gemm64(0, 0, M, kp, kw, U, k, w.E, kp, w.Z, k, s));       // U E   (M x kp)
    DMRG_TRY(gemm64(1, 0, kp, N, kw, w.E, kp, C, N, U, N, s));         // E^T C (kp x N)
    C = U;
    U = w.Z;
    wt.assign(l2.begin(), l2.end());
  }
  if (absorb == 0) {
    DMRG_TRY(gt_copy2d(U, k, lo, kp, m, kp, s));
    DMRG_TRY(gt_copy2d(C, N, ro, n, kp, n, s));
  } else {
    DMRG_TRY(gt_transpose(C, N, kp, m, lo, kp, s));     // left = C^T (m x kp)
    DMRG_TRY(gt_transpose(U, k, n, kp, ro, n, s));      // right = U^T (kp x n)
  }
  double kept = 0.0;
  for (int j = 0; j < kp; ++j) kept += wt[j];
  if (svals)
    for (int i = 0; i < kw; ++i) svals[i] = std::sqrt(std::max(wt[i], 0.0));
  if (nvals) *nvals = kw;
  if (keep) *keep = kp;
  if (disc) *disc = hacc > 0.0 ? std::max(0.0, 1.0 - kept / hacc) : 0.0;
  return DMRG_OK;
}

// ---------------------------------------------------------------- Ritz values after the split-TF32 subspace
size_t subspace_ritz_workspace_bytes(int m, int n, int k) {
  const size_t d = sizeof(double);
  const size_t big = (size_t)std::max(m, n);
  return align_up(64) + align_up(d * big * k) + align_up(d * (size_t)k * k) + syev_jacobi_workspace_bytes(k) +
         gram_digits_workspace_bytes((int)big, k) + align_up(64);
}

// lo (m x k, ld k) and ro (k x n) are the fixed-rank factors of theta from
// subspace_truncate (absorb 0: lo orthonormal columns, ro = lo^T theta;
// absorb 1: ro orthonormal rows, lo = theta ro^T).  svals (k) receives the
// Ritz singular values of the kept problem: the square roots of the
// eigenvalues of the k x k Gram of the other factor (digit Gram, Jacobi in
// FP32: the factors are FP32-accurate, and so are these values).
int subspace_ritz(int m, int n, int k, int absorb, double* lo, double* ro, double* svals, void* work,
                  size_t work_bytes, cudaStream_t s) {
  if (subspace_ritz_workspace_bytes(m, n, k) > work_bytes) return DMRG_ERR_WORKSPACE;
  const size_t d = sizeof(double);
  const size_t big = (size_t)std::max(m, n);
  char* p = static_cast<char*>(work);
  int* err = reinterpret_cast<int*>(p); p += align_up(64);
  double* T1 = reinterpret_cast<double*>(p); p += align_up(d * big * k);
  double* G = reinterpret_cast<double*>(p); p += align_up(d * (size_t)k * k);
  void* sw = p; p += syev_jacobi_workspace_bytes(k);
  void* gw = p;
  const size_t gw_bytes = gram_digits_workspace_bytes((int)big, k);
  DMRG_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  if (absorb == 0) {
    DMRG_TRY(gt_transpose(ro, n, k, n, T1, k, s));      // T1 = ro^T (n x k)
    DMRG_TRY(gram_digits(T1, k, n, k, G, gw, gw_bytes, err, s));
  } else {
    DMRG_TRY(gram_digits(lo, k, m, k, G, gw, gw_bytes, err, s));
  }
  std::vector<double> lam(k);
  DMRG_TRY(syev_jacobi(k, G, k, lam.data(), 40, nullptr, sw, syev_jacobi_workspace_bytes(k), s, 1));
  int e = 0;
  DMRG_CUDA_TRY(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  if (e != 0) return e;
  for (int i = 0; i < k; ++i) svals[i] = std::sqrt(std::max(lam[i], 0.0));
  return DMRG_OK;
}

}  // namespace dmrg

// Truncation of a two-site tensor by warm-started subspace iteration, for
// the split-TF32 sweep at large bond dimension when the kept dimension is
// fixed by maxdim (cutoff <= 0): no eigensolver, only GEMMs on the tensor
// cores, one of them a Gram matrix accurate to ~1e-13 (exact digit products,
// gram.cu).
//
//   keep the left factor (absorb 0), starting from X = the tensor across the
//   bond (k x n, orthonormal rows in a right-canonical MPS):
//     W = orth(X^T)      n x k
//     Z = theta W        m x k     (iters times, with W = orth(theta^T Q)
//     Q = orth(Z)        m x k      between two rounds)
//     C = Q^T theta      right factor (k x n); left factor Q
//   keep the right factor (absorb 1): the same on theta^T, returning
//     left = theta Q (m x k) and right = Q^T (k x n, orthonormal rows).
// The products with theta are split-TF32.
//
// orth() is the polar factor of the block by Newton-Schulz iterations, which
// are GEMMs only (FP16-split operand pairs on the tensor cores); the final
// left/right basis gets one more correction from the near-FP64 Gram matrix
// so that it is orthonormal to ~1e-13 (a basis that is only FP32-orthonormal
// lets the norm environment drift along the chain).
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "tf32x3.cuh"

namespace dmrg {

namespace {

__device__ __forceinline__ float hash_uniform(unsigned long long seed, long long i) {
  unsigned long long z = seed ^ (0x9e3779b97f4a7c15ull * (unsigned long long)(i + 1));
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  return static_cast<float>((z >> 40) * (1.0 / 16777216.0)) - 0.5f;
}

__global__ void random_fill_kernel(double* __restrict__ Z, long long ldz, int m, int c0, int c1, unsigned long long seed) {
  const long long total = (long long)m * (c1 - c0);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / (c1 - c0)), c = c0 + (int)(i % (c1 - c0));
    unsigned long long z = seed ^ (0x9e3779b97f4a7c15ull * (unsigned long long)(r * 131071 + c + 1));
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    Z[(long long)r * ldz + c] = ((z >> 11) * (1.0 / 9007199254740992.0)) - 0.5;
  }
}

// copy rows of a (rows x cols, ld) block into dst (ld_dst)
__global__ void copy2d_kernel(const double* __restrict__ src, long long lds, double* __restrict__ dst, long long ldd,
                              int rows, int cols) {
  const long long total = (long long)rows * cols;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    dst[(long long)r * ldd + c] = src[(long long)r * lds + c];
  }
}

__global__ void sumsq_kernel(const double* __restrict__ x, long long n, double* __restrict__ out) {
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

inline int egrid(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  if (g < 1) g = 1;
  return (int)g;
}

// dst (cols x rows, ld = ldd) = src^T, src rows x cols with leading dim lds
__global__ void transpose_kernel(const double* __restrict__ src, long long lds, int rows, int cols,
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

int transpose(const double* src, long long lds, int rows, int cols, double* dst, long long ldd, cudaStream_t s) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  if (grid.y > 65535) return DMRG_ERR_ARG;
  transpose_kernel<<<grid, 256, 0, s>>>(src, lds, rows, cols, dst, ldd);
  DMRG_CHECK_LAUNCH();
  return DMRG_OK;
}

// ---------------------------------------------------------------- polar orthonormalisation
// Orthonormal basis of range(Z) as the polar factor of Z, by Newton-Schulz
// iterations that use only (split-TF32) GEMMs:
//   columns scaled to unit norm, then /sqrt(k) so every singular value <= 1;
//   quintic steps X <- aX + X(bA + cA^2), A = X^T X, with (a,b,c) chosen so
//   that small singular values grow by ~3.4x per step while all stay in
//   (0, 1.3);
//   cubic steps X <- X(1.5 I - 0.5 A) until max|A - I| < tol.
// Directions of Z at the FP32 noise level (or exactly dependent ones, after
// a tiny random perturbation) become orthonormal completions, so the result
// is orthonormal whatever the conditioning of Z.

// f[c] = extra / |Z[:, c]| (0 for a zero column), from the squared norms
__global__ void col_factor_kernel(double* __restrict__ n2, int k, double extra) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < k) n2[c] = n2[c] > 0.0 ? extra / sqrt(n2[c]) : 0.0;
}

// Z[r][c] = Z[r][c] f[c] + eps u(r k + c), u uniform in [-1/2, 1/2): unit
// columns scaled by 1/sqrt(k), plus a tiny random perturbation that keeps
// exactly dependent directions from staying at 0.  Row r = blockIdx.y.
__global__ void scale_perturb_kernel(double* __restrict__ Z, long long ld, int k, const double* __restrict__ f,
                                     double eps, unsigned long long seed) {
  const int r = blockIdx.y, c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  const long long i = (long long)r * k + c;
  double* z = Z + (long long)r * ld + c;
  // FP64 as the column norms: with both in FP32 one ill-conditioned case
  // (a half-random start, tests/test_gpu_truncation.py) no longer converged
  // within the step limit.  The draw is widened from its bit pattern.
  *z = fma(*z, f[c], eps * widen(hash_uniform(seed, i)));
}

// part[y][c] = sum of Z[r][c]^2 over the rows of chunk y (rows 32 y + ty +
// 32 gridDim.y j for row lane ty): blocks of 32 columns x 32 row lanes
// (coalesced 256-byte row segments), gridDim.y row chunks so that 1024
// columns spread over 4 x 32 SMs; lanes combined in shared memory in a
// fixed order (deterministic)
constexpr int COLSQ_CHUNKS = 4;
__global__ void __launch_bounds__(1024) colsq_kernel(const double* __restrict__ Z, long long ld, int m, int k,
                                                     double* __restrict__ part) {
  __shared__ double sh[32][33];
  const int lane = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + lane;
  double s = 0.0;
  if (c < k)
    for (int r = blockIdx.y * 32 + ty; r < m; r += 32 * gridDim.y) {
      const double z = Z[(long long)r * ld + c];
      s = fma(z, z, s);
    }
  sh[ty][lane] = s;
  __syncthreads();
  if (ty == 0 && c < k) {
    double t = 0.0;
    for (int j = 0; j < 32; ++j) t += sh[j][lane];
    part[(long long)blockIdx.y * k + c] = t;
  }
}

// n2[c] = sum of the chunk partials, in chunk order
__global__ void colsq_sum_kernel(const double* __restrict__ part, int chunks, int k, double* __restrict__ n2) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  double t = 0.0;
  for (int y = 0; y < chunks; ++y) t += part[(long long)y * k + c];
  n2[c] = t;
}

// B = b*A + c*I  (k x k), also reports max|A - I| into *dev.  Blocks walk
// whole rows (row r = blockIdx.y + j gridDim.y); the grid is two blocks per
// SM, so it ends in at most POLY_BLOCKS atomics on *dev (one per block):
// one block per row of a 1024 x 1024 matrix spent ~10 us in serialised
// atomics.
constexpr int POLY_BLOCKS = 2 * 152;
inline dim3 poly_grid(int k) { return dim3(1, k < POLY_BLOCKS ? k : POLY_BLOCKS); }
__global__ void poly_kernel(const double* __restrict__ A, int k, double b, double c, double* __restrict__ B,
                            unsigned long long* __restrict__ dev) {
  double mx = 0.0;
  for (int r = blockIdx.y; r < k; r += gridDim.y)
    for (int cc = threadIdx.x; cc < k; cc += blockDim.x) {
      const long long i = (long long)r * k + cc;
      const double a = A[i];
      B[i] = b * a + (r == cc ? c : 0.0);
      const double dv = fabs(a - (r == cc ? 1.0 : 0.0));
      mx = dv <= mx ? mx : (dv == dv ? dv : INFINITY);   // a non-finite entry reports +inf
    }
  // block max first, then one atomic per block (max of non-negative doubles
  // via their bit patterns): a per-thread atomic on one address serialises
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    atomicMax(dev, __double_as_longlong(m));
  }
}

// FP16 operand pair of x * scale (scale a power of two that keeps |x scale|
// inside the FP16 range): hi = fp16(x s), lo = fp16(x s - hi).  Computed in
// FP32 from x rounded to FP32 (the pair resolves 22 bits, FP32 holds 24):
// FP64 arithmetic and conversions run at a small fraction of the FP32 rate
// on GB300.
__device__ __forceinline__ void split_h(float x, float scale, __half& hi, __half& lo) {
  const float v = x * scale;
  hi = __float2half_rn(v);
  lo = __float2half_rn(v - __half2float(hi));
}

// B = b*A + c*I (k x k) stored as the FP16 operand pair [r][Kk] (scaled) of
// the next GEMM; also reports max|A - I| into *dev
__global__ void poly_split_kernel(const double* __restrict__ A, int k, double b, double c, double scale,
                                  __half* __restrict__ hi, __half* __restrict__ lo, int Kk,
                                  unsigned long long* __restrict__ dev) {
  // whole rows per block as in poly_kernel (one atomic per block); FP32
  // arithmetic (A carries the FP32-level accuracy of the split products)
  const float bf = static_cast<float>(b), cf = static_cast<float>(c), sf = static_cast<float>(scale);
  float mxf = 0.f;
  for (int r = blockIdx.y; r < k; r += gridDim.y)
    for (int cc = threadIdx.x; cc < k; cc += blockDim.x) {
      const float a = narrow(A[(long long)r * k + cc]);
      split_h(fmaf(bf, a, r == cc ? cf : 0.f), sf, hi[(long long)r * Kk + cc], lo[(long long)r * Kk + cc]);
      const float dv = fabsf(a - (r == cc ? 1.f : 0.f));
      if (!(dv <= mxf)) mxf = dv == dv ? dv : INFINITY;   // a non-finite entry reports +inf
    }
  double mx = mxf;
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    atomicMax(dev, __double_as_longlong(m));
  }
}

// FP16 operand pairs of X (m x k, ld) in both layouts the iteration reads:
// row-major xr[r][Kk] and transposed xt[c][Km] (through a 32 x 33 tile);
// padding columns are written as zero
__global__ void split_both_kernel(const double* __restrict__ X, long long ld, int m, int k, int Km, int Kk,
                                  double scale, __half* __restrict__ xr_hi, __half* __restrict__ xr_lo,
                                  __half* __restrict__ xt_hi, __half* __restrict__ xt_lo) {
  __shared__ float t[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const float sf = static_cast<float>(scale);
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + j, c = c0 + tx;
    const float v = (r < m && c < k) ? narrow(X[(long long)r * ld + c]) : 0.f;
    t[j][tx] = v;
    if (r < m && c < Kk) split_h(v, sf, xr_hi[(long long)r * Kk + c], xr_lo[(long long)r * Kk + c]);
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int c = c0 + j, r = r0 + tx;
    if (c < k && r < Km) split_h(t[tx][j], sf, xt_hi[(long long)c * Km + r], xt_lo[(long long)c * Km + r]);
  }
}

inline int pad64s(long long x) { return (int)((x + 63) / 64 * 64); }

// X (m x k, ld) = (hi + lo) / scale from the row-major FP16 operand pair of
// the polar iterate ([r][Kk])
__global__ void pair_to_f64_kernel(const __half* __restrict__ hi, const __half* __restrict__ lo, int Kk, int m, int k,
                                   float inv_scale, double* __restrict__ X, long long ld) {
  const long long total = (long long)m * k;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / k), c = (int)(i - (i / k) * k);
    const long long o = (long long)r * Kk + c;
    X[(long long)r * ld + c] = widen((__half2float(hi[o]) + __half2float(lo[o])) * inv_scale);
  }
}

// FP16 operand arrays of the polar iteration ([rows][K] pairs of scaled
// values, K padded to 64):
//   xt  X^T [k][Km]  both operands of the Gram X^T X (K = m)
//   xr  X   [m][Kk]  A operand of X B (K = k); two of them, because the
//                    GEMM that reads one writes the next iterate's split
//   as  A   [k][Kk]  A operand of A (c A + b I)
//   ps  c A + b I    B operand of the same product
//   bs  B   [k][Kk]  B operand of X B (B is symmetric)
// Each GEMM epilogue writes the splits the next GEMM reads, so the
// iteration runs without separate split kernels.  The values are bounded
// (|X| <= 1, |A| <= 1.5, |c A + b I| < 8, |B| < 14), so fixed power-of-two
// scales keep every pair inside the FP16 range.
struct PolarSplits {
  __half *xt_hi, *xt_lo, *xr_hi[2], *xr_lo[2], *as_hi, *as_lo, *ps_hi, *ps_lo, *bs_hi, *bs_lo;
};
constexpr double SX = 4096.0, SA = 4096.0, SP = 4096.0, SB = 2048.0;

size_t polar_split_bytes(int m, int k) {
  const size_t Km = pad64s(m), Kk = pad64s(k), f = sizeof(__half);
  return 2 * align_up(f * k * Km, 1024) + 4 * align_up(f * m * Kk, 1024) + 6 * align_up(f * k * Kk, 1024);
}

PolarSplits polar_splits(void* base, int m, int k) {
  const size_t Km = pad64s(m), Kk = pad64s(k), f = sizeof(__half);
  char* p = static_cast<char*>(base);
  auto take = [&](size_t n) {
    __half* r = reinterpret_cast<__half*>(p);
    p += align_up(f * n, 1024);
    return r;
  };
  PolarSplits ps;
  ps.xt_hi = take(k * Km);
  ps.xt_lo = take(k * Km);
  for (int i = 0; i < 2; ++i) {
    ps.xr_hi[i] = take(m * Kk);
    ps.xr_lo[i] = take(m * Kk);
  }
  ps.as_hi = take(k * Kk);
  ps.as_lo = take(k * Kk);
  ps.ps_hi = take(k * Kk);
  ps.ps_lo = take(k * Kk);
  ps.bs_hi = take(k * Kk);
  ps.bs_lo = take(k * Kk);
  return ps;
}

// The split-TF32 iterations leave |X^T X - I| at the 1e-6 level, which is
// what a product accurate to ~5e-7 can resolve.  A left basis that is only
// that orthonormal makes the norm environment drift by ~N x 1e-6 over a
// chain, so a kept basis gets one correction with a Gram matrix from exact
// digit products (~1e-13, gram.cu; the FP64 CUDA-core Gram beyond its size
// limit):
//   E = X^T X - I,  X <- X (I - E/2)   (residual O(E^2)),
// where the product X (E/2) only needs the split-TF32 relative accuracy
// because E is already tiny.
int orth_fp64_correct(double* Z, long long ld, int m, int k, double* A, double* B, unsigned long long* dev, void* gw,
                      size_t gw_bytes, int* err, cudaStream_t s) {
  // the Gram from exact digit products on the tensor cores; the FP64
  // CUDA-core Gram beyond its size limit
  const int st = gram_digits(Z, ld, m, k, A, gw, gw_bytes, err, s);
  if (st == DMRG_ERR_ARG || st == DMRG_ERR_WORKSPACE) DMRG_TRY(tgemm_gram(Z, ld, m, k, A, s));
  else DMRG_TRY(st);
  DMRG_CUDA_TRY(cudaMemsetAsync(dev, 0, sizeof(unsigned long long), s));
  poly_kernel<<<poly_grid(k), 256, 0, s>>>(A, k, -0.5, 0.5, B, dev);
  DMRG_CHECK_LAUNCH();
  return tf32x3_gemm_ex(0, 0, m, k, k, 1.f, Z, ld, B, k, 1, Z, ld, gw, err, s);
}

// max|A - I| of a k x k Gram matrix (host value; synchronises the stream)
int gram_deviation(const double* A, int k, double* B, unsigned long long* dev, double* out, cudaStream_t s) {
  DMRG_CUDA_TRY(cudaMemsetAsync(dev, 0, sizeof(unsigned long long), s));
  poly_kernel<<<poly_grid(k), 256, 0, s>>>(A, k, 1.0, 0.0, B, dev);
  DMRG_CHECK_LAUNCH();
  unsigned long long h = 0;
  DMRG_CUDA_TRY(cudaMemcpyAsync(&h, dev, sizeof(h), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  memcpy(out, &h, sizeof(double));
  return DMRG_OK;
}

int orth_polar(double* Z, long long ld, int m, int k, double* A, double* B, double* n2, unsigned long long* dev,
               void* gw, size_t gw_bytes, void* splits, int* err, bool exact, cudaStream_t s) {
  const int Km = pad64s(m), Kk = pad64s(k);
  const PolarSplits ps = polar_splits(splits, m, k);
  // the K padding of the split arrays must read as zero
  if (Km != m || Kk != k) DMRG_CUDA_TRY(cudaMemsetAsync(splits, 0, polar_split_bytes(m, k), s));
  const dim3 sgrid((k + 31) / 32, (Km > m ? Km : m) / 32 + 1);
  if (sgrid.y > 65535 || m > 65535 || k > 65535) return DMRG_ERR_ARG;
  // A = X^T X (FP64), optionally with its scaled split for A (c A + b I)
  auto gram = [&](bool with_split) -> int {
    GemmOut g{};
    g.C = A; g.ldm = k; g.ldn = 1; g.M = k; g.N = k; g.out_f64 = 1; g.alpha = (float)(1.0 / (SX * SX));
    if (with_split) { g.rhi = ps.as_hi; g.rlo = ps.as_lo; g.rld = Kk; g.split_scale = SA; }
    return f16x3_gemm_split(ps.xt_hi, ps.xt_lo, ps.xt_hi, ps.xt_lo, k, k, Km, g, err, s);
  };
  // an input that is already orthonormal (the usual warm start) skips the
  // iterations
  double d0 = 1.0;
  split_both_kernel<<<sgrid, 256, 0, s>>>(Z, ld, m, k, Km, Kk, SX, ps.xr_hi[0], ps.xr_lo[0], ps.xt_hi, ps.xt_lo);
  DMRG_CHECK_LAUNCH();
  DMRG_TRY(gram(false));
  DMRG_TRY(gram_deviation(A, k, B, dev, &d0, s));
  if (d0 < 1e-5) return exact ? orth_fp64_correct(Z, ld, m, k, A, B, dev, gw, gw_bytes, err, s) : DMRG_OK;
  // column scaling: unit columns / sqrt(k)  (=> all singular values <= 1)
  // the chunk partials go to B (k x k, free until the final correction)
  const int chunks = k >= COLSQ_CHUNKS ? COLSQ_CHUNKS : 1;
  colsq_kernel<<<dim3((k + 31) / 32, chunks), 1024, 0, s>>>(Z, ld, m, k, B);
  DMRG_CHECK_LAUNCH();
  colsq_sum_kernel<<<(k + 255) / 256, 256, 0, s>>>(B, chunks, k, n2);
  DMRG_CHECK_LAUNCH();
  col_factor_kernel<<<(k + 255) / 256, 256, 0, s>>>(n2, k, 1.0 / sqrt((double)k));
  DMRG_CHECK_LAUNCH();
  // the perturbation (spectral norm ~5e-8) stays below the rounding of the
  // FP16 operand pairs (~2.4e-7 of |X|), so it adds no error of its own
  scale_perturb_kernel<<<dim3((k + 255) / 256, m), 256, 0, s>>>(Z, ld, k, n2, 1e-7 / sqrt((double)m),
                                                                0x5eed5ull + (unsigned)k);
  DMRG_CHECK_LAUNCH();
  split_both_kernel<<<sgrid, 256, 0, s>>>(Z, ld, m, k, Km, Kk, SX, ps.xr_hi[0], ps.xr_lo[0], ps.xt_hi, ps.xt_lo);
  DMRG_CHECK_LAUNCH();
  int cur = 0;
  // 14 quintic steps (3.4x per step for small singular values) lift a
  // direction from the ~2e-8 perturbation level into the band [0.7, 1.2];
  // a few cubic steps then converge quadratically.  The iterates live only
  // as their FP16 operand pairs (written by each X B epilogue); the FP64
  // basis is formed once from the final pair.
  const int quintic = 14, cubic_max = 16;
  double d = 1.0;
  for (int it = 0; it < quintic + cubic_max; ++it) {
    const bool q = it < quintic;
    DMRG_TRY(gram(q));
    // X B, written as the next iterate's two splits only
    GemmOut xb{};
    xb.C = nullptr; xb.M = m; xb.N = k; xb.out_f64 = 1; xb.alpha = (float)(1.0 / (SX * SB));
    xb.rhi = ps.xr_hi[1 - cur]; xb.rlo = ps.xr_lo[1 - cur]; xb.rld = Kk;
    xb.thi = ps.xt_hi; xb.tlo = ps.xt_lo; xb.tld = Km; xb.split_scale = SX;
    if (q) {
      // B = a I + A (b I + c A) (split only), so that X <- X B is the quintic
      // step a X + b X A + c X A^2 as one product
      const double a = 3.4445, b = -4.7750, c = 2.0315;
      DMRG_CUDA_TRY(cudaMemsetAsync(dev, 0, sizeof(unsigned long long), s));
      poly_split_kernel<<<poly_grid(k), 256, 0, s>>>(A, k, c, b, SP, ps.ps_hi, ps.ps_lo, Kk, dev);
      DMRG_CHECK_LAUNCH();
      GemmOut b2{};
      b2.C = nullptr; b2.M = k; b2.N = k; b2.out_f64 = 1; b2.alpha = (float)(1.0 / (SA * SP)); b2.diag = a;
      b2.rhi = ps.bs_hi; b2.rlo = ps.bs_lo; b2.rld = Kk; b2.split_scale = SB;
      DMRG_TRY(f16x3_gemm_split(ps.as_hi, ps.as_lo, ps.ps_hi, ps.ps_lo, k, k, Kk, b2, err, s));
    } else {
      // convergence check on A, then X <- X (1.5 I - 0.5 A)
      DMRG_CUDA_TRY(cudaMemsetAsync(dev, 0, sizeof(unsigned long long), s));
      poly_split_kernel<<<poly_grid(k), 256, 0, s>>>(A, k, -0.5, 1.5, SB, ps.bs_hi, ps.bs_lo, Kk, dev);
      DMRG_CHECK_LAUNCH();
      unsigned long long h = 0;
      DMRG_CUDA_TRY(cudaMemcpyAsync(&h, dev, sizeof(h), cudaMemcpyDeviceToHost, s));
      DMRG_CUDA_TRY(cudaStreamSynchronize(s));
      memcpy(&d, &h, sizeof(d));
      if (d < 5e-6) break;
    }
    DMRG_TRY(f16x3_gemm_split(ps.xr_hi[cur], ps.xr_lo[cur], ps.bs_hi, ps.bs_lo, m, k, Kk, xb, err, s));
    cur = 1 - cur;
  }
  pair_to_f64_kernel<<<egrid((long long)m * k), 256, 0, s>>>(ps.xr_hi[cur], ps.xr_lo[cur], Kk, m, k,
                                                              (float)(1.0 / SX), Z, ld);
  DMRG_CHECK_LAUNCH();
  // a basis still far from orthonormal (a direction below the perturbation
  // level, or a non-finite value) is reported instead of being corrected:
  // the caller falls back to the FP64 SVD
  if (!(d < 1e-3)) return DMRG_ERR_NOCONV;
  if (exact) DMRG_TRY(orth_fp64_correct(Z, ld, m, k, A, B, dev, gw, gw_bytes, err, s));
  return DMRG_OK;
}

}  // namespace

// scratch shared by the split-TF32 GEMMs and the digit Gram
size_t gemm_scratch_bytes(int big) {
  const size_t a = tf32x3_gemm_ex_workspace_bytes(big, big, big);
  const size_t b = gram_digits_workspace_bytes(big, big);
  return a > b ? a : b;
}

size_t subspace_workspace_bytes(int m, int n, int k) {
  const size_t big = (size_t)(m > n ? m : n);
  const size_t d = sizeof(double);
  return align_up(256, 1024) + align_up(d * (size_t)m * n, 1024) + 3 * align_up(d * big * k, 1024) +
         2 * align_up(d * (size_t)k * k, 1024) + align_up(d * k, 1024) +
         gemm_scratch_bytes((int)big) + polar_split_bytes((int)big, k) + align_up(64, 1024);
}

// theta (m x n row-major).  absorb 0 keeps an orthonormal LEFT basis; X is
// the tensor on the other side of the bond, kx x n (ld n) with (nominally)
// orthonormal rows.  absorb 1 keeps an orthonormal RIGHT basis; X is the
// left tensor, m x kx (ld kx) with orthonormal columns.  k vectors are kept;
// start vectors beyond kx are random.
// Outputs: left (m x k), right (k x n), *disc = discarded weight fraction.
//
// The start is an orthonormal basis of the OTHER side (the right space for
// a kept left basis) because it is exactly orthonormal in a canonical MPS,
// whereas the centre tensor on the kept side carries the singular values:
// starting from it, its weak directions sit ~s_k^2/s_1^2 below the strong
// ones after the first product and drown in the FP32-level rounding of the
// orthonormalisation.
int subspace_truncate(int m, int n, int k, const double* theta, const double* X, int kx, int absorb, int iters,
                      double* left, double* right, double* disc, void* work, size_t work_bytes, cudaStream_t s) {
  if (k <= 0 || k > m || k > n || kx < 0 || kx > k || iters < 1 || iters > 8) return DMRG_ERR_ARG;
  if (subspace_workspace_bytes(m, n, k) > work_bytes) return DMRG_ERR_WORKSPACE;
  const size_t big = (size_t)(m > n ? m : n);
  const size_t d = sizeof(double);
  char* p = static_cast<char*>(work);
  int* err = reinterpret_cast<int*>(p); p += align_up(256, 1024);
  double* Tt = reinterpret_cast<double*>(p); p += align_up(d * (size_t)m * n, 1024);
  double* S = reinterpret_cast<double*>(p); p += align_up(d * big * k, 1024);
  double* Y = reinterpret_cast<double*>(p); p += align_up(d * big * k, 1024);
  double* C = reinterpret_cast<double*>(p); p += align_up(d * big * k, 1024);
  double* PA = reinterpret_cast<double*>(p); p += align_up(d * (size_t)k * k, 1024);
  double* PB_ = reinterpret_cast<double*>(p); p += align_up(d * (size_t)k * k, 1024);
  double* Pn2 = reinterpret_cast<double*>(p); p += align_up(d * k, 1024);
  void* gw = p;
  const size_t gw_bytes = gemm_scratch_bytes((int)big);
  p += gw_bytes;
  void* splits = p; p += polar_split_bytes((int)big, k);
  double* acc = reinterpret_cast<double*>(p);
  unsigned long long* pdev = reinterpret_cast<unsigned long long*>(acc + 4);
  DMRG_CUDA_TRY(cudaMemsetAsync(err, 0, 256, s));
  DMRG_CUDA_TRY(cudaMemsetAsync(acc, 0, 64, s));
  auto orth = [&](double* Zp, int rows, bool exact) -> int {
    return orth_polar(Zp, k, rows, k, PA, PB_, Pn2, pdev, gw, gw_bytes, splits, err, exact, s);
  };

  // canonical problem: keep the left basis of Th (M x N); W (N x k) is an
  // orthonormal basis of the other side
  const double* Th = theta;
  int M = m, N = n;
  if (absorb == 1) {
    DMRG_TRY(transpose(theta, n, m, n, Tt, m, s));   // Tt = theta^T (n x m)
    Th = Tt; M = n; N = m;
    if (kx > 0) {
      copy2d_kernel<<<egrid((long long)N * kx), 256, 0, s>>>(X, kx, Y, k, N, kx);   // W0 = X (m x kx)
      DMRG_CHECK_LAUNCH();
    }
  } else if (kx > 0) {
    DMRG_TRY(transpose(X, n, kx, n, Y, k, s));       // W0 = X^T (n x kx)
  }
  if (kx < k) {
    random_fill_kernel<<<egrid((long long)N * (k - kx)), 256, 0, s>>>(Y, k, N, kx, k, 0x51ab5eedULL + (unsigned)N);
    DMRG_CHECK_LAUNCH();
  }
  DMRG_TRY(orth(Y, N, false));
  for (int it = 0; it < iters; ++it) {
    // Z = Th W (M x k), Q = orth(Z) (into S)
    DMRG_TRY(tf32x3_gemm_ex(0, 0, M, k, N, 1.f, Th, N, Y, k, 0, S, k, gw, err, s));
    DMRG_TRY(orth(S, M, it == iters - 1));
    if (it + 1 < iters) {
      // W = orth(Th^T Q) (N x k)
      DMRG_TRY(tf32x3_gemm_ex(1, 0, N, k, M, 1.f, Th, N, S, k, 0, Y, k, gw, err, s));
      DMRG_TRY(orth(Y, N, false));
    }
  }
  // C = Q^T Th (k x N)
  DMRG_TRY(tf32x3_gemm_ex(1, 0, k, N, M, 1.f, S, k, Th, N, 0, C, N, gw, err, s));
  sumsq_kernel<<<egrid((long long)k * N), 256, 0, s>>>(C, (long long)k * N, acc);
  DMRG_CHECK_LAUNCH();
  sumsq_kernel<<<egrid((long long)m * n), 256, 0, s>>>(theta, (long long)m * n, acc + 1);
  DMRG_CHECK_LAUNCH();
  if (absorb == 0) {
    copy2d_kernel<<<egrid((long long)m * k), 256, 0, s>>>(S, k, left, k, m, k);
    DMRG_CHECK_LAUNCH();
    copy2d_kernel<<<egrid((long long)k * n), 256, 0, s>>>(C, N, right, n, k, n);
    DMRG_CHECK_LAUNCH();
  } else {
    DMRG_TRY(transpose(S, k, n, k, right, n, s));   // right = Q^T (k x n)
    DMRG_TRY(transpose(C, N, k, m, left, k, s));    // left = C^T (m x k)
  }
  double h[2];
  int e = 0;
  DMRG_CUDA_TRY(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  if (e != 0) return e;
  if (!(h[0] == h[0]) || !(h[1] == h[1])) return DMRG_ERR_NAN;
  if (disc) *disc = h[1] > 0.0 ? fmax(0.0, 1.0 - h[0] / h[1]) : 0.0;
  return DMRG_OK;
}

}  // namespace dmrg

// Truncation of a two-site tensor by warm-started subspace iteration, for
// the split-TF32 sweep at large bond dimension when the kept dimension is
// fixed by maxdim (cutoff <= 0): no eigensolver, only GEMMs on the tensor
// cores plus one small Cholesky per 32-column panel.
//
//   keep the left factor (absorb 0):
//     Y = theta^T X      X: m x k start basis (the current left site tensor)
//     W = orth(Y)        n x k
//     Z = theta W        m x k
//     Q = orth(Z)        left factor  (m x k, orthonormal columns)
//     C = Q^T theta      right factor (k x n)
//   keep the right factor (absorb 1): the same on theta^T, returning
//     left = theta Q (m x k) and right = Q^T (k x n, orthonormal rows).
//
// orth() is block classical Gram-Schmidt run twice (BCGS2): each 32-column
// panel is projected against the finished panels twice (split-TF32 GEMMs)
// and then orthonormalised by two rounds of Cholesky-QR in FP64 inside one
// CTA.  Columns whose remaining norm falls below 1e-13 of the panel are
// zeroed (they carry no weight of theta).  The result is orthonormal to
// FP32-level accuracy, which the variational sweep tolerates; energies are
// refined in FP64 separately.
#include <cmath>
#include <vector>

#include "tf32x3.cuh"

namespace dmrg {

namespace {

constexpr int PB = 32;   // panel width
constexpr int CH = 128;  // rows staged per chunk

constexpr int PT = 256;  // threads of the panel kernel
constexpr int NE = PB * PB / PT;  // Gram entries per thread

// GB300 runs FP64 at 1/64 of the FP32 rate, so the panel arithmetic (Gram
// products, triangular update) is FP32; the 32x32 Cholesky factor and its
// inverse are FP64.  Two Cholesky-QR rounds give FP32-level orthonormality.
__global__ void __launch_bounds__(PT) panel_cholqr2_kernel(double* __restrict__ Z, long long ldz, int m, int c0,
                                                           int b) {
  extern __shared__ double sh[];
  double* G = sh;                                   // PB x (PB+1), FP64
  double* Ri = G + PB * (PB + 1);                   // PB x (PB+1): inverse factor, FP64
  float* Rf = reinterpret_cast<float*>(Ri + PB * (PB + 1));  // same, FP32
  float* tile = Rf + PB * (PB + 1);                 // CH x (PB+1)
  __shared__ int dead[PB];
  const int tid = threadIdx.x;
  const int gj = tid % PB;
  const int gi = tid / PB;  // rows gi, gi + PT/PB, ...
  for (int rep = 0; rep < 2; ++rep) {
    // ---- Gram G = P^T P, two entries per thread (FP32 products, FP64 across chunks)
    double acc[NE];
#pragma unroll
    for (int e = 0; e < NE; ++e) acc[e] = 0.0;
    for (int r0 = 0; r0 < m; r0 += CH) {
      for (int e = tid; e < CH * PB; e += PT) {
        const int rr = e / PB, cc = e % PB;
        const int r = r0 + rr;
        tile[rr * (PB + 1) + cc] = (r < m && cc < b) ? static_cast<float>(Z[(long long)r * ldz + c0 + cc]) : 0.f;
      }
      __syncthreads();
      const int rows = min(CH, m - r0);
      float pp[NE];
#pragma unroll
      for (int e = 0; e < NE; ++e) pp[e] = 0.f;
      for (int rr = 0; rr < rows; ++rr) {
        const float xj = tile[rr * (PB + 1) + gj];
#pragma unroll
        for (int e = 0; e < NE; ++e) pp[e] = fmaf(tile[rr * (PB + 1) + gi + e * (PT / PB)], xj, pp[e]);
      }
#pragma unroll
      for (int e = 0; e < NE; ++e) acc[e] += pp[e];
      __syncthreads();
    }
#pragma unroll
    for (int e = 0; e < NE; ++e) {
      const int r = gi + e * (PT / PB);
      G[r * (PB + 1) + gj] = (r < b && gj < b) ? acc[e] : (r == gj ? 1.0 : 0.0);
    }
    __syncthreads();
    double tr = 0.0;
    for (int i = 0; i < b; ++i) tr = fmax(tr, G[i * (PB + 1) + i]);
    const double floor_ = 1e-12 * tr;   // FP32-level rank threshold
    // ---- Cholesky G = R^T R in place (upper triangle), right-looking, FP64
    for (int k = 0; k < PB; ++k) {
      if (tid == 0) {
        const double p = G[k * (PB + 1) + k];
        dead[k] = (k >= b) || !(p > floor_);
        G[k * (PB + 1) + k] = dead[k] ? 1.0 : sqrt(p);
      }
      __syncthreads();
      const double piv = G[k * (PB + 1) + k];
      const bool dk = dead[k];
      if (tid < PB && tid > k) G[k * (PB + 1) + tid] = dk ? 0.0 : G[k * (PB + 1) + tid] / piv;
      __syncthreads();
      for (int e = tid; e < PB * PB; e += PT) {
        const int i = e / PB, j = e % PB;
        if (i > k && j >= i) G[i * (PB + 1) + j] -= G[k * (PB + 1) + i] * G[k * (PB + 1) + j];
      }
      __syncthreads();
    }
    // ---- inverse of the upper factor, one column per lane of warp 0 (FP64, stored FP32)
    if (tid < PB) {
      const int j = tid;
      for (int i = 0; i < PB; ++i) Ri[i * (PB + 1) + j] = 0.0;
      if (!dead[j]) {
        Ri[j * (PB + 1) + j] = 1.0 / G[j * (PB + 1) + j];
        for (int i = j - 1; i >= 0; --i) {
          double s = 0.0;
          for (int l = i + 1; l <= j; ++l) s += G[i * (PB + 1) + l] * Ri[l * (PB + 1) + j];
          Ri[i * (PB + 1) + j] = dead[i] ? 0.0 : -s / G[i * (PB + 1) + i];
        }
      }
      for (int i = 0; i < PB; ++i) Rf[i * (PB + 1) + j] = static_cast<float>(Ri[i * (PB + 1) + j]);
    }
    __syncthreads();
    // ---- P <- P R^{-1} row by row in FP32 registers
    for (int r = tid; r < m; r += PT) {
      double* zr = Z + (long long)r * ldz + c0;
      float row[PB];
#pragma unroll
      for (int i = 0; i < PB; ++i) row[i] = i < b ? static_cast<float>(zr[i]) : 0.f;
      // column blocks of 8 in descending order: block jb only reads entries
      // i < 8*jb + 8, none of which a later (lower) block has overwritten
#pragma unroll
      for (int jb = PB / 8 - 1; jb >= 0; --jb) {
        float o[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) o[t] = 0.f;
#pragma unroll
        for (int i = 0; i < 8 * jb + 8; ++i) {
          const float ri = row[i];
#pragma unroll
          for (int t = 0; t < 8; ++t)
            if (i <= 8 * jb + t) o[t] = fmaf(ri, Rf[i * (PB + 1) + 8 * jb + t], o[t]);
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) row[8 * jb + t] = o[t];
      }
#pragma unroll
      for (int j = 0; j < PB; ++j)
        if (j < b) zr[j] = static_cast<double>(row[j]);
    }
    __syncthreads();
  }
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

struct OrthWs {
  double* H;   // k x PB projections
  void* gw;    // split-GEMM scratch
  int* err;
};

size_t orth_ws_bytes(int m, int k) {
  return align_up(sizeof(double) * (size_t)k * PB, 1024) + tf32x3_gemm_ex_workspace_bytes(m > k ? m : k, m > k ? m : k, m > k ? m : k) +
         align_up(256, 1024);
}

// Z (m x k, row-major, ld) -> orthonormal columns (zero columns for null directions)
int orth_bcgs2(double* Z, long long ld, int m, int k, const OrthWs& w, cudaStream_t s) {
  static bool attr = false;
  const size_t smem = 2 * sizeof(double) * (size_t)PB * (PB + 1) + sizeof(float) * ((size_t)PB * (PB + 1) + (size_t)CH * (PB + 1));
  if (!attr) {
    DMRG_CUDA_TRY(cudaFuncSetAttribute(panel_cholqr2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  for (int c0 = 0; c0 < k; c0 += PB) {
    const int b = (k - c0) < PB ? (k - c0) : PB;
    if (c0 > 0) {
      for (int pass = 0; pass < 2; ++pass) {
        // H = Q^T Z_j  (c0 x b),  Z_j -= Q H
        DMRG_TRY(tf32x3_gemm_ex(1, 0, c0, b, m, 1.f, Z, ld, Z + c0, ld, 0, w.H, PB, w.gw, w.err, s));
        DMRG_TRY(tf32x3_gemm_ex(0, 0, m, b, c0, -1.f, Z, ld, w.H, PB, 1, Z + c0, ld, w.gw, w.err, s));
      }
    }
    panel_cholqr2_kernel<<<1, PT, smem, s>>>(Z, ld, m, c0, b);
    DMRG_CHECK_LAUNCH();
  }
  return DMRG_OK;
}

// dst (cols x rows, ld = rows) = src^T, src rows x cols with leading dim lds
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

}  // namespace

size_t subspace_workspace_bytes(int m, int n, int k) {
  const size_t big = (size_t)(m > n ? m : n);
  const size_t d = sizeof(double);
  return align_up(256, 1024) + align_up(d * (size_t)m * n, 1024) + 4 * align_up(d * big * k, 1024) +
         orth_ws_bytes((int)big, k) + tf32x3_gemm_ex_workspace_bytes((int)big, (int)big, (int)big) + align_up(64, 1024);
}

// theta (m x n row-major).  absorb 0 keeps an orthonormal LEFT basis; X is
// the start basis m x kx (ld kx).  absorb 1 keeps an orthonormal RIGHT basis;
// X is kx x n (ld n).  k vectors are kept; start columns beyond kx are random.
// Outputs: left (m x k), right (k x n), *disc = discarded weight fraction.
int subspace_truncate(int m, int n, int k, const double* theta, const double* X, int kx, int absorb, double* left,
                      double* right, double* disc, void* work, size_t work_bytes, cudaStream_t s) {
  if (k <= 0 || k > m || k > n || kx < 0 || kx > k) return DMRG_ERR_ARG;
  if (subspace_workspace_bytes(m, n, k) > work_bytes) return DMRG_ERR_WORKSPACE;
  const size_t big = (size_t)(m > n ? m : n);
  const size_t d = sizeof(double);
  char* p = static_cast<char*>(work);
  int* err = reinterpret_cast<int*>(p); p += align_up(256, 1024);
  double* Tt = reinterpret_cast<double*>(p); p += align_up(d * (size_t)m * n, 1024);
  double* S = reinterpret_cast<double*>(p); p += align_up(d * big * k, 1024);
  double* Y = reinterpret_cast<double*>(p); p += align_up(d * big * k, 1024);
  double* C = reinterpret_cast<double*>(p); p += align_up(d * big * k, 1024);
  double* Xs = reinterpret_cast<double*>(p); p += align_up(d * big * k, 1024);
  OrthWs ow;
  ow.H = reinterpret_cast<double*>(p);
  ow.gw = p + align_up(sizeof(double) * (size_t)k * PB, 1024);
  ow.err = err;
  p += orth_ws_bytes((int)big, k);
  void* gw = p; p += tf32x3_gemm_ex_workspace_bytes((int)big, (int)big, (int)big);
  double* acc = reinterpret_cast<double*>(p);
  DMRG_CUDA_TRY(cudaMemsetAsync(err, 0, 256, s));
  DMRG_CUDA_TRY(cudaMemsetAsync(acc, 0, 64, s));

  // canonical problem: keep the left basis of Th (M x N)
  const double* Th = theta;
  int M = m, N = n;
  const double* Xc = X;
  long long ldx = kx;
  if (absorb == 1) {
    DMRG_TRY(transpose(theta, n, m, n, Tt, m, s));   // Tt = theta^T (n x m)
    Th = Tt; M = n; N = m;
    if (kx > 0) DMRG_TRY(transpose(X, n, kx, n, Xs, kx, s));  // Xs = X^T (n x kx)
    Xc = Xs;
  }
  if (kx > 0) {
    copy2d_kernel<<<egrid((long long)M * kx), 256, 0, s>>>(Xc, ldx, S, k, M, kx);
    DMRG_CHECK_LAUNCH();
  }
  if (kx < k) {
    random_fill_kernel<<<egrid((long long)M * (k - kx)), 256, 0, s>>>(S, k, M, kx, k, 0x51ab5eedULL + (unsigned)M);
    DMRG_CHECK_LAUNCH();
  }
  // Y = Th^T S (N x k), W = orth(Y)
  DMRG_TRY(tf32x3_gemm_ex(1, 0, N, k, M, 1.f, Th, N, S, k, 0, Y, k, gw, err, s));
  DMRG_TRY(orth_bcgs2(Y, k, N, k, ow, s));
  // Z = Th W (M x k), Q = orth(Z)  (into S)
  DMRG_TRY(tf32x3_gemm_ex(0, 0, M, k, N, 1.f, Th, N, Y, k, 0, S, k, gw, err, s));
  DMRG_TRY(orth_bcgs2(S, k, M, k, ow, s));
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

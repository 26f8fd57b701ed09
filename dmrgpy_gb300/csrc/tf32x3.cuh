// Split-TF32 (3 products, FP32 accumulation) contraction path on tcgen05.
#pragma once
#include "common.cuh"

namespace dmrg {

// Output description of one split-TF32 GEMM C[M,N] = alpha * sum_k A[M,k] B[N,k]
// (both operands K-major split arrays).  The fields after alpha are optional
// (zero = unused) and need an FP64 output: the stored value is
//   v = alpha*acc + diag*[row == col] (+ C if accumulate),
// written to C when C is non-null and as TF32 hi/lo pairs row-major
// ([row*rld + col]) and/or transposed ([col*tld + row]), which are the
// operand layouts of the next GEMMs of an iteration.
struct GemmOut {
  void* C;
  long long ldm, ldn;   // element strides of C
  int M, N;
  int out_f64;          // 1: store double, 0: store float
  int accumulate;       // 1: C += alpha*result, 0: C = alpha*result
  float alpha;
  double diag;
  // split outputs: TF32 pairs (float) from the tf32 GEMM, FP16 pairs of
  // v * split_scale (__half) from the fp16 GEMM
  void* rhi;
  void* rlo;
  long long rld;
  void* thi;
  void* tlo;
  long long tld;
  double split_scale;
};

// C (M x N) from split operands A (M x Kp) and B (N x Kp), fp32 [rows][Kp]
// arrays holding TF32 hi/lo pairs (Kp a multiple of 32, zero beyond K)
int tf32x3_gemm_split(const float* Ahi, const float* Alo, const float* Bhi, const float* Blo, int M, int N, int Kp,
                      const GemmOut& out, int* err, cudaStream_t s);
// The same product from FP16 operand pairs ([rows][Kp] __half, Kp a
// multiple of 64): two kind::f16 MMAs per K-step of 16 for the price of one
// kind::tf32 step of 8, with the FP32 accumulation kept to 32-wide runs.
// Operands are scaled by powers of two into the FP16 range; alpha carries
// the inverse scales.
int f16x3_gemm_split(const void* Ahi, const void* Alo, const void* Bhi, const void* Blo, int M, int N, int Kp,
                     const GemmOut& out, int* err, cudaStream_t s);
// hi/lo[r][k] = split(in[r*ld + k]) (k < K, zero up to Kp)
int tf32x3_split_rows(const double* in, long long ld, int R, int K, int Kp, float* hi, float* lo, cudaStream_t s);
// hi/lo[c][r] = split(in[r*ld + c]) (r < R, zero up to Rp)
int tf32x3_split_transpose(const double* in, long long ld, int R, int C, int Rp, float* hi, float* lo,
                           cudaStream_t s);

size_t tf32x3_heff_workspace_bytes(const dmrg_heff_t& o);
int tf32x3_heff_apply(const dmrg_heff_t& o, const double* x, double* y, void* work, cudaStream_t s);
// split L/R and the two-site MPO once per operator; then apply per iteration
int tf32x3_heff_prepare(const dmrg_heff_t& o, void* work, cudaStream_t s);
int tf32x3_heff_apply_prepared(const dmrg_heff_t& o, const double* x, double* y, void* work, cudaStream_t s);
// bounded-wait status recorded by the tcgen05 kernels since the last prepare (syncs the stream)
int tf32x3_heff_status(const dmrg_heff_t& o, void* work, cudaStream_t s);
size_t tf32x3_env_workspace_bytes(int chil, int d, int chir, int wl, int wr);
int tf32x3_env(int side, int chil, int d, int chir, int wl, int wr, const double* E, const double* W, const double* A,
               double* Enew, void* work, cudaStream_t s);

size_t tf32x3_gemm_workspace_bytes(int m, int k, int n);
int tf32x3_gemm(int m, int k, int n, const double* A, const double* B, double* C, void* work, cudaStream_t s);

// C (m x n, ldc) (+)= alpha op(A) op(B) on split-TF32 tensor cores (see tf32x3.cu)
size_t tf32x3_gemm_ex_workspace_bytes(int m, int n, int k);
int tf32x3_gemm_ex(int transA, int transB, int m, int n, int k, float alpha, const double* A, long long lda,
                   const double* B, long long ldb, int accumulate, double* C, long long ldc, void* work, int* err,
                   cudaStream_t s);

// G (k x k, ld k) = X^T X for X (m x k, ld) with FP64-level accuracy from
// exact digit products on the tensor cores (gram.cu); m <= 32768
size_t gram_digits_workspace_bytes(int m, int k);
int gram_digits(const double* X, long long ld, int m, int k, double* G, void* work, size_t work_bytes, int* err,
                cudaStream_t s);
int tgemm_gram(const double* X, long long ld, int m, int k, double* G, cudaStream_t stream);

// warm-started subspace-iteration truncation (subspace.cu)
size_t subspace_workspace_bytes(int m, int n, int k);
int subspace_truncate(int m, int n, int k, const double* theta, const double* X, int kx, int absorb, int iters,
                      double* left, double* right, double* disc, void* work, size_t work_bytes, cudaStream_t s);

}  // namespace dmrg

// Internal interface of the H_eff / environment contraction plans.
#pragma once
#include <vector>

#include "common.cuh"

namespace dmrg {

// FP64 / complex FP64 path (strided CUDA-core contractions)
// one strided contraction of a plan (alpha 1, beta 0)
struct GStep {
  TGemm g;
  const void* A;
  const void* B;
  void* C;
};
template <typename T> int heff_fp64_plan(const dmrg_heff_t& o, const T* x, T* y, T* P, T* Q, GStep* steps);
template <typename T>
int env_left_plan(long long cl, long long d, long long cr, long long wl, long long wr, const T* L, const T* W,
                  const T* A, T* Lnew, T* P, GStep* steps);
template <typename T>
int env_right_plan(long long cl, long long d, long long cr, long long wl, long long wr, const T* R, const T* W,
                   const T* B, T* Rnew, T* P, GStep* steps);
template <typename T> size_t heff_fp64_elems(const dmrg_heff_t& o, size_t* p_elems, size_t* q_elems);
template <typename T> int heff_apply_fp64(const dmrg_heff_t& o, const T* x, T* y, T* P, T* Q, cudaStream_t s);
size_t env_fp64_elems(int side, long long cl, long long d, long long cr, long long wl, long long wr);
template <typename T>
int env_left_fp64(long long cl, long long d, long long cr, long long wl, long long wr, const T* L, const T* W,
                  const T* A, T* Lnew, T* P, cudaStream_t s);
template <typename T>
int env_right_fp64(long long cl, long long d, long long cr, long long wl, long long wr, const T* R, const T* W,
                   const T* B, T* Rnew, T* P, cudaStream_t s);

// truncated SVD (one-sided Jacobi)
size_t svd_work_bytes(int dtype, int m, int n);
int svd_orientation_left(int m, int n, int absorb);
int svd_abs_floor(int left, int absorb);
template <typename T>
int hestenes_factor(const T* M, int m, int n, int left, void* work, double* host_s, int* sweeps, int abs_floor,
                    cudaStream_t s);
template <typename T>
int hestenes_output(int m, int n, int left, int keep, int absorb, void* work, T* lo, T* ro, cudaStream_t s);

// batched truncated SVD (one CTA per problem)
size_t svd_batch_work_bytes(int dtype, int nprob, const int* m, const int* n);
template <typename T>
int hestenes_batch_factor(int nprob, const int* m, const int* n, const T* const* M, void* work, double* host_s,
                          int ld_s, int absorb, cudaStream_t s);
template <typename T>
int hestenes_batch_output(int nprob, const int* m, const int* n, const int* keep, int absorb, void* work,
                          T* const* lo, T* const* ro, cudaStream_t s);

// host-side pieces of the Krylov drivers and of the truncation rule
bool tridiag_eig(int n, std::vector<double>& d, std::vector<double> e, std::vector<double>* z);
int lowest_ritz(const std::vector<double>& al, const std::vector<double>& be, double* ev, std::vector<double>* vec);
void keep_rule(const double* s, int n, double cutoff, int maxdim, int mindim, int* keep, double* disc);
void keep_rule_partial(const double* lam, int k, int c, double total, double cutoff, int maxdim, int mindim,
                       double rem, int* keep, double* disc);

// symmetric eigendecomposition by blocked Jacobi (syev.cu): eigenvalues to
// the host (descending), eigenvectors gathered afterwards from the workspace
size_t syev_jacobi_workspace_bytes(int n);
int syev_jacobi(int n, const double* A, long long lda, double* w, int max_sweeps, int* sweeps, void* work,
                size_t work_bytes, cudaStream_t s, int fp32 = 0);
int syev_vectors(int n, int ncols, double* out, long long ldo, int transposed, void* work, cudaStream_t s,
                 int fp32 = 0);

// Gram-matrix truncation (gramtrunc.cu)
constexpr int GRAM_FALLBACK = 100;   // internal: use the exact SVD instead
int sumsq_dev(const double* x, long long n, double* out, cudaStream_t s);
size_t gram_truncate_workspace_bytes(int m, int n, int absorb);
int gram_truncate(int m, int n, const double* M, double cutoff, int maxdim, int mindim, int absorb, double* lo,
                  double* ro, double* svals, int* keep, double* disc, int* sweeps, void* work, size_t work_bytes,
                  cudaStream_t s);
size_t rr_truncate_workspace_bytes(int m, int n, int k);
int rr_truncate(int m, int n, int k, const double* theta, const double* X, int kx, int absorb, int iters,
                double cutoff, int mindim, double* lo, double* ro, double* svals, int* nvals, int* keep, double* disc,
                void* work, size_t work_bytes, cudaStream_t s);
size_t subspace_ritz_workspace_bytes(int m, int n, int k);
int subspace_ritz(int m, int n, int k, int absorb, double* lo, double* ro, double* svals, void* work,
                  size_t work_bytes, cudaStream_t s);

// vector ops
template <typename T> int vaxpy2(T* y, const T* x1, const double* a1, const T* x2, const double* a2, long long n, cudaStream_t s);
template <typename T> int multidot_ws(const T* Q, long long ldq, int k, const T* w, long long n, T* h, double* partial, cudaStream_t s);

}  // namespace dmrg

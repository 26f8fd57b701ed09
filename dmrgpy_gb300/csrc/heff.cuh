// Internal interface of the H_eff / environment contraction plans.
#pragma once
#include "common.cuh"

namespace dmrg {

// FP64 / complex FP64 path (strided CUDA-core contractions)
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
template <typename T> int hestenes_factor(const T* M, int m, int n, void* work, double* host_s, int* sweeps, int abs_floor, cudaStream_t s);
template <typename T> int hestenes_output(int m, int n, int keep, int absorb, void* work, T* lo, T* ro, cudaStream_t s);

// vector ops
template <typename T> int vaxpy2(T* y, const T* x1, const double* a1, const T* x2, const double* a2, long long n, cudaStream_t s);
template <typename T> int multidot_ws(const T* Q, long long ldq, int k, const T* w, long long n, T* h, double* partial, cudaStream_t s);

}  // namespace dmrg

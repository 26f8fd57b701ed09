// Split-TF32 (3 products, FP32 accumulation) contraction path on tcgen05.
#pragma once
#include "common.cuh"

namespace dmrg {

size_t tf32x3_heff_workspace_bytes(const dmrg_heff_t& o);
int tf32x3_heff_apply(const dmrg_heff_t& o, const double* x, double* y, void* work, cudaStream_t s);
size_t tf32x3_env_workspace_bytes(int chil, int d, int chir, int wl, int wr);
int tf32x3_env(int side, int chil, int d, int chir, int wl, int wr, const double* E, const double* W, const double* A,
               double* Enew, void* work, cudaStream_t s);

size_t tf32x3_gemm_workspace_bytes(int m, int k, int n);
int tf32x3_gemm(int m, int k, int n, const double* A, const double* B, double* C, void* work, cudaStream_t s);

}  // namespace dmrg

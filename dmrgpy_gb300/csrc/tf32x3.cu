#include "tf32x3.cuh"

namespace dmrg {

size_t tf32x3_heff_workspace_bytes(const dmrg_heff_t&) { return 0; }
int tf32x3_heff_apply(const dmrg_heff_t&, const double*, double*, void*, cudaStream_t) { return DMRG_ERR_UNSUPPORTED; }
size_t tf32x3_env_workspace_bytes(int, int, int, int, int) { return 0; }
int tf32x3_env(int, int, int, int, int, int, const double*, const double*, const double*, double*, void*, cudaStream_t) {
  return DMRG_ERR_UNSUPPORTED;
}

size_t tf32x3_gemm_workspace_bytes(int, int, int) { return 0; }
int tf32x3_gemm(int, int, int, const double*, const double*, double*, void*, cudaStream_t) { return DMRG_ERR_UNSUPPORTED; }

}  // namespace dmrg

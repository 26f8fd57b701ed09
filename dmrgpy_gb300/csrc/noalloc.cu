// Allocation-free variant of the FP64 H_eff matvec.
//
// dmrg_heff_apply takes its intermediates from a caller workspace.  Some
// callers cannot provide one: a C or Fortran host that links only this
// library has no device allocator of its own, and a host whose device memory
// is fixed when it starts (a long sweep loop that must not stall or fail on
// an allocation half-way through) must not allocate per call.  For them,
// dmrg_heff_apply_noalloc runs the same kernels with their scratch placed in
// one file-scope device array of fixed size, so the call itself allocates
// nothing (no cudaMalloc, no cudaFree, no allocating library routine).
//
// Rules of use:
//   * The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and caches it by
//     device number; make that first call before any stream capture.  The
//     cache assumes the device's primary context (the runtime's) and no
//     cudaDeviceReset between calls, after which the address would be stale.
//   * The array belongs to the library's device image, so every device that
//     loads the library holds its 64 MiB until exit, called or not.
//   * Every call on every stream shares the one array: two calls whose
//     executions overlap (different streams, or host threads without
//     ordering between them) overwrite each other's intermediates and give
//     wrong results.  Callers serialise them, e.g. on one stream.
//   * Nothing in the array has to start at zero: each matvec writes every
//     intermediate element before reading it.
//   * Operators needing more than DMRG_NOALLOC_SCRATCH_BYTES of scratch are
//     rejected with DMRG_ERR_WORKSPACE before anything is launched.
#include <mutex>

#include "common.cuh"

namespace dmrg {
namespace {

static __device__ __align__(256) unsigned char g_heff_scratch[DMRG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// device address of g_heff_scratch on the current device (set up once)
int scratch_address(void** out) {
  int dev = 0;
  DMRG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return DMRG_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    DMRG_CUDA_TRY(cudaGetSymbolAddress(&p, g_heff_scratch));
    if (!p) return DMRG_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return DMRG_OK;
}

}  // namespace
}  // namespace dmrg

extern "C" int dmrg_heff_apply_noalloc(const dmrg_heff_t* op, const void* x, void* y, void* stream) {
  if (!op || !x || !y || x == y) return DMRG_ERR_ARG;
  if (op->precision != DMRG_PREC_FP64) return DMRG_ERR_UNSUPPORTED;
  const size_t need = dmrg_heff_workspace_bytes(op);
  if (need == 0) return DMRG_ERR_ARG;
  if (need > (size_t)DMRG_NOALLOC_SCRATCH_BYTES) return DMRG_ERR_WORKSPACE;
  void* scratch = nullptr;
  DMRG_TRY(dmrg::scratch_address(&scratch));
  return dmrg_heff_apply(op, x, y, scratch, (size_t)DMRG_NOALLOC_SCRATCH_BYTES, stream);
}

// Bounded-wait probe: one thread waits on a freshly initialised mbarrier
// that nothing arrives on, with the same bounded wait as the tcgen05
// kernels (mbar_wait, ~2 s of clock cycles), so the wait runs out, records
// DMRG_ERR_TIMEOUT and the kernel returns; the host reads the status and
// the context stays usable.  No trap, no fault, no unbounded spin.
#include "tcgen05.cuh"

namespace dmrg {
namespace {

__global__ void wait_probe_kernel(int* err, int* outcome) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) outcome[0] = mbar_wait(&bar, 0, err) ? 1 : 2;
}

}  // namespace
}  // namespace dmrg

extern "C" int dmrg_wait_timeout_probe(void* work, size_t work_bytes, void* stream) {
  if (!work || work_bytes < 256) return DMRG_ERR_WORKSPACE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* err = static_cast<int*>(work);
  int* outcome = err + 1;
  DMRG_CUDA_TRY(cudaMemsetAsync(work, 0, 2 * sizeof(int), s));
  dmrg::wait_probe_kernel<<<1, 32, 0, s>>>(err, outcome);
  DMRG_CHECK_LAUNCH();
  int h[2] = {0, 0};
  DMRG_CUDA_TRY(cudaMemcpyAsync(h, work, sizeof(h), cudaMemcpyDeviceToHost, s));
  DMRG_CUDA_TRY(cudaStreamSynchronize(s));
  if (h[1] == 1) return DMRG_OK;     // the barrier completed (cannot happen)
  return h[0] != 0 ? h[0] : DMRG_ERR_CUDA;
}

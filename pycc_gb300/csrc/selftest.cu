// Self-test of the bounded device-side waits, the failure detection of the tensor-core
// kernels: every mbarrier wait of those kernels gives up after the library's wait limit
// (pcg_set_wait_limit_ns), records a status code in a device word the host reads, and lets
// the kernel return, so a stalled pipeline never hangs the GPU.
#include "tc_common.cuh"

namespace pcg {
namespace {

// One warp: thread 0 initialises an mbarrier that expects one arrival and waits on its first
// phase with the kernels' own bounded wait.  No thread arrives, so the wait must expire; the
// kernel then records kStatusTimeoutProbe.  No TMA copy is issued and no TMEM is allocated,
// so nothing is left in flight when it returns.
__global__ void wait_probe_kernel(int* status, unsigned long long limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (!tc::mbar_wait(&bar, 0, limit_ns)) atomicExch(status, kStatusTimeoutProbe);
  }
  __syncwarp();
}

}  // namespace
}  // namespace pcg

// Waits on an mbarrier that nothing completes, bounded by the current wait limit; on expiry
// *status (device int) is set to 4.  Returns after the launch (asynchronous on `stream`).
extern "C" int pcg_wait_probe(int* status, void* stream) {
  if (!status) {
    pcg::set_error("pcg_wait_probe: status is null");
    return -1;
  }
  pcg::wait_probe_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(status, pcg::wait_limit_ns());
  PCG_CHECK_LAUNCH("pcg_wait_probe");
  return 0;
}

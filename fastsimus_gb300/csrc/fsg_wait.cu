// Self-test of the bounded mbarrier wait that every sweep kernel relies on (simus band kernel,
// tensor-core sweep, MLP forward): a wait whose phase never completes must give up, report
// FSG_ETIMEOUT through a status word and leave the context usable.  The kernel waits on a
// barrier that nothing arrives on (or, as the control, on one it arrived on itself).

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fsgb300.h"
#include "fsg_internal.h"
#include "fsg_tc.cuh"

namespace fsg {

__global__ void wait_selftest_kernel(int arrive, uint32_t max_tries, int32_t* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x != 0) return;
  tc::mbar_init(&bar, 1);
  tc::fence_mbar_init();
  if (arrive) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(&bar)) : "memory");
  *status = tc::mbar_wait_bounded(&bar, 0, max_tries) ? FSG_OK : FSG_ETIMEOUT;
}

}  // namespace fsg

extern "C" int32_t fsg_wait_selftest(int32_t arrive, int32_t max_tries, int32_t* status, void* stream) {
  if (!status || max_tries < 1) return fsg::set_error(FSG_EINVAL, "status must be non-NULL and max_tries >= 1");
  fsg::wait_selftest_kernel<<<1, 32, 0, reinterpret_cast<cudaStream_t>(stream)>>>(arrive != 0, (uint32_t)max_tries,
                                                                                 status);
  return fsg::check_cuda(cudaGetLastError(), "wait_selftest_kernel launch");
}

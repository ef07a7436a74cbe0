// simus_stash_kernel instantiations without full-frequency directivity.
#include "fsg_sweep_stash.cuh"

namespace fsg {

cudaError_t launch_simus_stash(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  if (c.kind == 2) return launch_simus_ws_any<false>(U, c, A, s);
  return launch_simus_stash_u<false>(U, c, A, s);
}

}  // namespace fsg

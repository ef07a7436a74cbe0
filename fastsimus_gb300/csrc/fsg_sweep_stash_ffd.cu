// simus_stash_kernel instantiations with full-frequency directivity.
#include "fsg_sweep_stash.cuh"

namespace fsg {

cudaError_t launch_simus_stash_ffd(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  if (c.kind == 2) return launch_simus_ws_any<true>(U, c, A, s);
  return launch_simus_stash_u<true>(U, c, A, s);
}

}  // namespace fsg

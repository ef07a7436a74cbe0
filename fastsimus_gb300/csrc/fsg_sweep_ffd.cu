// Instantiations of the plain sweep kernels with full-frequency directivity
// (full_frequency_directivity=True): each Green's term is weighted by sinc(k_f seg/2 sin(theta))
// at every frequency, as in the step bodies _simus_strategies.py:59-62 and
// _pfield_strategies.py:44-45 (driven from :77-81).  Kept in a translation unit of their own so that they compile
// in parallel with the default kernels of fsg_sweep.cu.

#include "fsg_sweep_kernels.cuh"

namespace fsg {

cudaError_t launch_simus_band_ffd(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  return launch_simus_band_u<true>(U, c, A, s);
}

cudaError_t launch_pfield_band_ffd(const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  return launch_pfield_band_gn<true>(c, A, s);
}

}  // namespace fsg

// fsg_simus_noalloc: the plain simus sweep for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a plugin inside a host application
// that owns all device memory and hands the plugin only its input and output buffers (a
// scanner's real-time processing chain, an inference-server backend with a fixed memory
// budget), or code that must not synchronise the device mid-stream, which cudaMalloc/cudaFree
// may do.  This entry point takes the same inputs and outputs as fsg_simus but no workspace:
// its scratch (the per-frequency tables and the partial spectra) lives in the
// file-scope device array below.
//
// Limits and behaviour:
//   - The scratch is kNoAllocScratchBytes (16 MiB).  fsg_simus cuts the scatterers into chunks
//     whose geometry cache fits the workspace it is given, so the scratch bounds only the fixed
//     part of a request: the per-frequency tables, the partial spectra (a few slots of
//     n_freq x n_elements complex64) and the geometry block of one tile.  That is about 12 MiB
//     for the 128-element, 1,142-frequency probe of the 200,000-scatterer frame, whatever the
//     scatterer count; a larger scatterer count only means more, smaller chunks.  Requests whose
//     fixed part does not fit (plans with many thousands of frequencies) are rejected with
//     FSG_EINVAL and a message; nothing is launched.
//   - The array is part of this library's device image, so every GPU that loads the library
//     holds the 16 MiB until the process exits.
//   - Host code cannot use the array's name as a device address.  The first call on each
//     device, with that device current, asks the runtime for the address
//     (cudaGetSymbolAddress) and caches it for the life of the process; make that first call
//     before any stream capture.  The cache assumes the device's primary context (the one the
//     CUDA runtime uses): after cudaDeviceReset, or with another driver-API context current on
//     the device, the cached address is not valid.
//   - All calls share the array and it keeps the last call's contents.  Every byte the sweep
//     reads is written earlier in the same call (tables by the set-up kernel; the partial
//     spectra are zeroed by the call, then accumulated by the band kernels; each tile's
//     geometry block is written before it is read), so nothing has to start at zero.
//   - Calls whose work overlaps on the GPU (different streams, or different host threads on
//     one device) race on the shared scratch and corrupt each other's results; serialise them.
//   - The call allocates nothing: no cudaMalloc, no cudaFree, no allocating library routine.

#include <cuda_runtime.h>

#include <mutex>

#include "../../include/fsgb300.h"
#include "fsg_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

int scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fsg::check_cuda(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fsg::set_error(FSG_EINVAL, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fsg::check_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return FSG_OK;
}

}  // namespace

extern "C" size_t fsg_simus_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int32_t fsg_simus_noalloc(const FsgProbe* probe, const FsgMedium* medium, const FsgFreqPlan* plan,
                                     const double* scat_xz, const double* rc, int64_t n_scat, const double* delays,
                                     const double* apod, int32_t full_frequency_directivity, int32_t out_layout,
                                     void* out, void* stream) {
  if (!probe || !plan) return fsg::set_error(FSG_EINVAL, "probe and plan must be non-NULL");
  if (probe->n_elements < 1 || probe->n_sub < 1 || plan->n_freq < 1 || n_scat < 0)
    return fsg::set_error(FSG_EINVAL, "fsg_simus_noalloc: cannot size the scratch for this request");
  int sms = 0;
  int st = fsg::device_sm_count(&sms);
  if (st != FSG_OK) return st;
  const size_t need = fsg::simus_min_workspace(probe, plan, n_scat, full_frequency_directivity ? 1 : 0, sms);
  if (need > kNoAllocScratchBytes)
    return fsg::set_error(FSG_EINVAL,
                          "fsg_simus_noalloc: this request needs at least %zu bytes of scratch but the static scratch "
                          "holds %zu bytes; use fsg_simus with a caller-provided workspace",
                          need, kNoAllocScratchBytes);
  void* scratch = nullptr;
  st = scratch_address(&scratch);
  if (st != FSG_OK) return st;
  return fsg_simus(probe, medium, plan, scat_xz, rc, n_scat, delays, apod, full_frequency_directivity, out_layout,
                   out, scratch, kNoAllocScratchBytes, stream);
}

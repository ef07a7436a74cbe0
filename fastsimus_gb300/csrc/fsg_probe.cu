// Measurement utility: an FP32 FMA throughput probe used to state the FP32 roofline of the
// plain sweep kernels (the machine's measured-peaks file covers HBM bandwidth and bf16 tensor
// rate only).  Each thread runs 8 independent FMA chains; flops = 2 * 8 * iters * threads.

#include <cuda_runtime.h>

#include "../../include/fsgb300.h"
#include "fsg_internal.h"

namespace fsg {

__global__ void __launch_bounds__(256) fp32_fma_probe_kernel(float* out, int iters, float seed) {
  float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float b = 0.999999f, c = 1e-7f;
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
    a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
    a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
  }
  float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains live; never true in practice
}

}  // namespace fsg

extern "C" int32_t fsg_fp32_fma_probe(float* out, int32_t blocks, int32_t iters, double* flops, void* stream) {
  if (!out || blocks < 1 || iters < 1 || !flops) return fsg::set_error(FSG_EINVAL, "bad probe arguments");
  fsg::fp32_fma_probe_kernel<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(out, iters, 0.5f);
  *flops = 2.0 * 8.0 * (double)iters * 256.0 * (double)blocks;
  return fsg::check_cuda(cudaGetLastError(), "fp32_fma_probe launch");
}

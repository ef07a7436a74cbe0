// Spectrum -> RF epilogue: irfft of the conjugated spectrum over its nonzero band, plus the
// smooth -100 dB gate (simus.py:336-367), in two kernels.
//
// rf[n][e] = (1/N) sum_k w_k Re(conj(S[k][e]) exp(i 2 pi k n / N)),  n < (N + 1) / 2,
// w_k = 1 for k = 0 and k = N/2, 2 otherwise, k <= N/2 (the Hermitian half that a C2R
// transform reads; the imaginary parts of the DC and Nyquist bins drop out because
// sin(0) = sin(pi n) = 0).  Only the selected band [k_first, k_first + k_count) of the
// simus spectrum is nonzero, so the sum runs over it alone.  The transform is a real GEMM
// [cos | sin](n, k) x [Re S ; Im S](k, e) with the twiddles looked up by the exact integer
// index (k n) mod N in a table of N entries, FP32 accumulation.
//
// The gate multiplies by 0.5 (1 + tanh((|rf| / max|rf| - 1e-5) / 1e-6)) with each frame's own
// peak; the first kernel folds its output tile's peak into a per-frame word with an integer
// atomicMax on the float bits (|rf| >= 0, so the order of the bits is the order of the
// values and the result does not depend on the order of the atomics).

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/fsgb300.h"
#include "fsg_internal.h"

namespace fsg {

constexpr int kRfTN = 32;  // samples per CTA tile
constexpr int kRfTE = 64;  // elements per CTA tile
constexpr int kRfK = 32;   // frequencies per shared-memory chunk

__global__ void twiddle_kernel(float2* tw, int N) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  double s, c;
  sincospi(2.0 * (double)j / (double)N, &s, &c);
  tw[j] = make_float2((float)c, (float)s);
}

__global__ void __launch_bounds__(256) irfft_kernel(const float2* __restrict__ S, int64_t bstride, int E, int N,
                                                    int k0, int kc, const float2* __restrict__ tw, int n_samples,
                                                    float* __restrict__ rf, unsigned int* __restrict__ peak) {
  __shared__ __align__(16) float2 Ssh[kRfK][kRfTE];
  __shared__ __align__(16) float2 Tsh[kRfK][kRfTN];
  __shared__ unsigned int s_peak;
  const int b = blockIdx.z;
  const int n0 = blockIdx.x * kRfTN, e0 = blockIdx.y * kRfTE;
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;  // samples n0 + 2 ty + i, elements e0 + 4 tx + j
  const float2* Sb = S + (size_t)b * bstride;
  const float inv_n = 1.0f / (float)N;
  float acc[2][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  if (tid == 0) s_peak = 0u;
  for (int c0 = 0; c0 < kc; c0 += kRfK) {
    __syncthreads();
    for (int i = tid; i < kRfK * kRfTE; i += blockDim.x) {
      const int kk = i / kRfTE, ee = i % kRfTE, k = k0 + c0 + kk, e = e0 + ee;
      float2 v = make_float2(0.f, 0.f);
      if (c0 + kk < kc && e < E) {
        v = Sb[(size_t)k * E + e];
        const float w = (k == 0 || 2 * k == N) ? inv_n : 2.0f * inv_n;
        v.x *= w;
        v.y *= w;
      }
      Ssh[kk][ee] = v;
    }
    for (int i = tid; i < kRfK * kRfTN; i += blockDim.x) {
      const int kk = i / kRfTN, nn = i % kRfTN;
      const long long k = k0 + c0 + kk, n = n0 + nn;
      Tsh[kk][nn] = tw[(int)((k * n) % N)];
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < kRfK; ++kk) {
      const float4 t = *reinterpret_cast<const float4*>(&Tsh[kk][2 * ty]);
      const float4 sa = *reinterpret_cast<const float4*>(&Ssh[kk][4 * tx]);
      const float4 sb = *reinterpret_cast<const float4*>(&Ssh[kk][4 * tx + 2]);
      const float2 tv[2] = {make_float2(t.x, t.y), make_float2(t.z, t.w)};
      const float2 sv[4] = {make_float2(sa.x, sa.y), make_float2(sa.z, sa.w), make_float2(sb.x, sb.y),
                            make_float2(sb.z, sb.w)};
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(sv[j].x, tv[i].x, fmaf(sv[j].y, tv[i].y, acc[i][j]));
    }
  }
  float m = 0.f;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int n = n0 + 2 * ty + i;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int e = e0 + 4 * tx + j;
      if (n < n_samples && e < E) {
        rf[((size_t)b * n_samples + n) * E + e] = acc[i][j];
        m = fmaxf(m, fabsf(acc[i][j]));
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
  __syncthreads();
  if ((tid & 31) == 0) atomicMax(&s_peak, __float_as_uint(m));
  __syncthreads();
  if (tid == 0 && peak) atomicMax(&peak[b], s_peak);
}

__global__ void gate_kernel(float* __restrict__ rf, int64_t per_frame, int n_batch, const unsigned int* __restrict__ peak) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per_frame * n_batch) return;
  const float m = __uint_as_float(peak[i / per_frame]);
  const float v = rf[i];
  const float rel = fabsf(v) / (m + 1e-30f);
  rf[i] = v * (0.5f * (1.0f + tanhf((rel - 1e-5f) / 1e-6f)));
}

static size_t rf_a256(size_t v) { return (v + 255) & ~size_t(255); }

}  // namespace fsg

using namespace fsg;

extern "C" size_t fsg_rf_workspace_size(int32_t n_fft, int32_t n_batch) {
  if (n_fft < 1 || n_batch < 1) return 0;
  return rf_a256((size_t)n_fft * 8) + rf_a256((size_t)n_batch * 4);
}

extern "C" int32_t fsg_irfft_gate(const void* spectrum, int32_t n_batch, int64_t batch_stride, int32_t n_freq_full,
                                  int32_t n_elements, int32_t n_fft, int32_t k_first, int32_t k_count, int32_t gate,
                                  float* rf_out, void* workspace, size_t workspace_bytes, void* stream_ptr) {
  if (!spectrum || !rf_out) return set_error(FSG_EINVAL, "spectrum and rf_out must be non-NULL");
  if (n_batch < 1 || n_elements < 1 || n_fft < 1 || n_freq_full < 1)
    return set_error(FSG_EINVAL, "n_batch, n_elements, n_fft and n_freq_full must be >= 1");
  if (k_first < 0 || k_count < 0 || k_first + k_count > n_freq_full)
    return set_error(FSG_EINVAL, "band [%d, %d) does not fit in n_freq_full = %d", k_first, k_first + k_count,
                     n_freq_full);
  if (batch_stride < (int64_t)n_freq_full * n_elements)
    return set_error(FSG_EINVAL, "batch_stride %lld is smaller than one spectrum", (long long)batch_stride);
  const size_t need = fsg_rf_workspace_size(n_fft, n_batch);
  if (!workspace || workspace_bytes < need)
    return set_error(FSG_EWORKSPACE, "workspace of %zu bytes is smaller than the %zu bytes required", workspace_bytes,
                     need);
  // a C2R transform of length N reads bins 0 .. N/2 only
  int kc = k_count;
  if (k_first > n_fft / 2) kc = 0;
  else if (k_first + kc > n_fft / 2 + 1) kc = n_fft / 2 + 1 - k_first;
  const int n_samples = (n_fft + 1) / 2;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream_ptr);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  float2* tw = reinterpret_cast<float2*>(ws);
  unsigned int* peak = reinterpret_cast<unsigned int*>(ws + rf_a256((size_t)n_fft * 8));
  int st;
  if ((st = check_cuda(cudaMemsetAsync(peak, 0, (size_t)n_batch * 4, s), "peak reset")) != FSG_OK) return st;
  twiddle_kernel<<<(n_fft + 255) / 256, 256, 0, s>>>(tw, n_fft);
  if ((st = check_cuda(cudaGetLastError(), "twiddle_kernel launch")) != FSG_OK) return st;
  dim3 grid((n_samples + kRfTN - 1) / kRfTN, (n_elements + kRfTE - 1) / kRfTE, n_batch);
  irfft_kernel<<<grid, 256, 0, s>>>(static_cast<const float2*>(spectrum), batch_stride, n_elements, n_fft, k_first, kc,
                                    tw, n_samples, rf_out, peak);
  if ((st = check_cuda(cudaGetLastError(), "irfft_kernel launch")) != FSG_OK) return st;
  if (gate) {
    const int64_t per = (int64_t)n_samples * n_elements;
    gate_kernel<<<(unsigned)((per * n_batch + 255) / 256), 256, 0, s>>>(rf_out, per, n_batch, peak);
    if ((st = check_cuda(cudaGetLastError(), "gate_kernel launch")) != FSG_OK) return st;
  }
  return FSG_OK;
}

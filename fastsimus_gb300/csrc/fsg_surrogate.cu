// Transmit-field surrogate support: the exact transmit field at arbitrary (x, z, f, theta)
// samples, and the hand-written kernels that train and evaluate a Fourier-feature MLP
// (BF16 weights, FP32 accumulation).
//
// Exact field (the training target and the judge of the network's error).  For a plane wave
// of steering angle theta on a linear array, delays tau_e = x_e sin(theta) / c - min_e(...)
// (tx_delay.py:116-189); the complex transmit pressure at (x, z) and frequency f is
//     p = pulse(f) probe(f) sum_{e,u} apod_e exp(i 2 pi f tau_e) G(x, z, e, u, f)
// with G as in _init_exponentials (_pfield_math.py:202-247) and the 1/n_sub of pfield.py:159-170
// -- the quantity inside _pfield_strategies.py:48 before |.|^2, evaluated in closed form (no
// recurrence: every sample has its own f and theta).
//
// MLP: features gamma(v) = [sin(2 pi B v), cos(2 pi B v)] of the normalised inputs (64 random
// frequencies, B fixed), 4 hidden layers of width 256 with SiLU, a linear (Re, Im) head.
// One tiled GEMM kernel with fused epilogues (bias + SiLU, SiLU derivative) serves the
// forward pass, both backward GEMMs and inference; weights are read as BF16 and every product
// accumulates in FP32.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/fsgb300.h"
#include "fsg_common.cuh"
#include "fsg_internal.h"

namespace fsg {

struct TxFieldArgs {
  const double* samples;  // [n][4]: x, z, f (Hz), theta (rad)
  int64_t n;
  float2* out;            // [n] complex transmit pressure
  const float4* src_pos;  // [E*U]
  const float2* rot_e;    // [E]
  float pitch;            // element x = (e - (E-1)/2) * pitch in float32 (utils/geometry.py:33-37)
  int E, U;
  double c, att, fc, bandwidth, n_wavelengths;
  SweepConst C;           // geometry constants (dk/dalpha unused)
};

__device__ double sinc_pi(double x) {  // numpy.sinc: sin(pi x) / (pi x)
  if (x == 0.0) return 1.0;
  const double px = kPi * x;
  return sin(px) / px;
}

__global__ void txfield_kernel(const TxFieldArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double x = a.samples[4 * i], z = a.samples[4 * i + 1], f = a.samples[4 * i + 2], th = a.samples[4 * i + 3];
  // pulse * probe at f (spectrum.py:24-107)
  const double w = 2.0 * kPi * f, wc = 2.0 * kPi * a.fc;
  const double dur = a.n_wavelengths / a.fc;
  const double pulse_im = sinc_pi(dur * (w - wc) / 2.0 / kPi) - sinc_pi(dur * (w + wc) / 2.0 / kPi);  // times i
  const double wb = a.bandwidth * wc;
  const double shape = log(126.0) / log(2.0 * wc / wb);
  const double sigma = wb / 2.0 / pow(log(2.0), 1.0 / shape);
  const double probe = sqrt(exp(-pow(fabs(w - wc) / sigma, shape)));
  // plane-wave delays: tau_e = x_e sin(theta)/c - min_e
  const double st = sin(th);
  double xmin = 1e300;
  for (int e = 0; e < a.E; ++e)
    xmin = fmin(xmin, (double)__fmul_rn(__fsub_rn((float)e, (float)((a.E - 1) * 0.5)), a.pitch) * st);
  const dfl xs = split_double(x), zs = split_double(z);
  const dfl kf = split_double(2.0 * kPi * f / a.c);
  const float alpha = (float)(a.att / 8.685889638065035 * f / 1e6 * 1e2);
  float2 acc = make_float2(0.f, 0.f);
  for (int e = 0; e < a.E; ++e) {
    // delay phase 2 pi f tau in cycles, reduced in double (one per element and sample)
    const double xe = (double)__fmul_rn(__fsub_rn((float)e, (float)((a.E - 1) * 0.5)), a.pitch);
    const double cyc = f * ((xe * st - xmin) / a.c);
    const double fr = cyc - rint(cyc);
    float sd, cd;
    sincospif((float)(2.0 * fr), &sd, &cd);
    float2 es = make_float2(0.f, 0.f);
    for (int u = 0; u < a.U; ++u) {
      const SrcGeo geo = source_geometry(xs, zs, a.src_pos[e * a.U + u], a.rot_e[e], a.C);
      const float2 g = anchor_value(geo.r_hi, geo.r_lo, geo.amp, make_float2(kf.hi, kf.lo), alpha);
      es = cadd(es, g);
    }
    acc = cfma(es, make_float2(cd, sd), acc);
  }
  // times pulse (= i * pulse_im) * probe
  const float s = (float)(pulse_im * probe);
  const bool out_field = z < 0.0;
  a.out[i] = out_field ? make_float2(0.f, 0.f) : make_float2(-acc.y * s, acc.x * s);
}

// ------------------------------------------------------------------------------------------
// Tiled GEMM with fused epilogues: C[m][n] = sum_k A(m, k) * B(k, n)
//   A(m, k) = A[m * a_sm + k * a_sk] (FP32),  B(k, n) = B[k * b_sk + n * b_sn] (FP32 or BF16)
// epilogue 0: C = acc (+ bias[n])
// epilogue 1: Z = acc + bias[n]; C = Z; C2 = silu(Z)        (forward hidden layer)
// epilogue 2: C = acc * silu'(Zs[m][n])                       (backward through SiLU)
// 64 x 64 output tile per CTA, 256 threads, 4 x 4 outputs per thread, K staged 16 at a time.
// ------------------------------------------------------------------------------------------
struct GemmArgs {
  const float* A;
  int64_t a_sm, a_sk;
  const void* B;
  int64_t b_sk, b_sn;
  int b_bf16;
  const float* bias;
  const float* Zs;  // for epilogue 2, leading dim ldc
  float* C;
  float* C2;
  int64_t ldc;
  int M, N, K, epi, accumulate;
};

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

__global__ void __launch_bounds__(256) gemm_kernel(const GemmArgs g) {
  __shared__ float As[16][65];
  __shared__ float Bs[16][65];
  const int tid = threadIdx.x;
  const int tm = tid / 16, tn = tid % 16;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < g.K; k0 += 16) {
    for (int i = tid; i < 16 * 64; i += 256) {
      // consecutive threads walk the unit-stride dimension of each operand (coalesced loads)
      int kk, mm;
      if (g.a_sk == 1) { mm = i / 16; kk = i % 16; } else { kk = i / 64; mm = i % 64; }
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < g.M && k < g.K) ? g.A[m * g.a_sm + k * g.a_sk] : 0.f;
      int kb, nn;
      if (g.b_sn == 1) { kb = i / 64; nn = i % 64; } else { nn = i / 16; kb = i % 16; }
      const int n = n0 + nn, kq = k0 + kb;
      float b = 0.f;
      if (n < g.N && kq < g.K) {
        const int64_t o = kq * g.b_sk + n * g.b_sn;
        b = g.b_bf16 ? __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(g.B)[o])
                     : reinterpret_cast<const float*>(g.B)[o];
      }
      Bs[kb][nn] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tm + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tn + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + tm + 16 * i, n = n0 + tn + 16 * j;
      if (m >= g.M || n >= g.N) continue;
      float v = acc[i][j];
      const int64_t o = m * g.ldc + n;
      if (g.epi == 0) {
        if (g.bias) v += g.bias[n];
        g.C[o] = g.accumulate ? g.C[o] + v : v;
      } else if (g.epi == 1) {
        v += g.bias[n];
        g.C[o] = v;
        g.C2[o] = silu(v);
      } else {
        g.C[o] = v * silu_grad(g.Zs[o]);
      }
    }
}

// Fourier features of normalised inputs u (n x 4): feat[n][j] = sin(2 pi B_j . u), feat[n][64 + j] = cos(...)
__global__ void fourier_features_kernel(const float* u, const float* Bmat, float* feat, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * 64) return;
  const int64_t r = i / 64;
  const int j = (int)(i % 64);
  const float t = Bmat[4 * j] * u[4 * r] + Bmat[4 * j + 1] * u[4 * r + 1] + Bmat[4 * j + 2] * u[4 * r + 2] +
                  Bmat[4 * j + 3] * u[4 * r + 3];
  float s, c;
  sincospif(2.0f * t, &s, &c);
  feat[r * 128 + j] = s;
  feat[r * 128 + 64 + j] = c;
}

// column sums: out[n] (+)= sum_m X[m][n]
__global__ void colsum_kernel(const float* X, int64_t M, int N, float* out, int accumulate) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int64_t m = 0; m < M; ++m) s += X[m * N + n];
  out[n] = accumulate ? out[n] + s : s;
}

// Adam on FP32 master weights, BF16 copy for the GEMMs.
__global__ void adam_kernel(float* w, __nv_bfloat16* w_bf16, const float* grad, float* m1, float* m2, int64_t n,
                            float lr, float b1, float b2, float eps, float bc1, float bc2, float grad_scale) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = grad[i] * grad_scale;
  const float a = b1 * m1[i] + (1.f - b1) * g;
  const float b = b2 * m2[i] + (1.f - b2) * g * g;
  m1[i] = a;
  m2[i] = b;
  const float v = w[i] - lr * (a / bc1) / (sqrtf(b / bc2) + eps);
  w[i] = v;
  if (w_bf16) w_bf16[i] = __float2bfloat16_rn(v);
}

}  // namespace fsg

using namespace fsg;

extern "C" int32_t fsg_txfield(const FsgProbe* probe, const FsgMedium* medium, double tx_n_wavelengths,
                               double bandwidth, const double* samples, int64_t n, void* out, void* workspace,
                               size_t workspace_bytes, void* stream_ptr) {
  if (!probe || !medium || !samples || !out) return set_error(FSG_EINVAL, "NULL argument");
  if (!isinf(probe->radius)) return set_error(FSG_EUNSUPPORTED, "transmit-field samples need a linear array");
  if (probe->n_elements < 1 || probe->n_sub < 1) return set_error(FSG_EINVAL, "bad probe");
  const int E = probe->n_elements, U = probe->n_sub;
  const size_t need = (size_t)E * U * 16 + (size_t)E * 8 + 1024;
  if (!workspace || workspace_bytes < need) return set_error(FSG_EWORKSPACE, "workspace too small (%zu < %zu)",
                                                             workspace_bytes, need);
  if (n <= 0) return FSG_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream_ptr);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  SetupArgs sa;
  memset(&sa, 0, sizeof(sa));
  sa.E = E;
  sa.U = U;
  sa.pitch = probe->pitch;
  sa.width = probe->element_width;
  sa.radius = probe->radius;
  sa.c = medium->speed_of_sound;
  sa.seg = probe->element_width / U;
  sa.t.src_pos = reinterpret_cast<float4*>(ws);
  sa.t.rot_e = reinterpret_cast<float2*>(ws + (size_t)E * U * 16);
  setup_tables<<<(E * U + 127) / 128, 128, 0, s>>>(sa);
  int st = check_cuda(cudaGetLastError(), "setup_tables launch");
  if (st != FSG_OK) return st;
  TxFieldArgs a;
  a.samples = samples;
  a.n = n;
  a.out = static_cast<float2*>(out);
  a.src_pos = sa.t.src_pos;
  a.rot_e = sa.t.rot_e;
  a.pitch = (float)probe->pitch;
  a.E = E;
  a.U = U;
  a.c = medium->speed_of_sound;
  a.att = medium->attenuation;
  a.fc = probe->freq_center;
  a.bandwidth = bandwidth;
  a.n_wavelengths = tx_n_wavelengths;
  FsgFreqPlan dummy;
  memset(&dummy, 0, sizeof(dummy));
  dummy.seg_length = probe->element_width / U;
  a.C = make_sweep_const(probe, medium, &dummy, 0);
  txfield_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
  return check_cuda(cudaGetLastError(), "txfield_kernel launch");
}

extern "C" int32_t fsg_mlp_gemm(const float* A, int64_t a_sm, int64_t a_sk, const void* B, int64_t b_sk, int64_t b_sn,
                                int32_t b_bf16, const float* bias, const float* Zs, float* C, float* C2, int64_t ldc,
                                int32_t M, int32_t N, int32_t K, int32_t epilogue, int32_t accumulate, void* stream) {
  if (!A || !B || !C || M < 0 || N < 0 || K < 0) return set_error(FSG_EINVAL, "bad gemm arguments");
  if (epilogue == 1 && (!bias || !C2)) return set_error(FSG_EINVAL, "epilogue 1 needs bias and C2");
  if (epilogue == 2 && !Zs) return set_error(FSG_EINVAL, "epilogue 2 needs Zs");
  if (M == 0 || N == 0) return FSG_OK;
  GemmArgs g{A, a_sm, a_sk, B, b_sk, b_sn, b_bf16, bias, Zs, C, C2, ldc, M, N, K, epilogue, accumulate};
  if ((M + 63) / 64 > 65535) return set_error(FSG_EINVAL, "M too large for one launch");
  gemm_kernel<<<dim3((N + 63) / 64, (M + 63) / 64), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(g);
  return check_cuda(cudaGetLastError(), "gemm_kernel launch");
}

extern "C" int32_t fsg_mlp_features(const float* u, const float* bmat, float* feat, int64_t n, void* stream) {
  if (!u || !bmat || !feat || n < 0) return set_error(FSG_EINVAL, "bad feature arguments");
  if (n == 0) return FSG_OK;
  fourier_features_kernel<<<(unsigned)((n * 64 + 255) / 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      u, bmat, feat, n);
  return check_cuda(cudaGetLastError(), "fourier_features launch");
}

extern "C" int32_t fsg_mlp_colsum(const float* X, int64_t M, int32_t N, float* out, int32_t accumulate, void* stream) {
  if (!X || !out) return set_error(FSG_EINVAL, "bad colsum arguments");
  colsum_kernel<<<(N + 127) / 128, 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(X, M, N, out, accumulate);
  return check_cuda(cudaGetLastError(), "colsum launch");
}

extern "C" int32_t fsg_mlp_adam(float* w, void* w_bf16, const float* grad, float* m1, float* m2, int64_t n, float lr,
                                float b1, float b2, float eps, int32_t step, float grad_scale, void* stream) {
  if (!w || !grad || !m1 || !m2 || n < 0 || step < 1) return set_error(FSG_EINVAL, "bad adam arguments");
  if (n == 0) return FSG_OK;
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      w, static_cast<__nv_bfloat16*>(w_bf16), grad, m1, m2, n, lr, b1, b2, eps, bc1, bc2, grad_scale);
  return check_cuda(cudaGetLastError(), "adam launch");
}

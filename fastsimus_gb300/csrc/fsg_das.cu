// Downstream beamforming of simulated RF: I/Q demodulation (fsg_rf2iq) and delay-and-sum
// (fsg_das matrix-free with compounding, fsg_dasmtx as a CSR matrix).  They restate MUST's
// rf2iq / dasmtx algorithms, which the reference's validation tests call through PyMUST
// (tests/_picmus_phantom_shared.py:407-460).
//
// rf2iq_kernel: one thread per (frame, channel) column.  The IIR recurrence is sequential in
// time, so a column is one thread's loop: forward over the odd-extended down-mixed signal
// (outputs of the record written to the channel-major IQ array, those of the right extension
// kept in a local array), then backward over them in place.  The filter runs as cascaded
// second-order sections in FP32 (a single high-order recursion loses ~1e-3 in FP32 at narrow
// cut-offs; the cascade stays at ~1e-6).  The down-mixing phasors depend on the sample only:
// each CTA tabulates them in shared memory (phase n fc / fs + fc tau reduced to [0, 1) cycles
// in FP64, then sincospif), so a column's step is a load, a multiply and the biquads.
//
// das_kernel: one thread per pixel, looping over groups of firings and, per element, over the
// group's firings.  The transmit delays (times c) and the element frames sit in shared memory;
// the I/Q samples are read channel-major, so the threads of a warp (consecutive pixels down an
// image column) read nearby samples of the same element.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/fsgb300.h"
#include "fsg_internal.h"

namespace fsg {

constexpr int kDasThreads = 256;      // dasmtx_kernel
constexpr int kDasImgThreads = 128;   // das_kernel: small CTAs spread the pixels evenly over the SMs
constexpr int kDasMaxE = 256;
constexpr int kDasFrameGroup = 32;  // firings whose transmit distances a thread holds at a time

struct Rf2IqArgs {
  const float* rf;   // [n_frames][n_samples][n_ch]
  float2* iq;        // [n_frames][n_ch][n_samples]
  int n_frames, n_samples, n_ch, n_sec, pad;
  double cyc_per_sample;  // fc / fs
  double cyc0;            // fc tau
  float sos[FSG_RF2IQ_MAX_SECTIONS][5];  // b0, b1, b2, a1, a2
  float zi[FSG_RF2IQ_MAX_SECTIONS][2];   // steady state for a unit input
};

constexpr int kIqChunk = 16;     // samples loaded ahead of the recurrence (memory-level parallelism)
constexpr int kIqTable = 2048;   // down-mixing phasors shared by a CTA's columns, per pass
constexpr int kIqThreads = 64;

// Down-mixing phasor of sample n: exp(-2 pi i (n fc / fs + fc tau)), the phase reduced to
// cycles in FP64.
__device__ __forceinline__ float2 phasor(const Rf2IqArgs& A, int n) {
  const double cyc = fma((double)n, A.cyc_per_sample, A.cyc0);
  const float frac = (float)(cyc - floor(cyc));
  float s, c;
  sincospif(2.0f * frac, &s, &c);
  return make_float2(c, -s);
}

__device__ __forceinline__ float2 downmix(const Rf2IqArgs& A, const float* col, int n) {
  const float v = col[(size_t)n * A.n_ch];
  const float2 e = phasor(A, n);
  return make_float2(v * e.x, v * e.y);
}

// One sample through the cascade of transposed direct-form-II biquads (real coefficients).
template <int NS>
__device__ __forceinline__ float2 iir_step(const Rf2IqArgs& A, float2 (*z)[2], float2 x) {
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const float* q = A.sos[s];
    const float2 y = make_float2(fmaf(q[0], x.x, z[s][0].x), fmaf(q[0], x.y, z[s][0].y));
    z[s][0] = make_float2(fmaf(q[1], x.x, fmaf(-q[3], y.x, z[s][1].x)), fmaf(q[1], x.y, fmaf(-q[3], y.y, z[s][1].y)));
    z[s][1] = make_float2(fmaf(q[2], x.x, -q[4] * y.x), fmaf(q[2], x.y, -q[4] * y.y));
    x = y;
  }
  return x;
}

template <int NS>
__device__ __forceinline__ void iir_init(const Rf2IqArgs& A, float2 (*z)[2], float2 x0) {
#pragma unroll
  for (int s = 0; s < NS; ++s)
#pragma unroll
    for (int k = 0; k < 2; ++k) z[s][k] = make_float2(A.zi[s][k] * x0.x, A.zi[s][k] * x0.y);
}

template <int NS>
__global__ void __launch_bounds__(kIqThreads) rf2iq_kernel(const __grid_constant__ Rf2IqArgs A) {
  __shared__ float2 ph[kIqTable];  // phasors of the samples n0 .. n0 + kIqTable - 1
  const int64_t colid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = colid < (int64_t)A.n_frames * A.n_ch;
  const int64_t cid = active ? colid : 0;
  const int fr = (int)(cid / A.n_ch), ch = (int)(cid % A.n_ch);
  const float* __restrict__ col = A.rf + (size_t)fr * A.n_samples * A.n_ch + ch;
  float2* __restrict__ y = A.iq + (size_t)cid * A.n_samples;
  const int N = A.n_samples, P = A.pad;
  float2 z[NS][2];
  float2 right[FSG_RF2IQ_MAX_PAD];
  float2 x0 = make_float2(0.f, 0.f), xn = x0;
  // forward pass over [2 x0 - x[P..1], x[0..N-1], 2 x[N-1] - x[N-2..N-1-P]]
  if (active) {
    x0 = downmix(A, col, 0);
    xn = downmix(A, col, N - 1);
    const float2 xp = downmix(A, col, P);
    iir_init<NS>(A, z, P > 0 ? make_float2(2.f * x0.x - xp.x, 2.f * x0.y - xp.y) : x0);
    for (int k = 0; k < P; ++k) {
      const float2 v = downmix(A, col, P - k);
      iir_step<NS>(A, z, make_float2(2.f * x0.x - v.x, 2.f * x0.y - v.y));
    }
  }
  // the record: the phasors are the same for every column, so the CTA tabulates them; the
  // recurrence is sequential, the loads are not, so each chunk's samples are requested first
  for (int n0 = 0; n0 < N; n0 += kIqTable) {
    __syncthreads();
    for (int j = threadIdx.x; j < kIqTable && n0 + j < N; j += blockDim.x) ph[j] = phasor(A, n0 + j);
    __syncthreads();
    if (!active) continue;
    const int n_end = min(N, n0 + kIqTable);
    for (int m0 = n0; m0 < n_end; m0 += kIqChunk) {
      float v[kIqChunk];
#pragma unroll
      for (int j = 0; j < kIqChunk; ++j) v[j] = m0 + j < n_end ? col[(size_t)(m0 + j) * A.n_ch] : 0.f;
#pragma unroll
      for (int j = 0; j < kIqChunk; ++j)
        if (m0 + j < n_end) {
          const float2 e = ph[m0 + j - n0];
          y[m0 + j] = iir_step<NS>(A, z, make_float2(v[j] * e.x, v[j] * e.y));
        }
    }
  }
  if (!active) return;
  for (int k = 0; k < P; ++k) {
    const float2 v = downmix(A, col, N - 2 - k);
    right[k] = iir_step<NS>(A, z, make_float2(2.f * xn.x - v.x, 2.f * xn.y - v.y));
  }
  // backward pass, started from the last forward output
  iir_init<NS>(A, z, P > 0 ? right[P - 1] : y[N - 1]);
  for (int k = P - 1; k >= 0; --k) iir_step<NS>(A, z, right[k]);
  for (int n1 = N - 1; n1 >= 0; n1 -= kIqChunk) {
    float2 w[kIqChunk];
#pragma unroll
    for (int j = 0; j < kIqChunk; ++j) w[j] = n1 - j >= 0 ? y[n1 - j] : make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < kIqChunk; ++j)
      if (n1 - j >= 0) {
        const float2 o = iir_step<NS>(A, z, w[j]);
        y[n1 - j] = make_float2(2.f * o.x, 2.f * o.y);
      }
  }
}

struct DasArgs {
  const float2* iq;    // [n_frames][E][n_s]
  const double* txd;   // [n_frames][E]
  const double* pix;   // [n_pix][2]
  float2* out;         // image [n_pix] or CSR values
  int* crow;           // dasmtx only
  int* col;
  int64_t n_pix;
  int n_frames, n_s, E, method, iq_rot;
  double pitch, radius;
  float c, inv_c, fs, two_fc, t0;
  float aperture;      // 1 / (2 f-number), or < 0 for every element
};

// Element centre and frame (sin, cos of its angle): linear arrays along x, convex arrays on
// the arc of the given radius with the apex at z = 0.
__device__ void das_element(const DasArgs& A, int e, float* x, float* z, float* sn, float* cs) {
  if (isinf(A.radius)) {
    *x = (float)(((double)e - 0.5 * (A.E - 1)) * A.pitch);
    *z = 0.f;
    *sn = 0.f;
    *cs = 1.f;
    return;
  }
  const double half = asin(A.pitch / 2.0 / A.radius);
  const double chord = 2.0 * A.radius * sin(half * (A.E - 1));
  const double apex = sqrt(A.radius * A.radius - (chord / 2.0) * (chord / 2.0));
  const double t0 = atan2(-chord / 2.0, apex), t1 = atan2(chord / 2.0, apex);
  const double te = (A.E > 1) ? ((e == A.E - 1) ? t1 : t0 + e * ((t1 - t0) / (A.E - 1))) : t0;
  *x = (float)(A.radius * sin(te));
  *z = (float)(A.radius * cos(te) - apex);
  *sn = (float)sin(te);
  *cs = (float)cos(te);
}

struct DasShared {
  float ex[kDasMaxE], ez[kDasMaxE], es[kDasMaxE], ec[kDasMaxE], ctx[kDasMaxE];
};

__device__ __forceinline__ void das_load_elements(const DasArgs& A, DasShared& S) {
  for (int e = threadIdx.x; e < A.E; e += blockDim.x) das_element(A, e, &S.ex[e], &S.ez[e], &S.es[e], &S.ec[e]);
}

__device__ __forceinline__ void das_load_delays(const DasArgs& A, DasShared& S, int f) {
  for (int e = threadIdx.x; e < A.E; e += blockDim.x) {
    const double v = A.txd[(size_t)f * A.E + e];
    S.ctx[e] = isnan(v) ? INFINITY : (float)(A.c * v);
  }
}

// Transmit distance of pixel (px, pz): the earliest arrival over the firing elements.
__device__ __forceinline__ float das_dtx(const DasArgs& A, const DasShared& S, float px, float pz) {
  float d = INFINITY;
  for (int e = 0; e < A.E; ++e) {
    const float dx = px - S.ex[e], dz = pz - S.ez[e];
    d = fminf(d, S.ctx[e] + sqrtf(fmaf(dx, dx, dz * dz)));
  }
  return d;
}

// Delay, fractional sample and I/Q rotation of element e for pixel (px, pz); false outside
// the receive aperture.
__device__ __forceinline__ bool das_tap(const DasArgs& A, const DasShared& S, int e, float px, float pz, float dtx,
                                        float* s, float2* rot) {
  const float dx = px - S.ex[e], dz = pz - S.ez[e];
  if (A.aperture >= 0.f) {
    const float ax = fmaf(dx, S.es[e], dz * S.ec[e]);
    const float lat = fmaf(dx, S.ec[e], -dz * S.es[e]);
    if (!(ax > 0.f) || fabsf(lat) > ax * A.aperture) return false;
  }
  const float t = (dtx + sqrtf(fmaf(dx, dx, dz * dz))) * A.inv_c;
  *s = (t - A.t0) * A.fs;
  if (A.iq_rot) {
    float sn, cs;
    sincospif(A.two_fc * t, &sn, &cs);
    *rot = make_float2(cs, sn);
  } else {
    *rot = make_float2(1.f, 0.f);
  }
  return true;
}

// Matrix-free compounded delay-and-sum.  The I/Q rotation exp(2 pi i fc (d_tx + d_rx) / c)
// factors into a transmit part per (pixel, firing) and a receive part per (pixel, element), so
// a thread first computes, for a group of firings, the transmit distance and rotation (kept in
// registers / local memory), then per element the receive distance, aperture test and rotation
// once, and per firing only the sample gather, the interpolation and one complex multiply-add.
// The group's transmit delays (times c) sit in dynamic shared memory, [firing][element].
__global__ void __launch_bounds__(kDasImgThreads, 4) das_kernel(const __grid_constant__ DasArgs A, int group) {
  __shared__ DasShared S;
  extern __shared__ float ctx_g[];  // [group][E]
  das_load_elements(A, S);
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < A.n_pix;
  const float px = valid ? (float)A.pix[2 * p] : 0.f, pz = valid ? (float)A.pix[2 * p + 1] : 0.f;
  const float k_cyc = 0.5f * A.two_fc * A.inv_c;  // cycles per metre of path, fc / c
  float dtx[kDasFrameGroup];
  float2 rtx[kDasFrameGroup];
  float2 acc = make_float2(0.f, 0.f);
  for (int g0 = 0; g0 < A.n_frames; g0 += group) {
    const int ng = min(group, A.n_frames - g0);
    __syncthreads();
    for (int i = threadIdx.x; i < ng * A.E; i += blockDim.x) {
      const double v = A.txd[(size_t)g0 * A.E + i];
      ctx_g[i] = isnan(v) ? INFINITY : (float)(A.c * v);
    }
    __syncthreads();
    if (!valid) continue;
    for (int j = 0; j < ng; ++j) {
      const float* cj = ctx_g + j * A.E;
      float d = INFINITY;
      for (int e = 0; e < A.E; ++e) {
        const float dx = px - S.ex[e], dz = pz - S.ez[e];
        d = fminf(d, cj[e] + sqrtf(fmaf(dx, dx, dz * dz)));
      }
      dtx[j] = d;
      float sn = 0.f, cs = 1.f;
      if (A.iq_rot && d < INFINITY) sincospif(2.f * k_cyc * d, &sn, &cs);
      rtx[j] = make_float2(cs, sn);
    }
    for (int e = 0; e < A.E; ++e) {
      const float dx = px - S.ex[e], dz = pz - S.ez[e];
      if (A.aperture >= 0.f) {
        const float ax = fmaf(dx, S.es[e], dz * S.ec[e]);
        const float lat = fmaf(dx, S.ec[e], -dz * S.es[e]);
        if (!(ax > 0.f) || fabsf(lat) > ax * A.aperture) continue;
      }
      const float dr = sqrtf(fmaf(dx, dx, dz * dz));
      float2 ae = make_float2(0.f, 0.f);
      const float2* ce = A.iq + ((size_t)g0 * A.E + e) * A.n_s;
      const size_t fstride = (size_t)A.E * A.n_s;
      const float last = (float)(A.n_s - 1);
      // branch-free taps (a tap outside the record reads sample 0 with weight 0), unrolled so
      // that the gathers of several firings are in flight together
      if (A.method == FSG_DAS_LINEAR) {
#pragma unroll 4
        for (int j = 0; j < ng; ++j) {
          const float s = ((dtx[j] + dr) * A.inv_c - A.t0) * A.fs;
          const float fi = floorf(s);
          const bool ok = fi >= 0.f && fi + 1.f <= last;
          const int i0 = ok ? (int)fi : 0;
          const float w = s - fi;
          const float2* cj = ce + j * fstride;
          const float2 a = cj[i0], b = cj[i0 + 1];
          const float2 v = ok ? make_float2(fmaf(w, b.x - a.x, a.x), fmaf(w, b.y - a.y, a.y)) : make_float2(0.f, 0.f);
          ae.x = fmaf(v.x, rtx[j].x, fmaf(-v.y, rtx[j].y, ae.x));
          ae.y = fmaf(v.x, rtx[j].y, fmaf(v.y, rtx[j].x, ae.y));
        }
      } else {
#pragma unroll 4
        for (int j = 0; j < ng; ++j) {
          const float s = ((dtx[j] + dr) * A.inv_c - A.t0) * A.fs;
          const float fi = floorf(s + 0.5f);
          const bool ok = fi >= 0.f && fi <= last;
          const float2 c = ce[j * fstride + (ok ? (int)fi : 0)];
          const float2 v = ok ? c : make_float2(0.f, 0.f);
          ae.x = fmaf(v.x, rtx[j].x, fmaf(-v.y, rtx[j].y, ae.x));
          ae.y = fmaf(v.x, rtx[j].y, fmaf(v.y, rtx[j].x, ae.y));
        }
      }
      float sn = 0.f, cs = 1.f;
      if (A.iq_rot) sincospif(2.f * k_cyc * dr, &sn, &cs);
      acc.x = fmaf(ae.x, cs, fmaf(-ae.y, sn, acc.x));
      acc.y = fmaf(ae.x, sn, fmaf(ae.y, cs, acc.y));
    }
  }
  if (valid) A.out[p] = acc;
}

__global__ void __launch_bounds__(kDasThreads) dasmtx_kernel(const __grid_constant__ DasArgs A) {
  __shared__ DasShared S;
  das_load_elements(A, S);
  das_load_delays(A, S, 0);
  __syncthreads();
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= A.n_pix) return;
  const int per = A.method == FSG_DAS_LINEAR ? 2 * A.E : A.E;
  A.crow[p] = (int)(p * per);
  if (p == A.n_pix - 1) A.crow[A.n_pix] = (int)(A.n_pix * per);
  const float px = (float)A.pix[2 * p], pz = (float)A.pix[2 * p + 1];
  const float dtx = das_dtx(A, S, px, pz);
  int* cl = A.col + p * per;
  float2* vl = A.out + p * per;
  for (int e = 0; e < A.E; ++e) {
    float s = 0.f;
    float2 rot = make_float2(0.f, 0.f);
    const bool on = dtx < INFINITY && das_tap(A, S, e, px, pz, dtx, &s, &rot);
    const int base = e * A.n_s;
    if (A.method == FSG_DAS_LINEAR) {
      const float fi = floorf(s);
      const bool in = on && fi >= 0.f && fi + 1.f <= (float)(A.n_s - 1);
      const int i0 = in ? (int)fi : 0;
      const float w = in ? s - fi : 0.f;
      const float g0 = in ? 1.f - w : 0.f;
      cl[2 * e] = base + i0;
      cl[2 * e + 1] = base + i0 + 1;
      vl[2 * e] = make_float2(g0 * rot.x, g0 * rot.y);
      vl[2 * e + 1] = make_float2(w * rot.x, w * rot.y);
    } else {
      const float fi = floorf(s + 0.5f);
      const bool in = on && fi >= 0.f && fi <= (float)(A.n_s - 1);
      cl[e] = base + (in ? (int)fi : 0);
      vl[e] = in ? rot : make_float2(0.f, 0.f);
    }
  }
}

}  // namespace fsg

using namespace fsg;

extern "C" int32_t fsg_rf2iq(const float* rf, int32_t n_frames, int32_t n_samples, int32_t n_channels, double fs,
                             double fc, double tau, int32_t n_sections, const double* sos, const double* zi,
                             int32_t pad, void* iq_out, void* stream) {
  if (!rf || !iq_out || !sos || !zi) return set_error(FSG_EINVAL, "rf, iq_out, sos and zi must be non-NULL");
  if (n_frames < 1 || n_channels < 1 || n_samples < 1)
    return set_error(FSG_EINVAL, "n_frames, n_samples and n_channels must be >= 1");
  if (n_sections < 1 || n_sections > FSG_RF2IQ_MAX_SECTIONS)
    return set_error(FSG_EUNSUPPORTED, "%d filter sections outside [1, %d]", n_sections, FSG_RF2IQ_MAX_SECTIONS);
  if (pad < 0 || pad > FSG_RF2IQ_MAX_PAD || pad >= n_samples)
    return set_error(FSG_EINVAL, "pad %d must be in [0, min(%d, n_samples - 1)]", pad, FSG_RF2IQ_MAX_PAD);
  if (!(fs > 0) || !(fc >= 0)) return set_error(FSG_EINVAL, "fs must be > 0 and fc >= 0");
  Rf2IqArgs A;
  A.rf = rf;
  A.iq = static_cast<float2*>(iq_out);
  A.n_frames = n_frames;
  A.n_samples = n_samples;
  A.n_ch = n_channels;
  A.n_sec = n_sections;
  A.pad = pad;
  A.cyc_per_sample = fc / fs;
  A.cyc0 = fc * tau;
  for (int sct = 0; sct < FSG_RF2IQ_MAX_SECTIONS; ++sct) {
    const bool on = sct < n_sections;
    if (on && sos[6 * sct + 3] != 1.0) return set_error(FSG_EINVAL, "section %d: a0 must be 1", sct);
    const int take[5] = {0, 1, 2, 4, 5};
    for (int k = 0; k < 5; ++k) A.sos[sct][k] = on ? (float)sos[6 * sct + take[k]] : 0.f;
    for (int k = 0; k < 2; ++k) A.zi[sct][k] = on ? (float)zi[2 * sct + k] : 0.f;
  }
  const int64_t cols = (int64_t)n_frames * n_channels;
  const unsigned grid = (unsigned)((cols + kIqThreads - 1) / kIqThreads);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  switch (n_sections) {
    case 1: rf2iq_kernel<1><<<grid, kIqThreads, 0, s>>>(A); break;
    case 2: rf2iq_kernel<2><<<grid, kIqThreads, 0, s>>>(A); break;
    case 3: rf2iq_kernel<3><<<grid, kIqThreads, 0, s>>>(A); break;
    default: rf2iq_kernel<4><<<grid, kIqThreads, 0, s>>>(A); break;
  }
  return check_cuda(cudaGetLastError(), "rf2iq_kernel launch");
}

static int das_args(const FsgProbe* probe, const FsgDasParams* p, int n_frames, int n_samples, const double* txd,
                    const double* pixels, int64_t n_pixels, DasArgs* A) {
  if (!probe || !p || !txd || (n_pixels > 0 && !pixels))
    return set_error(FSG_EINVAL, "probe, params, tx_delays and pixels must be non-NULL");
  if (probe->n_elements < 1 || probe->n_elements > kDasMaxE)
    return set_error(FSG_EUNSUPPORTED, "n_elements %d outside [1, %d]", probe->n_elements, kDasMaxE);
  if (!(probe->pitch > 0) || !(probe->radius > 0)) return set_error(FSG_EINVAL, "pitch and radius must be > 0");
  if (n_frames < 1 || n_samples < 2 || n_pixels < 0)
    return set_error(FSG_EINVAL, "n_frames >= 1, n_samples >= 2 and n_pixels >= 0 are required");
  if (!(p->speed_of_sound > 0) || !(p->fs > 0)) return set_error(FSG_EINVAL, "speed_of_sound and fs must be > 0");
  if (p->method != FSG_DAS_LINEAR && p->method != FSG_DAS_NEAREST)
    return set_error(FSG_EINVAL, "unknown interpolation method %d", p->method);
  A->txd = txd;
  A->pix = pixels;
  A->n_pix = n_pixels;
  A->n_frames = n_frames;
  A->n_s = n_samples;
  A->E = probe->n_elements;
  A->method = p->method;
  A->iq_rot = p->iq != 0;
  A->pitch = probe->pitch;
  A->radius = probe->radius;
  A->c = (float)p->speed_of_sound;
  A->inv_c = (float)(1.0 / p->speed_of_sound);
  A->fs = (float)p->fs;
  A->two_fc = (float)(2.0 * p->fc);
  A->t0 = (float)p->t0;
  A->aperture = p->fnumber > 0 ? (float)(0.5 / p->fnumber) : -1.f;
  A->crow = nullptr;
  A->col = nullptr;
  return FSG_OK;
}

extern "C" int32_t fsg_das(const FsgProbe* probe, const FsgDasParams* params, const void* iq, int32_t n_frames,
                           int32_t n_samples, const double* tx_delays, const double* pixels, int64_t n_pixels,
                           void* image_out, void* stream) {
  if (!iq || !image_out) return set_error(FSG_EINVAL, "iq and image_out must be non-NULL");
  DasArgs A;
  int st = das_args(probe, params, n_frames, n_samples, tx_delays, pixels, n_pixels, &A);
  if (st != FSG_OK) return st;
  if (n_pixels == 0) return FSG_OK;
  A.iq = static_cast<const float2*>(iq);
  A.out = static_cast<float2*>(image_out);
  const int group = n_frames < kDasFrameGroup ? n_frames : kDasFrameGroup;
  das_kernel<<<(unsigned)((n_pixels + kDasImgThreads - 1) / kDasImgThreads), kDasImgThreads,
               (size_t)group * A.E * sizeof(float), reinterpret_cast<cudaStream_t>(stream)>>>(A, group);
  return check_cuda(cudaGetLastError(), "das_kernel launch");
}

extern "C" int32_t fsg_dasmtx_nnz_per_row(int32_t method, int32_t n_elements) {
  return method == FSG_DAS_NEAREST ? n_elements : 2 * n_elements;
}

extern "C" int32_t fsg_dasmtx(const FsgProbe* probe, const FsgDasParams* params, int32_t n_samples,
                              const double* tx_delays, const double* pixels, int64_t n_pixels, int32_t* crow,
                              int32_t* col, void* val, void* stream) {
  if (!crow || !col || !val) return set_error(FSG_EINVAL, "crow, col and val must be non-NULL");
  DasArgs A;
  int st = das_args(probe, params, 1, n_samples, tx_delays, pixels, n_pixels, &A);
  if (st != FSG_OK) return st;
  const int64_t per = fsg_dasmtx_nnz_per_row(params->method, probe->n_elements);
  if (n_pixels * per > INT32_MAX || (int64_t)n_samples * probe->n_elements > INT32_MAX)
    return set_error(FSG_EUNSUPPORTED, "matrix of %lld non-zeros exceeds 32-bit CSR indices", (long long)(n_pixels * per));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (n_pixels == 0) return check_cuda(cudaMemsetAsync(crow, 0, sizeof(int32_t), s), "crow reset");
  A.iq = nullptr;
  A.out = static_cast<float2*>(val);
  A.crow = crow;
  A.col = col;
  dasmtx_kernel<<<(unsigned)((n_pixels + kDasThreads - 1) / kDasThreads), kDasThreads, 0, s>>>(A);
  return check_cuda(cudaGetLastError(), "dasmtx_kernel launch");
}

// Plain fused FP32 simus and pfield sweeps for GB300 (sm_103a).
//
// Work decomposition (one CTA = 256 threads):
//   blockIdx.x -> a frequency band of `fb` consecutive selected frequencies
//   blockIdx.y -> a slice of scatterers (simus) or grid points (pfield)
// A CTA walks its slice in tiles of `st` scatterers.  For each tile:
//   1. geometry: each thread computes the double-float distance, amplitude and recurrence
//      step of kSrcPerThread (scatterer, source) pairs and parks them in shared memory;
//   2. TX: the same thread advances its 16 transmit-weighted Green's terms through the band
//      (re-anchored every kAnchor steps), sums them, and the `gn` threads that share a
//      scatterer finish the sum over all E*U sources with warp shuffles.  The product
//      rc * pulse * probe * P is the scattered field W[f][s] (simus) or |.|^2 is
//      accumulated per point (pfield);
//   3. RX (simus): thread (element e, run of kAnchor frequencies) re-generates the receive
//      Green's terms of every scatterer of the tile from the parked geometry and accumulates
//      Y[e][f] += W[f][s] * mean_u G(s, e, u, f) in registers.
// Neither the scatterer x element Green's tile nor W ever leaves the SM; the only global
// output is one (F x E) partial spectrum per slice, summed in a fixed order by fsg_reduce.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "fsg_common.cuh"
#include "fsg_internal.h"

namespace fsg {

constexpr double kNeperToDb = 8.685889638065035;  // 20 / ln(10)

// Element / sub-element positions (utils/geometry.py:18-88, _pfield_math.py:40-67),
// per-frequency wavenumber / attenuation / spectra, per-anchor delay-apodization factors.
__global__ void setup_tables(SetupArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n_src = a.E * a.U;
  const bool linear = isinf(a.radius);
  if (i < n_src) {
    const int e = i / a.U, u = i % a.U;
    double xe, ze, te;
    if (linear) {
      // float32 arithmetic, as NumPy 2 evaluates arange(float32) - (N-1)/2 times pitch
      float idx = __fsub_rn((float)e, (float)((a.E - 1) * 0.5));
      xe = (double)__fmul_rn(idx, (float)a.pitch);
      ze = 0.0;
      te = 0.0;
    } else {
      double half = asin(a.pitch / 2.0 / a.radius);
      double total = half * (a.E - 1);
      double chord = 2.0 * a.radius * sin(total);
      double apex = sqrt(a.radius * a.radius - (chord / 2.0) * (chord / 2.0));
      double t0 = atan2(-chord / 2.0, apex), t1 = atan2(chord / 2.0, apex);
      te = (a.E > 1) ? ((e == a.E - 1) ? t1 : t0 + e * ((t1 - t0) / (a.E - 1))) : t0;
      xe = a.radius * sin(te);
      ze = a.radius * cos(te) - apex;
    }
    double off = -a.width / 2.0 + a.seg / 2.0 + u * a.seg;
    double sx = xe + off * cos(te);
    double sz = ze + off * sin(-te);
    dfl hx = split_double(sx), hz = split_double(sz);
    a.t.src_pos[i] = make_float4(hx.hi, hx.lo, hz.hi, hz.lo);
    if (u == 0) a.t.rot_e[e] = make_float2((float)cos(te), (float)sin(te));
  }
  if (i < a.F) {
    double f = a.f0 + i * a.df;
    dfl k = split_double(2.0 * kPi * f / a.c);
    a.t.kf[i] = make_float2(k.hi, k.lo);
    a.t.af[i] = (float)(a.att / kNeperToDb * f / 1e6 * 1e2);
    double pr = a.probe[i];
    a.t.pp[i] = make_float2((float)(a.pulse[2 * i] * pr), (float)(a.pulse[2 * i + 1] * pr));
    a.t.probe[i] = (float)pr;
  }
  if (i < a.n_anchor * a.E) {
    const int m = i / a.E, e = i % a.E;
    double tau = a.delays[e];
    double w = a.apod ? a.apod[e] : 1.0;
    if (isnan(tau)) { tau = 0.0; w = 0.0; }
    double f = a.f0 + (double)m * kAnchor * a.df;
    double s, c;
    sincos(2.0 * kPi * f * tau, &s, &c);
    a.t.da[i] = make_float2((float)(w * c), (float)(w * s));
    if (m == 0) {
      sincos(2.0 * kPi * a.df * tau, &s, &c);
      a.t.dstep[e] = make_float2((float)c, (float)s);
    }
  }
}

__device__ __forceinline__ dfl load_coord(const double* p) {
  return split_double(*p);
}

// Loads the band's per-frequency tables into shared memory.
__device__ __forceinline__ void load_band_tables(const BandArgs& A, const SmemLayout& L, unsigned char* sm, int f_b0) {
  float2* pp = reinterpret_cast<float2*>(sm + L.off_pp);
  float2* ka = reinterpret_cast<float2*>(sm + L.off_ka);
  float* aa = reinterpret_cast<float*>(sm + L.off_aa);
  float2* da = reinterpret_cast<float2*>(sm + L.off_da);
  const int na = A.fb / kAnchor;
  for (int i = threadIdx.x; i < A.fb; i += blockDim.x) {
    int f = f_b0 + i;
    pp[i] = (f < A.F) ? A.t.pp[f] : make_float2(0.f, 0.f);
  }
  for (int m = threadIdx.x; m < na; m += blockDim.x) {
    int f = min(f_b0 + m * kAnchor, A.F - 1);
    ka[m] = A.t.kf[f];
    aa[m] = A.t.af[f];
  }
  for (int i = threadIdx.x; i < na * A.E; i += blockDim.x) {
    int m = i / A.E, e = i % A.E;
    int ga = min(f_b0 / kAnchor + m, A.n_anchor - 1);
    da[i] = A.t.da[ga * A.E + e];
  }
}

// Geometry + TX over one band for one tile.  Each thread owns point `sl` of the tile and
// sources [g*16, g*16+16).  `sink(f_local, psum)` is called by the thread with g == 0 once
// per frequency with the full source sum.
template <class Sink>
__device__ __forceinline__ void tx_tile(const BandArgs& A, const SmemLayout& L, unsigned char* sm, int64_t p_idx,
                                        int sl, int g, Sink& sink) {
  float* b_rhi = reinterpret_cast<float*>(sm + L.off_rhi);
  float* b_rlo = reinterpret_cast<float*>(sm + L.off_rlo);
  float* b_amp = reinterpret_cast<float*>(sm + L.off_amp);
  float2* b_st = reinterpret_cast<float2*>(sm + L.off_step);
  const float2* ka = reinterpret_cast<const float2*>(sm + L.off_ka);
  const float* aa = reinterpret_cast<const float*>(sm + L.off_aa);
  const float2* da = reinterpret_cast<const float2*>(sm + L.off_da);

  // 1. geometry of my sources, parked in shared memory (rolled loop: one copy of the code)
  {
    const dfl xs = load_coord(A.pts + 2 * p_idx);
    const dfl zs = load_coord(A.pts + 2 * p_idx + 1);
#pragma unroll 1
    for (int i = 0; i < kSrcPerThread; ++i) {
      const int src = g * kSrcPerThread + i;
      if (src < A.n_src) {
        const int e = src / A.U, u = src - e * A.U;
        const int idx = (u * A.E + e) * L.pitch + sl;
        const SrcGeo geo = source_geometry(xs, zs, A.t.src_pos[src], A.t.rot_e[e], A.C);
        b_rhi[idx] = geo.r_hi;
        b_rlo[idx] = geo.r_lo;
        b_amp[idx] = geo.amp;
        b_st[idx] = geo.step;
      }
    }
  }
  // 2. transmit sweep: exact anchor every kTxAnchor steps, FP32 recurrence in between
  float2 G[kSrcPerThread];
  float2 S[kSrcPerThread];
  const int n_tx_anchor = (A.fb + kTxAnchor - 1) / kTxAnchor;
  for (int m = 0; m < n_tx_anchor; ++m) {
    const int am = m * (kTxAnchor / kAnchor);  // index into the band's kAnchor-spaced tables
#pragma unroll
    for (int i = 0; i < kSrcPerThread; ++i) {
      const int src = g * kSrcPerThread + i;
      G[i] = make_float2(0.f, 0.f);
      if (m == 0) S[i] = make_float2(0.f, 0.f);
      if (src < A.n_src) {
        const int e = src / A.U, u = src - e * A.U;
        const int idx = (u * A.E + e) * L.pitch + sl;
        G[i] = cmul(anchor_value(b_rhi[idx], b_rlo[idx], b_amp[idx], ka[am], aa[am]), da[am * A.E + e]);
        if (m == 0) S[i] = cmul(b_st[idx], A.t.dstep[e]);
      }
    }
    const int n_steps = min(kTxAnchor, A.fb - m * kTxAnchor);
#pragma unroll 2
    for (int j = 0; j < n_steps; ++j) {
      float2 ps = G[0];
      G[0] = cmul(G[0], S[0]);
#pragma unroll
      for (int i = 1; i < kSrcPerThread; ++i) {
        ps = cadd(ps, G[i]);
        G[i] = cmul(G[i], S[i]);
      }
      for (int off = 1; off < A.gn; off <<= 1) {
        ps.x += __shfl_xor_sync(0xffffffffu, ps.x, off);
        ps.y += __shfl_xor_sync(0xffffffffu, ps.y, off);
      }
      if (g == 0) sink(m * kTxAnchor + j, ps);
    }
  }
}

struct SimusSink {
  float2* W;        // [fb][st]
  const float2* pp; // [fb]
  float w;          // rc (0 when out of field or padding)
  int sl, st;
  __device__ __forceinline__ void operator()(int fl, float2 ps) {
    float2 v = cmul(pp[fl], ps);
    W[fl * st + sl] = make_float2(w * v.x, w * v.y);
  }
};

template <int U>
__global__ void __launch_bounds__(kThreads, 1) simus_band_kernel(const BandArgs A) {
  extern __shared__ __align__(16) unsigned char sm[];
  const SmemLayout L = smem_layout(A.gn, A.st, A.fb, A.E, true);
  const int tid = threadIdx.x;
  const int f_b0 = blockIdx.x * A.fb;
  const int64_t s_begin = (int64_t)blockIdx.y * A.per_slice;
  const int64_t s_end = min(A.n_pts, s_begin + A.per_slice);
  load_band_tables(A, L, sm, f_b0);

  const int g = tid % A.gn;
  const int sl = tid / A.gn;  // < st by construction (gn * st == 256)
  const int n_runs = A.fb / kAnchor;
  const bool rx_on = tid < A.E * n_runs;
  const int e_rx = tid % A.E;
  const int run = tid / A.E;

  float2 Y[kAnchor];
#pragma unroll
  for (int j = 0; j < kAnchor; ++j) Y[j] = make_float2(0.f, 0.f);

  float* b_rhi = reinterpret_cast<float*>(sm + L.off_rhi);
  float* b_rlo = reinterpret_cast<float*>(sm + L.off_rlo);
  float* b_amp = reinterpret_cast<float*>(sm + L.off_amp);
  float2* b_st = reinterpret_cast<float2*>(sm + L.off_step);
  float2* W = reinterpret_cast<float2*>(sm + L.off_w);
  const float2* pp = reinterpret_cast<const float2*>(sm + L.off_pp);
  __syncthreads();

  const float2 k_run = A.t.kf[min(f_b0 + (rx_on ? run : 0) * kAnchor, A.F - 1)];
  const float a_run = A.t.af[min(f_b0 + (rx_on ? run : 0) * kAnchor, A.F - 1)];

  for (int64_t t0 = s_begin; t0 < s_end; t0 += A.st) {
    // ---------------- geometry + TX ----------------
    {
      int64_t s = t0 + sl;
      bool valid = s < s_end;
      int64_t si = valid ? s : t0;
      float w = 0.f;
      if (valid) {
        double x = A.pts[2 * si], z = A.pts[2 * si + 1];
        bool out = z < 0.0;
        if (A.convex) out = out || (x * x + (z + A.apex) * (z + A.apex) <= A.radius2);
        w = out ? 0.f : (float)A.rc[si];
      }
      SimusSink sink{W, pp, w, sl, A.st};
      tx_tile(A, L, sm, si, sl, g, sink);
    }
    __syncthreads();
    // ---------------- RX ----------------
    if (rx_on) {
      float2 Yt[kAnchor];
#pragma unroll
      for (int j = 0; j < kAnchor; ++j) Yt[j] = make_float2(0.f, 0.f);
      for (int s = 0; s < A.st; ++s) {
        float2 Gu[U], Su[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int idx = (u * A.E + e_rx) * L.pitch + s;
          Gu[u] = anchor_value(b_rhi[idx], b_rlo[idx], b_amp[idx], k_run, a_run);
          Su[u] = b_st[idx];
        }
        const float2* Wcol = W + (run * kAnchor) * A.st + s;
#pragma unroll
        for (int j = 0; j < kAnchor; ++j) {
          float2 rp = Gu[0];
          Gu[0] = cmul(Gu[0], Su[0]);
#pragma unroll
          for (int u = 1; u < U; ++u) {
            rp = cadd(rp, Gu[u]);
            Gu[u] = cmul(Gu[u], Su[u]);
          }
          Yt[j] = cfma(Wcol[j * A.st], rp, Yt[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < kAnchor; ++j) Y[j] = cadd(Y[j], Yt[j]);
    }
    __syncthreads();
  }
  if (rx_on) {
    float2* out = reinterpret_cast<float2*>(A.partial) + (size_t)blockIdx.y * A.F * A.E;
#pragma unroll
    for (int j = 0; j < kAnchor; ++j) {
      int f = f_b0 + run * kAnchor + j;
      if (f < A.F) out[(size_t)f * A.E + e_rx] = Y[j];
    }
  }
}

struct PfieldSink {
  const float2* pp;
  float acc;
  int fb_valid;
  __device__ __forceinline__ void operator()(int fl, float2 ps) {
    if (fl < fb_valid) {
      float2 v = cmul(pp[fl], ps);
      acc = fmaf(v.x, v.x, fmaf(v.y, v.y, acc));
    }
  }
};

__global__ void __launch_bounds__(kThreads, 2) pfield_band_kernel(const BandArgs A) {
  extern __shared__ __align__(16) unsigned char sm[];
  const SmemLayout L = smem_layout(A.gn, A.st, A.fb, A.E, false);
  const int tid = threadIdx.x;
  const int f_b0 = blockIdx.x * A.fb;
  const int64_t p_begin = (int64_t)blockIdx.y * A.per_slice;
  const int64_t p_end = min(A.n_pts, p_begin + A.per_slice);
  load_band_tables(A, L, sm, f_b0);
  __syncthreads();
  const int g = tid % A.gn;
  const int sl = tid / A.gn;
  const float2* pp = reinterpret_cast<const float2*>(sm + L.off_pp);
  float* out = reinterpret_cast<float*>(A.partial) + (size_t)blockIdx.x * A.n_pts;
  for (int64_t t0 = p_begin; t0 < p_end; t0 += A.st) {
    int64_t p = t0 + sl;
    bool valid = p < p_end;
    int64_t pi = valid ? p : t0;
    PfieldSink sink{pp, 0.f, min(A.fb, A.F - f_b0)};
    tx_tile(A, L, sm, pi, sl, g, sink);
    if (valid && g == 0) {
      double x = A.pts[2 * pi], z = A.pts[2 * pi + 1];
      bool o = z < 0.0;
      if (A.convex) o = o || (x * x + (z + A.apex) * (z + A.apex) <= A.radius2);
      out[pi] = o ? 0.f : sink.acc;
    }
  }
}

// out (layout) = probe_f * corr * sum over slices of partial[q][f][e], fixed slice order.
__global__ void simus_reduce(const float2* __restrict__ partial, int n_slices, int F, int E,
                             const float* __restrict__ probe, float corr, int full, int n_rows, int idx0,
                             float2* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)n_rows * E) return;
  const int row = (int)(i / E), e = (int)(i % E);
  const int f = full ? row - idx0 : row;
  float2 acc = make_float2(0.f, 0.f);
  if (f >= 0 && f < F) {
    for (int q = 0; q < n_slices; ++q) acc = cadd(acc, partial[((size_t)q * F + f) * E + e]);
    float s = probe[f] * corr;
    acc = make_float2(acc.x * s, acc.y * s);
  }
  out[i] = acc;
}

__global__ void pfield_reduce(const float* __restrict__ partial, int n_bands, int64_t n_pts, float corr,
                              float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pts) return;
  float acc = 0.f;
  for (int b = 0; b < n_bands; ++b) acc += partial[(size_t)b * n_pts + i];
  out[i] = sqrtf(acc * corr);
}

template <int U>
static cudaError_t launch_simus_band(const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(simus_band_kernel<U>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  if (e != cudaSuccess) return e;
  simus_band_kernel<U><<<dim3(c.n_bands, c.n_slices), kThreads, c.smem, s>>>(A);
  return cudaGetLastError();
}

cudaError_t launch_simus_band_any(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  switch (U) {
    case 1: return launch_simus_band<1>(c, A, s);
    case 2: return launch_simus_band<2>(c, A, s);
    case 3: return launch_simus_band<3>(c, A, s);
    case 4: return launch_simus_band<4>(c, A, s);
    default: return cudaErrorInvalidValue;
  }
}


}  // namespace fsg

// Plain fused FP32 simus and pfield sweeps for GB300 (sm_103a): set-up tables, the geometry
// pre-pass, the reductions and the launch dispatch.  The band kernels themselves are templates
// in fsg_sweep_kernels.cuh.
//
// simus, per chunk of scatterers:
//   geometry_kernel    once per (scatterer, source): double-float distance, amplitude
//                      (obliquity x centre-frequency sinc / sqrt(r) / n_sub), recurrence step
//                      (and half_seg sin(theta) with full-frequency directivity), written as
//                      one shared-memory-layout block per tile into an L2-sized cache;
//   simus_band_kernel  one CTA per SM, each sweeping an even share of the chunk's (band, tile)
//                      units; per tile: TMA bulk copy of the tile's block, TX (packed FP32x2
//                      recurrences, reduce-scatter of the source sums across the point's lanes,
//                      W[s][f] = rc pulse probe P), RX (thread = element x 32 frequencies,
//                      Y[e][f] += W[s][f] mean_u G), added into the band's partial slot;
// then simus_reduce sums the slots' partial spectra in a fixed order.  Neither the
// scatterer x element Green's tile nor W ever leaves the SM.
// pfield: pfield_band_kernel computes its geometry in place (one band for large grids) and
// accumulates |pulse probe P|^2; pfield_reduce sums the bands and takes the square root.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "fsg_common.cuh"
#include "fsg_internal.h"
#include "fsg_sweep_kernels.cuh"

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
    if (a.t.dph) a.t.dph[i] = make_float2((float)c, (float)s);
    if (m == 0) {
      if (a.t.wtx) a.t.wtx[e] = (float)w;
      sincos(2.0 * kPi * a.df * tau, &s, &c);
      a.t.dstep[e] = make_float2((float)c, (float)s);
    }
  }
}

// Geometry of a chunk's tiles, once per (scatterer, source) for all frequency bands.  A CTA
// takes one tile at a time: its scatterers' coordinates are split into double-float pairs
// once, then thread i handles (source, point) items i, i + 256, ...; consecutive threads take
// consecutive points, so the writes of a warp are contiguous.  Points past the end of the
// scatterer list repeat the tile's first point (their rc is 0 in the band kernel).
__global__ void __launch_bounds__(kThreads) geometry_kernel(const BandArgs A, int64_t chunk_tiles) {
  __shared__ float4 xz[kThreads];  // st <= 64 points of the tile
  const SmemLayout L = smem_layout(A.st, A.fb, A.E, A.U, A.plane_pad, true, A.C.ffd != 0);
  const int items = A.n_src * A.st;
  for (int64_t tile = blockIdx.x; tile < chunk_tiles; tile += gridDim.x) {
    __syncthreads();
    if (threadIdx.x < A.st) {
      int64_t s = A.chunk_s0 + tile * A.st + threadIdx.x;
      if (s >= A.n_pts) s = A.chunk_s0 + tile * A.st;
      const dfl hx = load_coord(A.pts + 2 * s), hz = load_coord(A.pts + 2 * s + 1);
      xz[threadIdx.x] = make_float4(hx.hi, hx.lo, hz.hi, hz.lo);
    }
    __syncthreads();
    unsigned char* blk = A.geo + tile * A.geo_bytes;
    float* rhi = reinterpret_cast<float*>(blk + L.off_rhi);
    float* rlo = reinterpret_cast<float*>(blk + L.off_rlo);
    float* amp = reinterpret_cast<float*>(blk + L.off_amp);
    float2* stp = reinterpret_cast<float2*>(blk + L.off_step);
    float* dir = A.C.ffd ? reinterpret_cast<float*>(blk + L.off_dir) : nullptr;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int pt = it % A.st, src = it / A.st;
      const int e = src / A.U, u = src - e * A.U;
      const float4 c = xz[pt];
      store_geometry(rhi, rlo, amp, stp, dir, u * L.plane + e * L.pitch + pt, dfl{c.x, c.y}, dfl{c.z, c.w}, A, src);
    }
  }
}

// out (layout) = probe_f * corr * sum over slots of partial[q][f][e], fixed slot order.
__global__ void simus_reduce(const float2* __restrict__ partial, int n_slices, int F, int E,
                             const float* __restrict__ probe, float corr, int full, int n_rows, int idx0,
                             const int* __restrict__ status, const double* __restrict__ rx_delays, double f0,
                             double df, float2* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)n_rows * E) return;
  if (*status != FSG_OK) {  // a sweep CTA gave up waiting: make the failure visible in the output
    out[i] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
    return;
  }
  const int row = (int)(i / E), e = (int)(i % E);
  const int f = full ? row - idx0 : row;
  float2 acc = make_float2(0.f, 0.f);
  if (f >= 0 && f < F) {
    for (int q = 0; q < n_slices; ++q) acc = cadd(acc, partial[((size_t)q * F + f) * E + e]);
    float s = probe[f] * corr;
    acc = make_float2(acc.x * s, acc.y * s);
    if (rx_delays) {
      double tau = rx_delays[e];
      if (isnan(tau)) tau = 0.0;
      double sn, cs;
      sincos(2.0 * kPi * (f0 + f * df) * tau, &sn, &cs);
      acc = cmul(acc, make_float2((float)cs, (float)-sn));
    }
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

cudaError_t launch_simus_band_any(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  if (c.kind >= 1) return A.C.ffd ? launch_simus_stash_ffd(U, c, A, s) : launch_simus_stash(U, c, A, s);
  return A.C.ffd ? launch_simus_band_ffd(U, c, A, s) : launch_simus_band_u<false>(U, c, A, s);
}

cudaError_t launch_pfield_band_any(const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  return A.C.ffd ? launch_pfield_band_ffd(c, A, s) : launch_pfield_band_gn<false>(c, A, s);
}

}  // namespace fsg

// Internal declarations shared by the sweep kernels (fsg_sweep.cu) and the C ABI (fsg_api.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "fsg_common.cuh"
#include "../../include/fsgb300.h"

namespace fsg {

struct Tables {
  float4* src_pos;   // [n_src] x_hi, x_lo, z_hi, z_lo
  float2* rot_e;     // [E] (cos theta_e, sin theta_e)
  float2* kf;        // [F] k_f double-float
  float* af;         // [F] attenuation Np/m at f
  float2* pp;        // [F] pulse * probe
  float* probe;      // [F]
  float2* da;        // [n_anchor][E] apod * exp(i 2 pi f_anchor tau)
  float2* dstep;     // [E] exp(i 2 pi df tau)
  float2* dph;       // [n_anchor][E] exp(i 2 pi f_anchor tau) (no apodization; NULL: not written)
  float* wtx;        // [E] transmit apodization, 0 for an element whose delay is NaN
};

struct SetupArgs {
  int E, U, F, n_anchor;
  double pitch, width, radius, c, att, f0, df, seg;
  const double* delays;
  const double* apod;
  const double* pulse;  // F complex128
  const double* probe;  // F float64
  Tables t;
};

struct BandArgs {
  const double* pts;   // [n_pts*2]
  const double* rc;    // [n_pts] (simus) or NULL (pfield)
  int64_t n_pts;
  int64_t per_slice;   // points per slice (multiple of st)
  Tables t;
  SweepConst C;
  int E, U, n_src, gn, st, fb, F, n_anchor;
  int plane_pad;       // extra words between the sub-element planes of the geometry arrays
  int convex;
  double apex, radius2;
  void* partial;       // simus: float2 [slots][F][E], zeroed, accumulated; pfield: float [bands][n_pts]
  // simus: scatterers are processed in chunks; the geometry of a chunk's tiles is computed
  // once by geometry_kernel into `geo` (one SmemLayout geometry block of geo_bytes per tile)
  // and copied into shared memory by each band's CTA with a TMA bulk copy
  unsigned char* geo;
  size_t geo_bytes;
  int64_t chunk_s0;    // first scatterer of the chunk (pts / rc are indexed globally)
  // simus: the chunk's n_bands x chunk_tiles (band, tile) units are split evenly over `grid`
  // CTAs in band-major order (cta_of_unit); the CTAs covering one band add into its partial
  // slots 0, 1, ... (< n_slots) in CTA order
  int64_t chunk_tiles;
  int n_bands, n_slots, grid;
  int* status;         // FSG_ETIMEOUT when a bounded wait gave up
};

// The CTA whose share of the units [0, units) split over `grid` CTAs contains unit x.  CTA c
// owns the units [c units / grid, (c + 1) units / grid).
__host__ __device__ inline int cta_of_unit(int64_t x, int64_t units, int grid) {
  return (int)(((x + 1) * grid - 1) / units);
}

struct SmemLayout {
  // Geometry arrays hold one value per (source, tile point): sub-element plane u, element e,
  // point column sl at u * plane + e * pitch + sl.  pitch = st + 1 keeps the receive reads
  // (consecutive elements) conflict-free; plane_pad spreads the transmit accesses (lanes =
  // sources g + GN i of one or more points) over the banks.
  int pitch, plane;
  size_t off_rhi, off_rlo, off_amp, off_step, off_dir, off_w, off_pp, off_kb, off_ka, off_aa, off_da, off_y, total;
  size_t geo_bytes;    // the geometry arrays, contiguous from offset 0
};

__host__ __device__ inline size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

// With ffd, a fifth geometry array holds half_seg * sin(theta) per (source, point).
__host__ __device__ inline SmemLayout smem_layout(int st, int fb, int E, int U, int plane_pad, bool with_w,
                                                  bool ffd = false) {
  SmemLayout L;
  L.pitch = st + 1;
  L.plane = E * L.pitch + plane_pad;
  size_t n = (size_t)U * L.plane;
  size_t o = 0;
  L.off_rhi = o; o = align16(o + n * 4);
  L.off_rlo = o; o = align16(o + n * 4);
  L.off_amp = o; o = align16(o + n * 4);
  L.off_step = o; o = align16(o + n * 8);
  L.off_dir = o; o = align16(o + (ffd ? n * 4 : 0));
  L.geo_bytes = o;
  L.off_w = o; o = align16(o + (with_w ? (size_t)fb * st * 8 : 0));
  L.off_pp = o; o = align16(o + (size_t)fb * 8);
  L.off_kb = o; o = align16(o + (size_t)fb * 4);  // FP32 wavenumber of each band frequency
  int na = fb / kAnchor;
  L.off_ka = o; o = align16(o + (size_t)na * 8);
  L.off_aa = o; o = align16(o + (size_t)na * 4);
  L.off_da = o; o = align16(o + (size_t)na * E * 8);
  // simus: each thread's running receive spectrum Y[kAnchor], laid out [j][thread]
  L.off_y = o; o = align16(o + (with_w ? (size_t)kAnchor * kThreads * 8 : 0));
  L.total = o;
  return L;
}

// simus_stash_kernel: frequencies per stash sub-block, and its shared memory.  Region 0 holds
// first the tile's geometry block (SmemLayout offsets) and then the stash [st][kStashFreqs][ep]
// of complex Green's terms, ep = E rounded up to odd (the transmit lanes of 2 to 8 points write
// one sub-block row each without bank conflicts).
constexpr int kStashFreqs = 8;
constexpr size_t kMaxDynSmem = 227 * 1024;
struct StashLayout {
  SmemLayout g;
  int ep;
  size_t off_w, off_pp, off_kb, off_dph, off_dstep, off_y, total;
};
__host__ __device__ inline StashLayout stash_layout(int st, int fb, int E, int U, int plane_pad, bool ffd) {
  StashLayout S;
  S.g = smem_layout(st, fb, E, U, plane_pad, true, ffd);
  S.ep = E | 1;
  const size_t stash = (size_t)st * kStashFreqs * S.ep * 8;
  size_t o = align16(S.g.geo_bytes > stash ? S.g.geo_bytes : stash);
  S.off_w = o; o = align16(o + (size_t)st * kStashFreqs * 8);
  S.off_pp = o; o = align16(o + (size_t)fb * 8);
  S.off_kb = o; o = align16(o + (ffd ? (size_t)fb * 4 : 0));
  S.off_dph = o; o = align16(o + (size_t)E * 8);
  S.off_dstep = o; o = align16(o + (size_t)E * 8);
  S.off_y = o; o = align16(o + (size_t)fb * E * 8);
  S.total = o;
  return S;
}

// simus_ws_kernel: the tile's geometry block from offset 0, then two stash buffers
// [stx][kStashFreqs][ep], two W buffers [stx][kStashFreqs] and the band tables.
struct WsLayout {
  SmemLayout g;  // the tile's geometry block, from offset 0
  int ep;
  size_t off_stash, off_w, off_pp, off_kb, off_dph, off_dstep, total;
};
__host__ __device__ inline WsLayout ws_layout(int stx, int fb, int E, int U, int plane_pad, bool ffd) {
  WsLayout S;
  S.g = smem_layout(stx, fb, E, U, plane_pad, true, ffd);
  S.ep = E | 1;
  size_t o = (S.g.geo_bytes + 127) & ~size_t(127);
  S.off_stash = o; o = align16(o + 2 * (size_t)stx * kStashFreqs * S.ep * 8);
  S.off_w = o; o = align16(o + 2 * (size_t)stx * kStashFreqs * 8);
  S.off_pp = o; o = align16(o + (size_t)fb * 8);
  S.off_kb = o; o = align16(o + (ffd ? (size_t)fb * 4 : 0));
  S.off_dph = o; o = align16(o + (size_t)E * 8);
  S.off_dstep = o; o = align16(o + (size_t)E * 8);
  S.total = o;
  return S;
}

struct SweepConfig {
  int kind;            // simus: 0 = simus_band_kernel, 1 = simus_stash_kernel
  int gn, st, fb, n_bands, plane_pad;
  int n_slices;        // pfield: point slices; simus: partial-spectrum slots per band
  int64_t per_slice;   // pfield: points per slice
  int64_t chunk_tiles; // simus: tiles per chunk
  int64_t n_chunks;
  size_t geo_bytes;    // simus: geometry block per tile
  size_t smem;
};

__global__ void setup_tables(SetupArgs a);
// Geometry of every (scatterer, source) of one chunk into A.geo (tile-major SmemLayout blocks).
__global__ void geometry_kernel(const BandArgs A, int64_t chunk_tiles);
// Launches simus_band_kernel<U> or simus_stash_kernel<U> (U = n_sub in 1..4), as c.kind says,
// with c's grid and shared memory.
cudaError_t launch_simus_band_any(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s);
cudaError_t launch_simus_stash(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s);
cudaError_t launch_simus_stash_ffd(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s);
// Launches pfield_band_kernel<gn> with c's grid and shared memory.
cudaError_t launch_pfield_band_any(const SweepConfig& c, const BandArgs& A, cudaStream_t s);
// rx_delays (NULL: none) undoes the transmit delay phase that the stash kernel leaves on its
// receive sums: out *= exp(-i 2 pi (f0 + f df) tau_e), tau_e = rx_delays[e] (NaN = 0).
__global__ void simus_reduce(const float2* __restrict__ partial, int n_slices, int F, int E,
                             const float* __restrict__ probe, float corr, int full, int n_rows, int idx0,
                             const int* __restrict__ status, const double* __restrict__ rx_delays, double f0,
                             double df, float2* __restrict__ out);
__global__ void pfield_reduce(const float* __restrict__ partial, int n_bands, int64_t n_pts, float corr,
                              float* __restrict__ out);

int set_error(int code, const char* fmt, ...);
int device_sm_count(int* out);
// The smallest workspace in which fsg_simus runs this request (one-tile scatterer chunks).
size_t simus_min_workspace(const FsgProbe* probe, const FsgFreqPlan* plan, int64_t n_scat, int ffd, int num_sms);
SweepConst make_sweep_const(const FsgProbe* p, const FsgMedium* m, const FsgFreqPlan* plan, int ffd);
void convex_geometry(const FsgProbe* p, int* convex, double* apex, double* radius2);
int check_cuda(cudaError_t err, const char* what);

}  // namespace fsg

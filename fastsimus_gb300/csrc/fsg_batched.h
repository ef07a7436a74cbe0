// Internal declarations of the batched multi-transmit sweep (fsg_batched.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fsg_common.cuh"

namespace fsg {

constexpr int kMaxPhantoms = 64;
constexpr int kBatchMaxE = 128;
constexpr int kBatchMaxTx = 80;

struct BatchPhantom {
  const double* scat;       // [n_scat*2]
  const double* rc;         // [n_scat]
  int64_t n_scat;
  int64_t tile0;            // tensor-core path: this phantom's first tile in the geometry cache
  int64_t geo0;             // FP32 batched path: this phantom's first scatterer in the geometry cache
  int n_freq, n_freq_full, freq_idx_start, n_bands, n_chunks, item0;
  double f0, df;
  float corr;
  float dalpha;             // per-step attenuation of this phantom's plan (Np/m)
  float2 dk;                // per-step wavenumber of this phantom's plan (double-float)
  const double* pulse_src;  // plan pulse spectrum, complex128 [n_freq]
  const double* probe_src;  // plan probe spectrum, float64 [n_freq]
  float2* kf;               // workspace: k_f double-float
  float* af;                // attenuation Np/m
  float2* freq_hz;          // f double-float
  float2* pp;               // pulse * probe
  float* probe;
  float2* out;              // [n_tx][n_freq_full][E] complex64 (caller-owned)
};

struct BatchArgs {
  BatchPhantom ph[kMaxPhantoms];
  int n_phantoms, n_items, E, U, n_tx, convex;
  int64_t chunk;
  const float4* src_pos;
  const float2* rot_e;
  const float2* tau;        // [n_tx][E] double-float seconds (NaN -> 0)
  const float* apod;        // [n_tx][E] (NaN delay -> 0)
  SweepConst C;
  double apex, radius2;
  int* queue;
  float2* partial;          // [n_items][fb][80][64]
  const float2* tx_in;      // optional [n_scat][n_freq][n_tx] transmit field (phantom 0); NULL = compute
  // geometry of every (scatterer, source), computed once per sweep by batched_geometry_kernel:
  // record (geo0 + s) * E * U + e * U + u holds (r_hi, r_lo, amp, step.x) and step.y
  float4* geo_a;
  float* geo_b;
  // full-frequency directivity: half_seg * sin(theta) per record (NULL: the centre-frequency
  // directivity is folded into the amplitude)
  float* geo_c;
};

struct BatchSetupArgs {
  BatchPhantom ph[kMaxPhantoms];
  int n_phantoms, n_tx, E;
  double c, att;
  const double* delays;     // [n_tx][E]
  const double* apod_src;   // [n_tx][E] or NULL
  float2* tau;
  float* apod;
};

struct BatchReduceArgs {
  BatchPhantom ph[kMaxPhantoms];
  int n_phantoms, n_tx, E, fb;
  int tx_pad, e_pad;        // partial layout [item][fb][tx_pad][e_pad]
  int apply_pp;             // 1: the partials lack the pulse x probe factor (tensor-core path)
  const float2* partial;
};

size_t batched_smem_bytes(int fb, int eb, int bt, int pk);
// Padded element count of the FP32 batched kernel's tiles (64 or 128).
int batched_pad_elements(int n_elements);
__global__ void batched_geometry_kernel(const __grid_constant__ BatchArgs A);
// Launches batched_kernel<fb, eb, bt, pk, minb, nth>; cudaErrorInvalidValue for a shape that is not compiled.
cudaError_t launch_batched(int fb, int eb, int bt, int pk, int minb, int nth, int grid, const BatchArgs& A,
                           cudaStream_t s);
bool batched_shape_supported(int fb, int eb, int bt, int pk, int minb, int nth);
__global__ void batched_setup(const __grid_constant__ BatchSetupArgs a);
__global__ void batched_reduce(const __grid_constant__ BatchReduceArgs a);

}  // namespace fsg

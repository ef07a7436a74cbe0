// Templates of the plain sweep kernels (simus_band_kernel, pfield_band_kernel) and their
// launchers, shared by the translation units that instantiate them: fsg_sweep.cu (without
// full-frequency directivity) and fsg_sweep_ffd.cu (with it), compiled in parallel.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "fsg_common.cuh"
#include "fsg_internal.h"
#include "fsg_tc.cuh"

namespace fsg {

constexpr size_t kBulkPiece = 32 * 1024;            // bytes per TMA bulk copy instruction
constexpr uint32_t kBulkWaitTries = 1u << 26;       // bound on the polls of one copy's mbarrier

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
  float* kb = reinterpret_cast<float*>(sm + L.off_kb);
  for (int i = threadIdx.x; i < A.fb; i += blockDim.x) {
    int f = f_b0 + i;
    pp[i] = (f < A.F) ? A.t.pp[f] : make_float2(0.f, 0.f);
    kb[i] = A.t.kf[min(f, A.F - 1)].x;
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

// Geometry of one (point, source) into the geometry arrays at word index idx; with
// full-frequency directivity also half_seg * sin(theta) into dir.
__device__ __forceinline__ void store_geometry(float* rhi, float* rlo, float* amp, float2* stp, float* dir, int idx,
                                               dfl xs, dfl zs, const BandArgs& A, int src) {
  const int e = src / A.U;
  const SrcGeo geo = source_geometry(xs, zs, A.t.src_pos[src], A.t.rot_e[e], A.C);
  rhi[idx] = geo.r_hi;
  rlo[idx] = geo.r_lo;
  amp[idx] = geo.amp;
  stp[idx] = geo.step;
  if (dir) dir[idx] = A.C.half_seg * geo.sth;
}

// TX over one band for one tile (with the tile's geometry computed here first when kGeo).
// Each thread owns point `sl` of the tile and sources g + GN i (i < 16); the GN threads of a
// point are GN adjacent lanes of one warp.  Frequencies are processed in blocks of GN steps:
// every lane keeps its partial source sums of the block, then a reduce-scatter across the GN
// lanes (log2 GN shuffle levels, halving the exchanged values each level) leaves lane g with
// the full sum of frequency block + g.  `sink(f_local, psum)` is therefore called by every
// lane, once per block, each for its own frequency.  With FFD every term is weighted by its
// directivity at the step's frequency, sinc(k_f half_seg sin(theta)), folded into the packed
// source sum as a fused multiply-add.
template <int GN, bool kGeo, bool FFD, class Sink>
__device__ __forceinline__ void tx_tile(const BandArgs& A, const SmemLayout& L, unsigned char* sm, int64_t p_idx,
                                        int sl, int g, Sink& sink) {
  float* b_rhi = reinterpret_cast<float*>(sm + L.off_rhi);
  float* b_rlo = reinterpret_cast<float*>(sm + L.off_rlo);
  float* b_amp = reinterpret_cast<float*>(sm + L.off_amp);
  float2* b_st = reinterpret_cast<float2*>(sm + L.off_step);
  const float2* ka = reinterpret_cast<const float2*>(sm + L.off_ka);
  const float* aa = reinterpret_cast<const float*>(sm + L.off_aa);
  const float2* da = reinterpret_cast<const float2*>(sm + L.off_da);
  float* b_dir = reinterpret_cast<float*>(sm + L.off_dir);
  const float* kb = reinterpret_cast<const float*>(sm + L.off_kb);

  // 1. geometry of my sources, parked in shared memory (rolled loop: one copy of the code)
  if constexpr (kGeo) {
    const dfl xs = load_coord(A.pts + 2 * p_idx);
    const dfl zs = load_coord(A.pts + 2 * p_idx + 1);
#pragma unroll 1
    for (int i = 0; i < kSrcPerThread; ++i) {
      const int src = g + GN * i;
      if (src < A.n_src) {
        const int e = src / A.U, u = src - e * A.U;
        store_geometry(b_rhi, b_rlo, b_amp, b_st, FFD ? b_dir : nullptr, u * L.plane + e * L.pitch + sl, xs, zs, A,
                       src);
      }
    }
  }
  // 2. transmit sweep: exact anchor every kTxAnchor steps, FP32 recurrence in between.
  // The thread's sources i = 2p and 2p+1 share one packed FP32x2 lane pair (real and
  // imaginary parts in separate pairs), so a step costs four packed instructions per two
  // sources and the source sum two packed adds.
  constexpr int kPairs = kSrcPerThread / 2;
  float2 Gr[kPairs], Gi[kPairs], Sr[kPairs], Si[kPairs], Sn[kPairs];
  float2 Dh[FFD ? kPairs : 1];  // FFD: half_seg sin(theta) of the pair's two sources
  const int n_tx_anchor = (A.fb + kTxAnchor - 1) / kTxAnchor;
  for (int m = 0; m < n_tx_anchor; ++m) {
    const int am = m * (kTxAnchor / kAnchor);  // index into the band's kAnchor-spaced tables
#pragma unroll
    for (int p = 0; p < kPairs; ++p) {
      float2 gv[2], sv[2];
      float dv[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int src = g + GN * (2 * p + h);
        gv[h] = make_float2(0.f, 0.f);
        sv[h] = make_float2(0.f, 0.f);
        dv[h] = 0.f;
        if (src < A.n_src) {
          const int e = src / A.U, u = src - e * A.U;
          const int idx = u * L.plane + e * L.pitch + sl;
          gv[h] = cmul(anchor_value(b_rhi[idx], b_rlo[idx], b_amp[idx], ka[am], aa[am]), da[am * A.E + e]);
          if (m == 0) sv[h] = cmul(b_st[idx], A.t.dstep[e]);
          if (FFD) dv[h] = b_dir[idx];
        }
      }
      if constexpr (FFD) Dh[p] = make_float2(dv[0], dv[1]);
      Gr[p] = make_float2(gv[0].x, gv[1].x);
      Gi[p] = make_float2(gv[0].y, gv[1].y);
      if (m == 0) {
        Sr[p] = make_float2(sv[0].x, sv[1].x);
        Si[p] = make_float2(sv[0].y, sv[1].y);
        Sn[p] = make_float2(-sv[0].y, -sv[1].y);
      }
    }
    const int n_steps = min(kTxAnchor, A.fb - m * kTxAnchor);  // a multiple of kAnchor, so of GN
#pragma unroll 1
    for (int jb = 0; jb < n_steps; jb += GN) {
      float vr[GN], vi[GN];
#pragma unroll
      for (int j = 0; j < GN; ++j) {
        float2 ar, ai;
        if constexpr (FFD) {
          const float k = kb[m * kTxAnchor + jb + j];
          const float2 kk = make_float2(k, k);
#pragma unroll
          for (int p = 0; p < kPairs; ++p) {
            const float2 d = sinc_poly2(__fmul2_rn(Dh[p], kk));
            ar = p ? __ffma2_rn(Gr[p], d, ar) : __fmul2_rn(Gr[p], d);
            ai = p ? __ffma2_rn(Gi[p], d, ai) : __fmul2_rn(Gi[p], d);
            cstep2(Gr[p], Gi[p], Sr[p], Si[p], Sn[p]);
          }
        } else {
          ar = Gr[0];
          ai = Gi[0];
          cstep2(Gr[0], Gi[0], Sr[0], Si[0], Sn[0]);
#pragma unroll
          for (int p = 1; p < kPairs; ++p) {
            ar = __fadd2_rn(ar, Gr[p]);
            ai = __fadd2_rn(ai, Gi[p]);
            cstep2(Gr[p], Gi[p], Sr[p], Si[p], Sn[p]);
          }
        }
        vr[j] = ar.x + ar.y;
        vi[j] = ai.x + ai.y;
      }
      // reduce-scatter: at level h the lane with bit h set keeps the upper half of its values
#pragma unroll
      for (int h = GN / 2; h >= 1; h >>= 1) {
        const bool up = (g & h) != 0;
#pragma unroll
        for (int i = 0; i < h; ++i) {
          const float sr = up ? vr[i] : vr[i + h], si = up ? vi[i] : vi[i + h];
          const float kr = up ? vr[i + h] : vr[i], ki = up ? vi[i + h] : vi[i];
          vr[i] = kr + __shfl_xor_sync(0xffffffffu, sr, h);
          vi[i] = ki + __shfl_xor_sync(0xffffffffu, si, h);
        }
      }
      sink(m * kTxAnchor + jb + g, make_float2(vr[0], vi[0]));
    }
  }
}

struct SimusSink {
  float2* W;        // [st][fb]
  const float2* pp; // [fb]
  float w;          // rc (0 when out of field or padding)
  int sl, fb;
  __device__ __forceinline__ void operator()(int fl, float2 ps) {
    float2 v = cmul(pp[fl], ps);
    W[sl * fb + fl] = make_float2(w * v.x, w * v.y);
  }
};

// One CTA sweeps its share of the chunk's (band, tile) units: units [c W / G, (c + 1) W / G) of
// W = n_bands x chunk_tiles in band-major order, i.e. one or two segments of consecutive tiles
// of one band each.  Per segment: the band's tables into shared memory, then per tile the TMA
// copy of the tile's geometry block, the transmit sums (tx_tile) into W, and the receive
// accumulation of every element over the tile's scatterers; at the end of the segment the
// running receive spectrum is added into the band's partial slot for this CTA.
template <int U, int GN, bool FFD>
__global__ void __launch_bounds__(kThreads, 1) simus_band_kernel(const BandArgs A) {
  extern __shared__ __align__(16) unsigned char sm[];
  const SmemLayout L = smem_layout(A.st, A.fb, A.E, A.U, A.plane_pad, true, FFD);
  __shared__ uint64_t s_mbar;
  __shared__ int s_fail;
  const int tid = threadIdx.x;
  if (tid == 0) {
    tc::mbar_init(&s_mbar, 1);
    tc::fence_mbar_init();
    s_fail = 0;
  }

  const int g = tid % GN;
  const int sl = tid / GN;  // < st by construction (gn * st == 256)
  const int n_runs = A.fb / kAnchor;
  const bool rx_on = tid < A.E * n_runs;
  const int e_rx = tid % A.E;
  const int run = tid / A.E;

  float* b_rhi = reinterpret_cast<float*>(sm + L.off_rhi);
  float* b_rlo = reinterpret_cast<float*>(sm + L.off_rlo);
  float* b_amp = reinterpret_cast<float*>(sm + L.off_amp);
  float2* b_st = reinterpret_cast<float2*>(sm + L.off_step);
  float2* W = reinterpret_cast<float2*>(sm + L.off_w);
  const float2* pp = reinterpret_cast<const float2*>(sm + L.off_pp);
  const float* b_dir = reinterpret_cast<const float*>(sm + L.off_dir);
  const float* kb = reinterpret_cast<const float*>(sm + L.off_kb);
  // Running receive spectrum of this thread, kept in shared memory ([j][thread]) so the
  // registers go to the per-tile partials and the recurrence state.
  float2* Ys = reinterpret_cast<float2*>(sm + L.off_y);

  const int64_t units = (int64_t)A.n_bands * A.chunk_tiles;
  const int64_t u_end = (int64_t)(blockIdx.x + 1) * units / A.grid;
  const int64_t s_stop = min(A.n_pts, A.chunk_s0 + A.chunk_tiles * A.st);
  uint32_t phase = 0;
  for (int64_t u = (int64_t)blockIdx.x * units / A.grid; u < u_end;) {
    const int band = (int)(u / A.chunk_tiles);
    const int64_t t_lo = u - (int64_t)band * A.chunk_tiles;
    const int64_t t_hi = min(A.chunk_tiles, t_lo + (u_end - u));
    u += t_hi - t_lo;
    const int slot = (int)blockIdx.x - cta_of_unit((int64_t)band * A.chunk_tiles, units, A.grid);
    const int f_b0 = band * A.fb;
    // the previous segment's readers of the tables finished at the barrier that closed its
    // last tile
    load_band_tables(A, L, sm, f_b0);
#pragma unroll
    for (int j = 0; j < kAnchor; ++j) Ys[j * kThreads + tid] = make_float2(0.f, 0.f);
    __syncthreads();

    const float2 k_run = A.t.kf[min(f_b0 + (rx_on ? run : 0) * kAnchor, A.F - 1)];
    const float a_run = A.t.af[min(f_b0 + (rx_on ? run : 0) * kAnchor, A.F - 1)];

    for (int64_t tile = t_lo; tile < t_hi; ++tile) {
      const int64_t t0 = A.chunk_s0 + tile * A.st;
      // ---------------- geometry: TMA bulk copy of the tile's block ----------------
      // The previous tile's reads of these arrays finished at the barrier that closed it; the
      // proxy fence orders them before the asynchronous writes.  Thread 0 waits (bounded) and
      // the barrier publishes the data and the outcome to the CTA.
      if (tid == 0) {
        const unsigned char* src = A.geo + tile * A.geo_bytes;
        tc::fence_proxy_async_smem();
        tc::mbar_arrive_expect_tx(&s_mbar, (uint32_t)A.geo_bytes);
        for (size_t off = 0; off < A.geo_bytes; off += kBulkPiece)
          tc::bulk_g2s(sm + off, src + off, (uint32_t)min(kBulkPiece, A.geo_bytes - off), &s_mbar);
        if (!tc::mbar_wait_bounded(&s_mbar, phase, kBulkWaitTries)) s_fail = 1;
      }
      phase ^= 1u;
      __syncthreads();
      if (s_fail) break;
      // ---------------- TX ----------------
      {
        int64_t s = t0 + sl;
        bool valid = s < s_stop;
        int64_t si = valid ? s : t0;
        float w = 0.f;
        if (valid) {
          double x = A.pts[2 * si], z = A.pts[2 * si + 1];
          bool out = z < 0.0;
          if (A.convex) out = out || (x * x + (z + A.apex) * (z + A.apex) <= A.radius2);
          w = out ? 0.f : (float)A.rc[si];
        }
        SimusSink sink{W, pp, w, sl, A.fb};
        tx_tile<GN, false, FFD>(A, L, sm, si, sl, g, sink);
      }
      __syncthreads();
      // ---------------- RX ----------------
      if (rx_on) {
        float2 Yt[kAnchor];
#pragma unroll
        for (int j = 0; j < kAnchor; ++j) Yt[j] = make_float2(0.f, 0.f);
#pragma unroll 1
        // two scatterers per pass (st is even): independent recurrences give the scheduler two
        // chains per sub-element to interleave; both accumulate into the same partial
        for (int s = 0; s < A.st; s += 2) {
          // the scatterers' fields over my run of frequencies: contiguous, read 2 per load
          const float4* Wa = reinterpret_cast<const float4*>(W + s * A.fb + run * kAnchor);
          const float4* Wb = reinterpret_cast<const float4*>(W + (s + 1) * A.fb + run * kAnchor);
          float2 Ga[U], Sa[U], Gb[U], Sb[U];
          float2 Dab[FFD ? U : 1];  // FFD: half_seg sin(theta) of (s, s + 1)
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int idx = u * L.plane + e_rx * L.pitch + s;
            Ga[u] = anchor_value(b_rhi[idx], b_rlo[idx], b_amp[idx], k_run, a_run);
            Sa[u] = b_st[idx];
            Gb[u] = anchor_value(b_rhi[idx + 1], b_rlo[idx + 1], b_amp[idx + 1], k_run, a_run);
            Sb[u] = b_st[idx + 1];
            if constexpr (FFD) Dab[u] = make_float2(b_dir[idx], b_dir[idx + 1]);
          }
#pragma unroll
          for (int j = 0; j < kAnchor; ++j) {
            float2 ra, rb;
            if constexpr (FFD) {
              // each sub-element term weighted by its directivity at this frequency
              const float k = kb[run * kAnchor + j];
              ra = rb = make_float2(0.f, 0.f);
#pragma unroll
              for (int u = 0; u < U; ++u) {
                const float2 d = sinc_poly2(__fmul2_rn(Dab[u], make_float2(k, k)));
                ra = make_float2(fmaf(Ga[u].x, d.x, ra.x), fmaf(Ga[u].y, d.x, ra.y));
                rb = make_float2(fmaf(Gb[u].x, d.y, rb.x), fmaf(Gb[u].y, d.y, rb.y));
                Ga[u] = cmul(Ga[u], Sa[u]);
                Gb[u] = cmul(Gb[u], Sb[u]);
              }
            } else {
              ra = Ga[0];
              rb = Gb[0];
              Ga[0] = cmul(Ga[0], Sa[0]);
              Gb[0] = cmul(Gb[0], Sb[0]);
#pragma unroll
              for (int u = 1; u < U; ++u) {
                ra = cadd(ra, Ga[u]);
                rb = cadd(rb, Gb[u]);
                Ga[u] = cmul(Ga[u], Sa[u]);
                Gb[u] = cmul(Gb[u], Sb[u]);
              }
            }
            const float4 wa = Wa[j >> 1], wb = Wb[j >> 1];
            Yt[j] = cfma((j & 1) ? make_float2(wa.z, wa.w) : make_float2(wa.x, wa.y), ra, Yt[j]);
            Yt[j] = cfma((j & 1) ? make_float2(wb.z, wb.w) : make_float2(wb.x, wb.y), rb, Yt[j]);
          }
        }
#pragma unroll
        for (int j = 0; j < kAnchor; ++j) Ys[j * kThreads + tid] = cadd(Ys[j * kThreads + tid], Yt[j]);
      }
      __syncthreads();
    }
    if (s_fail) break;
    if (slot >= A.n_slots) {  // cannot happen for the host's slot count; fail loudly if it does
      if (tid == 0) atomicExch(A.status, FSG_EINVAL);
      break;
    }
    if (rx_on) {
      float2* out = reinterpret_cast<float2*>(A.partial) + (size_t)slot * A.F * A.E;
#pragma unroll
      for (int j = 0; j < kAnchor; ++j) {
        int f = f_b0 + run * kAnchor + j;
        if (f < A.F) {
          float2* o = out + (size_t)f * A.E + e_rx;
          *o = cadd(*o, Ys[j * kThreads + tid]);
        }
      }
    }
  }
  if (tid == 0 && s_fail) atomicExch(A.status, FSG_ETIMEOUT);
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

template <int GN, bool FFD>
__global__ void __launch_bounds__(kThreads, (GN >= 32 || FFD) ? 1 : 2) pfield_band_kernel(const BandArgs A) {
  extern __shared__ __align__(16) unsigned char sm[];
  const SmemLayout L = smem_layout(A.st, A.fb, A.E, A.U, A.plane_pad, false, FFD);
  const int tid = threadIdx.x;
  const int f_b0 = blockIdx.x * A.fb;
  const int64_t p_begin = (int64_t)blockIdx.y * A.per_slice;
  const int64_t p_end = min(A.n_pts, p_begin + A.per_slice);
  load_band_tables(A, L, sm, f_b0);
  __syncthreads();
  const int g = tid % GN;
  const int sl = tid / GN;
  const float2* pp = reinterpret_cast<const float2*>(sm + L.off_pp);
  float* out = reinterpret_cast<float*>(A.partial) + (size_t)blockIdx.x * A.n_pts;
  for (int64_t t0 = p_begin; t0 < p_end; t0 += A.st) {
    int64_t p = t0 + sl;
    bool valid = p < p_end;
    int64_t pi = valid ? p : t0;
    PfieldSink sink{pp, 0.f, min(A.fb, A.F - f_b0)};
    tx_tile<GN, true, FFD>(A, L, sm, pi, sl, g, sink);
    // each lane holds the band's |p|^2 over its own frequencies: sum the GN lanes in a fixed tree
    float acc = sink.acc;
#pragma unroll
    for (int off = 1; off < GN; off <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (valid && g == 0) {
      double x = A.pts[2 * pi], z = A.pts[2 * pi + 1];
      bool o = z < 0.0;
      if (A.convex) o = o || (x * x + (z + A.apex) * (z + A.apex) <= A.radius2);
      out[pi] = o ? 0.f : acc;
    }
  }
}

template <int U, int GN, bool FFD>
static cudaError_t launch_simus_band(const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  cudaError_t e =
      cudaFuncSetAttribute(simus_band_kernel<U, GN, FFD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  if (e != cudaSuccess) return e;
  simus_band_kernel<U, GN, FFD><<<A.grid, kThreads, c.smem, s>>>(A);
  return cudaGetLastError();
}

template <int U, bool FFD>
static cudaError_t launch_simus_band_gn(const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  switch (c.gn) {
    case 4: return launch_simus_band<U, 4, FFD>(c, A, s);
    case 8: return launch_simus_band<U, 8, FFD>(c, A, s);
    case 16: return launch_simus_band<U, 16, FFD>(c, A, s);
    case 32: return launch_simus_band<U, 32, FFD>(c, A, s);
    default: return cudaErrorInvalidValue;
  }
}

template <bool FFD>
static cudaError_t launch_simus_band_u(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  switch (U) {
    case 1: return launch_simus_band_gn<1, FFD>(c, A, s);
    case 2: return launch_simus_band_gn<2, FFD>(c, A, s);
    case 3: return launch_simus_band_gn<3, FFD>(c, A, s);
    case 4: return launch_simus_band_gn<4, FFD>(c, A, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int GN, bool FFD>
static cudaError_t launch_pfield_band(const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  cudaError_t e =
      cudaFuncSetAttribute(pfield_band_kernel<GN, FFD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  if (e != cudaSuccess) return e;
  pfield_band_kernel<GN, FFD><<<dim3(c.n_bands, c.n_slices), kThreads, c.smem, s>>>(A);
  return cudaGetLastError();
}

template <bool FFD>
static cudaError_t launch_pfield_band_gn(const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  switch (c.gn) {
    case 4: return launch_pfield_band<4, FFD>(c, A, s);
    case 8: return launch_pfield_band<8, FFD>(c, A, s);
    case 16: return launch_pfield_band<16, FFD>(c, A, s);
    case 32: return launch_pfield_band<32, FFD>(c, A, s);
    default: return cudaErrorInvalidValue;
  }
}

// Full-frequency-directivity launchers (fsg_sweep_ffd.cu).
cudaError_t launch_simus_band_ffd(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s);
cudaError_t launch_pfield_band_ffd(const SweepConfig& c, const BandArgs& A, cudaStream_t s);

}  // namespace fsg

// Batched multi-transmit, multi-phantom simus sweep (plain FP32, CUDA cores).
//
// Many plane-wave transmits share one plan per phantom (the reference's multi-transmit
// pattern, tests/_picmus_phantom_shared.py:319-367), so the Green's terms of a
// (scatterer, element, frequency) are generated once and used by every transmit.  Per
// frequency the two contractions of the step body (_simus_strategies.py:64-73) become small
// complex GEMMs over a tile of 64 scatterers:
//     TX:  P[s][t]  = sum_e Gm[s][e] * D[e][t]      (D = apod * exp(i 2 pi f tau_t,e))
//     RX:  Y[e][t] += sum_s Gm[s][e] * W[s][t]      (W = rc_s * pulse * probe * P)
// with Gm = mean_u G(s, e, u, f) generated in shared memory from the exact double-float
// anchor of each band.  With full-frequency directivity every term is weighted at its own
// frequency by sinc(k_f half_seg sin(theta)) (_simus_strategies.py:59-62), from half_seg
// sin(theta) cached per (scatterer, source) beside the rest of the geometry.  Y for the CTA's band (1 or 2 frequencies) stays in registers across
// all scatterer tiles of the work item.
//
// Persistent launch: one CTA per SM (x blocks_per_sm) pulls work items
// (phantom, band, scatterer chunk) from an atomic counter until the queue is empty -- there is
// no waiting anywhere, a CTA simply exits when the counter passes the item count.  Each item
// writes its partial spectrum; batched_reduce sums the chunks of a (phantom, band) in fixed
// order, so results are deterministic.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <type_traits>

#include "../../include/fsgb300.h"
#include "fsg_batched.h"
#include "fsg_common.cuh"
#include "fsg_internal.h"

namespace fsg {

constexpr int kBTX = 80;       // padded transmits
constexpr int kWPitch = 81;    // complex per W / D row
// Elements are padded to EB = 64 or 128 (a template parameter); a Gm row holds EB + 1 complex
// values (the pad keeps column reads conflict-free).
__host__ __device__ constexpr int gm_pitch(int eb) { return eb + 1; }

__device__ __forceinline__ void df_mul_exact(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = fmaf(a, b, -p);
}

// exp(i 2 pi f tau) for double-float f (Hz) and tau (s): the product reaches ~200 rad.
__device__ __forceinline__ float2 cis_two_pi_ftau(float2 f, float2 tau) {
  float p, e;
  df_mul_exact(f.x, tau.x, p, e);
  e = fmaf(f.x, tau.y, e);
  e = fmaf(f.y, tau.x, e);
  // p + e cycles; reduce the integer part away exactly
  float n = rintf(p);
  float x = __fsub_rn(p, n);  // exact
  x = __fadd_rn(x, e);
  float s, c;
  sincospif(2.0f * x, &s, &c);
  return make_float2(c, s);
}

// The B operands (D of the transmit product, W of the receive product) of the packed register
// tile: (b.x, b.y, -b.y, b.x), so that acc + a b is two FP32x2 FMAs with a broadcast,
// (acc.x, acc.y) + (a.x, a.x)(b.x, b.y) + (a.y, a.y)(-b.y, b.x), rounding exactly like cfma.
__device__ __forceinline__ float4 pk_operand(float2 b) { return make_float4(b.x, b.y, -b.y, b.x); }
__device__ __forceinline__ float2 pk_cfma(float2 a, float4 b, float2 acc) {
  acc = __ffma2_rn(make_float2(a.x, a.x), make_float2(b.x, b.y), acc);
  return __ffma2_rn(make_float2(a.y, a.y), make_float2(b.z, b.w), acc);
}

// FB frequencies per item, EB padded elements, BT scatterers per tile, NTH threads (256 or 512:
// 4 or 8 row groups of warps x 2 column groups); the transmit register tile is
// BT / (4 NTH / 64) scatterer rows x 5 transmits per thread, the receive tile EB / (4 NTH / 64)
// element rows x 5 transmits.  PK: the complex MACs on the FP32x2 pipe with (b, conj-swapped
// b) operands in shared memory.  MINB: CTAs per SM the register budget is cut for.
template <int FB, int EB, int BT, bool PK, int MINB, int NTH>
__global__ void __launch_bounds__(NTH, MINB) batched_kernel(const __grid_constant__ BatchArgs A) {
  extern __shared__ __align__(16) unsigned char sm[];
  constexpr int kGmPitch = gm_pitch(EB);
  constexpr int NWM = NTH / 64;                                      // row groups of warps
  constexpr int kRows = EB / (4 * NWM);                              // receive rows per thread
  constexpr int kTRows = BT / (4 * NWM);                             // transmit rows per thread
  using BOp = typename std::conditional<PK, float4, float2>::type;  // a B-operand entry
  float2* Gm = reinterpret_cast<float2*>(sm);                       // [FB][BT][kGmPitch]
  BOp* D = reinterpret_cast<BOp*>(Gm + FB * BT * kGmPitch);          // [FB][EB][kWPitch]
  BOp* W = D + FB * EB * kWPitch;                                    // [BT][kWPitch]
  float* rcs = reinterpret_cast<float*>(W + BT * kWPitch);           // [BT]
  __shared__ int s_item;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp % NWM, wn = warp / NWM, lm = lane & 3, ln = lane >> 2;
  const int E = A.E, U = A.U, T = A.n_tx;

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(A.queue, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= A.n_items) break;
    // decode item -> (phantom, band, chunk)
    int p = 0;
    while (p + 1 < A.n_phantoms && item >= A.ph[p + 1].item0) ++p;
    const BatchPhantom& P = A.ph[p];
    const int local = item - P.item0;
    const int band = local % P.n_bands;
    const int chunk = local / P.n_bands;
    const int f0 = band * FB;
    const int nf = min(FB, P.n_freq - f0);
    const int64_t s_begin = (int64_t)chunk * A.chunk;
    const int64_t s_end = min(P.n_scat, s_begin + A.chunk);

    // --- transmit matrices D[f][e][t] for the band (exact, per item) ---
    for (int i = tid; i < FB * EB * kBTX; i += NTH) {
      const int f = i / (EB * kBTX), r = i % (EB * kBTX), e = r / kBTX, t = r % kBTX;
      float2 v = make_float2(0.f, 0.f);
      if (f < nf && e < E && t < T) {
        const float2 tau = A.tau[t * E + e];  // double-float seconds, NaN already mapped to 0
        const float w = A.apod[t * E + e];
        if (w != 0.0f) {
          const float2 fr = P.freq_hz[f0 + f];
          float2 c = cis_two_pi_ftau(fr, tau);
          v = make_float2(w * c.x, w * c.y);
        }
      }
      if constexpr (PK) D[(f * EB + e) * kWPitch + t] = pk_operand(v);
      else D[(f * EB + e) * kWPitch + t] = v;
    }
    // band constants
    float2 pp[FB];
#pragma unroll
    for (int f = 0; f < FB; ++f) pp[f] = (f < nf) ? P.pp[f0 + f] : make_float2(0.f, 0.f);
    const float2 k0 = P.kf[f0];
    const float a0 = P.af[f0];
    const float kb0 = k0.x, kb1 = (f0 + 1 < P.n_freq) ? P.kf[f0 + 1].x : 0.f;  // FP32 k_f for the directivity
    SweepConst C = A.C;  // probe constants; the recurrence step belongs to this phantom's plan
    C.dk = P.dk;
    C.dalpha = P.dalpha;

    float2 Y[FB][kRows][5];
#pragma unroll
    for (int f = 0; f < FB; ++f)
#pragma unroll
      for (int i = 0; i < kRows; ++i)
#pragma unroll
        for (int j = 0; j < 5; ++j) Y[f][i][j] = make_float2(0.f, 0.f);

    for (int64_t t0 = s_begin; t0 < s_end; t0 += BT) {
      // --- the tile's reflectivities (0 out of field) ---
      if (tid < BT) {
        const int64_t s = t0 + tid;
        float w = 0.f;
        if (s < s_end) {
          const double x = P.scat[2 * s], z = P.scat[2 * s + 1];
          bool out = z < 0.0;
          if (A.convex) out = out || (x * x + (z + A.apex) * (z + A.apex) <= A.radius2);
          w = out ? 0.f : (float)P.rc[s];
        }
        rcs[tid] = w;
      }
      __syncthreads();
      // --- Green's matrix Gm[f][s][e] for the tile: thread (e, s-group of BT * EB / 256) ---
      {
        constexpr int kSpg = BT * EB / NTH;
        const int e = tid % EB;
        const int sg = tid / EB;
        for (int k = 0; k < kSpg; ++k) {
          const int sl = sg * kSpg + k;
          const int64_t s = t0 + sl;
          float2 g0 = make_float2(0.f, 0.f), g1 = make_float2(0.f, 0.f);
          if (e < E && s < s_end) {
            // cached geometry of (s, e, u): the U records of a thread are contiguous
            const int64_t rec = (P.geo0 + s) * (int64_t)(E * U) + e * U;
            for (int u = 0; u < U; ++u) {
              const float4 ga = A.geo_a[rec + u];
              const float2 a = anchor_value(ga.x, ga.y, ga.z, k0, a0);
              if (A.geo_c) {
                const float x = A.geo_c[rec + u];
                const float d0 = sinc_poly(kb0 * x);
                g0 = make_float2(fmaf(a.x, d0, g0.x), fmaf(a.y, d0, g0.y));
                if (FB > 1) {
                  const float2 a1 = cmul(a, make_float2(ga.w, A.geo_b[rec + u]));
                  const float d1 = sinc_poly(kb1 * x);
                  g1 = make_float2(fmaf(a1.x, d1, g1.x), fmaf(a1.y, d1, g1.y));
                }
              } else {
                g0 = cadd(g0, a);
                if (FB > 1) g1 = cadd(g1, cmul(a, make_float2(ga.w, A.geo_b[rec + u])));
              }
            }
          }
          Gm[sl * kGmPitch + e] = g0;
          if (FB > 1) Gm[(BT + sl) * kGmPitch + e] = g1;
        }
      }
      __syncthreads();
#pragma unroll
      for (int f = 0; f < FB; ++f) {
        const float2* G = Gm + f * BT * kGmPitch;
        if (A.tx_in) {
          // transmit field supplied by the caller (already includes pulse * probe): W = rc * p
          for (int i = tid; i < BT * kBTX; i += NTH) {
            const int sl = i / kBTX, t = i % kBTX;
            const int64_t sg = t0 + sl;
            float2 v = make_float2(0.f, 0.f);
            if (sg < s_end && t < T && f < nf) {
              const float2 pv = A.tx_in[((size_t)sg * P.n_freq + (f0 + f)) * T + t];
              v = make_float2(rcs[sl] * pv.x, rcs[sl] * pv.y);
            }
            if constexpr (PK) W[sl * kWPitch + t] = pk_operand(v);
            else W[sl * kWPitch + t] = v;
          }
        } else {
          // --- TX: P[s][t] = sum_e G[s][e] D[e][t]; thread rows s = wm*(BT/4) + lm + 4i,
          //     cols t = wn*40 + ln*5 + j
          float2 acc[kTRows][5];
  #pragma unroll
          for (int i = 0; i < kTRows; ++i)
  #pragma unroll
            for (int j = 0; j < 5; ++j) acc[i][j] = make_float2(0.f, 0.f);
          const BOp* Df = D + f * EB * kWPitch;
  #pragma unroll 4
          for (int e = 0; e < EB; ++e) {
            float2 a[kTRows];
            BOp b[5];
  #pragma unroll
            for (int i = 0; i < kTRows; ++i) a[i] = G[(wm * (BT / NWM) + lm + 4 * i) * kGmPitch + e];
  #pragma unroll
            for (int j = 0; j < 5; ++j) b[j] = Df[e * kWPitch + wn * 40 + ln * 5 + j];
  #pragma unroll
            for (int i = 0; i < kTRows; ++i)
  #pragma unroll
              for (int j = 0; j < 5; ++j) {
                if constexpr (PK) acc[i][j] = pk_cfma(a[i], b[j], acc[i][j]);
                else acc[i][j] = cfma(a[i], b[j], acc[i][j]);
              }
          }
          // W[s][t] = rc_s * pulse * probe * P
  #pragma unroll
          for (int i = 0; i < kTRows; ++i) {
            const int s = wm * (BT / NWM) + lm + 4 * i;
            const float w = rcs[s];
            const float2 sc = make_float2(w * pp[f].x, w * pp[f].y);
  #pragma unroll
            for (int j = 0; j < 5; ++j) {
              const float2 v = cmul(sc, acc[i][j]);
              if constexpr (PK) W[s * kWPitch + wn * 40 + ln * 5 + j] = pk_operand(v);
              else W[s * kWPitch + wn * 40 + ln * 5 + j] = v;
            }
          }
        }
        __syncthreads();
        // --- RX: Y[e][t] += sum_s G[s][e] W[s][t]; thread rows e = wm*(EB/4) + lm + 4i
#pragma unroll 4
        for (int s = 0; s < BT; ++s) {
          float2 a[kRows];
          BOp b[5];
#pragma unroll
          for (int i = 0; i < kRows; ++i) a[i] = G[s * kGmPitch + wm * (EB / NWM) + lm + 4 * i];
#pragma unroll
          for (int j = 0; j < 5; ++j) b[j] = W[s * kWPitch + wn * 40 + ln * 5 + j];
#pragma unroll
          for (int i = 0; i < kRows; ++i)
#pragma unroll
            for (int j = 0; j < 5; ++j) {
              if constexpr (PK) Y[f][i][j] = pk_cfma(a[i], b[j], Y[f][i][j]);
              else Y[f][i][j] = cfma(a[i], b[j], Y[f][i][j]);
            }
        }
        __syncthreads();
      }
    }
    // --- partial spectrum of this item: [item][f][t][e] ---
    float2* out = A.partial + (size_t)item * FB * kBTX * EB;
#pragma unroll
    for (int f = 0; f < FB; ++f)
#pragma unroll
      for (int i = 0; i < kRows; ++i)
#pragma unroll
        for (int j = 0; j < 5; ++j) {
          const int e = wm * (EB / NWM) + lm + 4 * i, t = wn * 40 + ln * 5 + j;
          out[((size_t)f * kBTX + t) * EB + e] = Y[f][i][j];
        }
  }
}

// Per-phantom frequency tables and the shared source / transmit tables.
__global__ void batched_setup(const __grid_constant__ BatchSetupArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (p < a.n_phantoms) {
    const BatchPhantom& P = a.ph[p];
    if (i < P.n_freq) {
      const double f = P.f0 + i * P.df;
      dfl k = split_double(2.0 * kPi * f / a.c);
      P.kf[i] = make_float2(k.hi, k.lo);
      P.af[i] = (float)(a.att / 8.685889638065035 * f / 1e6 * 1e2);
      dfl fh = split_double(f);
      P.freq_hz[i] = make_float2(fh.hi, fh.lo);
      const double pr = P.probe_src[i];
      P.pp[i] = make_float2((float)(P.pulse_src[2 * i] * pr), (float)(P.pulse_src[2 * i + 1] * pr));
      P.probe[i] = (float)pr;
    }
  }
  if (p == 0 && i < a.n_tx * a.E) {
    double tau = a.delays[i];
    double w = a.apod_src ? a.apod_src[i] : 1.0;
    if (isnan(tau)) { tau = 0.0; w = 0.0; }
    dfl t = split_double(tau);
    a.tau[i] = make_float2(t.hi, t.lo);
    a.apod[i] = (float)w;
  }
}

// out_p[t][row][e] = corr * probe_f * sum_chunks partial[item(p, band, chunk)][f - band*FB][t][e]
__global__ void batched_reduce(const __grid_constant__ BatchReduceArgs a) {
  const int p = blockIdx.y;
  const BatchPhantom& P = a.ph[p];
  const int64_t n_out = (int64_t)a.n_tx * P.n_freq_full * a.E;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_out; i += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(i % a.E);
    const int64_t r = i / a.E;
    const int row = (int)(r % P.n_freq_full);
    const int t = (int)(r / P.n_freq_full);
    const int f = row - P.freq_idx_start;
    float2 acc = make_float2(0.f, 0.f);
    if (f >= 0 && f < P.n_freq) {
      const int band = f / a.fb, fl = f % a.fb;
      for (int c = 0; c < P.n_chunks; ++c) {
        const int item = P.item0 + c * P.n_bands + band;
        acc = cadd(acc, a.partial[(((size_t)item * a.fb + fl) * a.tx_pad + t) * a.e_pad + e]);
      }
      if (a.apply_pp) acc = cmul(acc, P.pp[f]);
      const float s = P.probe[f] * P.corr;
      acc = make_float2(acc.x * s, acc.y * s);
    }
    P.out[i] = acc;
  }
}

// Geometry of every (scatterer, source) of every phantom, once per sweep (the FP32 path keeps
// the plain kernels' double-float distance and accurate step, so the cache carries r as a
// double-float pair).  A CTA takes `spb` scatterers at a time: their coordinates are split
// once into shared memory, then consecutive threads write consecutive sources.
__global__ void __launch_bounds__(kThreads) batched_geometry_kernel(const __grid_constant__ BatchArgs A) {
  __shared__ float4 xz[kThreads];
  const BatchPhantom& P = A.ph[blockIdx.y];
  const int n_src = A.E * A.U;
  const int spb = n_src >= kThreads ? 1 : kThreads / n_src;
  SweepConst C = A.C;
  C.dk = P.dk;
  C.dalpha = P.dalpha;
  for (int64_t s0 = (int64_t)blockIdx.x * spb; s0 < P.n_scat; s0 += (int64_t)gridDim.x * spb) {
    __syncthreads();
    if (threadIdx.x < spb && s0 + threadIdx.x < P.n_scat) {
      const int64_t s = s0 + threadIdx.x;
      const dfl hx = split_double(P.scat[2 * s]), hz = split_double(P.scat[2 * s + 1]);
      xz[threadIdx.x] = make_float4(hx.hi, hx.lo, hz.hi, hz.lo);
    }
    __syncthreads();
    for (int it = threadIdx.x; it < spb * n_src; it += blockDim.x) {
      const int sl = it / n_src, src = it % n_src;
      const int64_t s = s0 + sl;
      if (s >= P.n_scat) continue;
      const float4 c = xz[sl];
      const SrcGeo g = source_geometry(dfl{c.x, c.y}, dfl{c.z, c.w}, A.src_pos[src], A.rot_e[src / A.U], C);
      const int64_t rec = (P.geo0 + s) * (int64_t)n_src + src;
      A.geo_a[rec] = make_float4(g.r_hi, g.r_lo, g.amp, g.step.x);
      A.geo_b[rec] = g.step.y;
      if (A.geo_c) A.geo_c[rec] = C.half_seg * g.sth;
    }
  }
}

size_t batched_smem_bytes(int fb, int eb, int bt, int pk) {
  const size_t bop = pk ? sizeof(float4) : sizeof(float2);
  return (size_t)fb * bt * gm_pitch(eb) * sizeof(float2) + ((size_t)fb * eb * kWPitch + (size_t)bt * kWPitch) * bop +
         bt * sizeof(float);
}

int batched_pad_elements(int n_elements) { return n_elements <= 64 ? 64 : 128; }

template <int FB, int EB, int BT, bool PK, int MINB, int NTH>
static cudaError_t launch_batched_t(int grid, const BatchArgs& A, cudaStream_t s) {
  const size_t smem = batched_smem_bytes(FB, EB, BT, PK);
  auto k = batched_kernel<FB, EB, BT, PK, MINB, NTH>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<grid, NTH, smem, s>>>(A);
  return cudaGetLastError();
}

// The compiled tile shapes (batched_shape_supported lists them).
#define FSG_BATCHED_SHAPES(X)                                                                            \
  X(2, 64, 64, false, 1, 256) X(2, 64, 32, false, 1, 256) X(1, 64, 64, false, 1, 256)                  \
  X(1, 64, 32, false, 1, 256) X(1, 64, 128, false, 1, 256) X(1, 64, 64, true, 1, 256)                 \
  X(1, 64, 32, true, 1, 256) X(1, 64, 32, false, 2, 256) X(1, 128, 64, false, 1, 256)                 \
  X(1, 128, 32, false, 1, 256) X(2, 64, 64, false, 1, 512) X(1, 64, 64, false, 1, 512)                \
  X(1, 64, 128, false, 1, 512) X(1, 128, 64, false, 1, 512)

bool batched_shape_supported(int fb, int eb, int bt, int pk, int minb, int nth) {
#define FSG_X(FB, EB, BT, PK, MINB, NTH) \
  if (fb == FB && eb == EB && bt == BT && pk == (int)PK && minb == MINB && nth == NTH) return true;
  FSG_BATCHED_SHAPES(FSG_X)
#undef FSG_X
  return false;
}

cudaError_t launch_batched(int fb, int eb, int bt, int pk, int minb, int nth, int grid, const BatchArgs& A,
                           cudaStream_t s) {
#define FSG_X(FB, EB, BT, PK, MINB, NTH)                                                  \
  if (fb == FB && eb == EB && bt == BT && pk == (int)PK && minb == MINB && nth == NTH) \
    return launch_batched_t<FB, EB, BT, PK, MINB, NTH>(grid, A, s);
  FSG_BATCHED_SHAPES(FSG_X)
#undef FSG_X
  return cudaErrorInvalidValue;
}

}  // namespace fsg

// ------------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------------

namespace {

using namespace fsg;

size_t a256(size_t v) { return (v + 255) & ~size_t(255); }

struct BatchPlanLayout {
  int fb, eb, bt, pk, minb, nth, chunk, n_items;
  int n_bands[kMaxPhantoms], n_chunks[kMaxPhantoms], item0[kMaxPhantoms];
  int64_t geo0[kMaxPhantoms], max_scat;
  size_t off_src, off_rot, off_tau, off_apod, off_queue, off_tab[kMaxPhantoms], off_partial, off_geo_a, off_geo_b,
      off_geo_c, total;
};

int plan_layout(const FsgProbe* probe, const FsgPhantom* ph, int n_ph, int n_tx, const FsgBatchTuning* tu,
                BatchPlanLayout* L, int ffd = 0) {
  L->eb = batched_pad_elements(probe->n_elements);
  // two frequencies per item only fit the 64-element tile's shared memory
  L->fb = (L->eb > 64 || (tu && tu->freqs_per_item == 1)) ? 1 : 2;
  L->bt = (tu && tu->tile_scatterers > 0) ? tu->tile_scatterers : 64;
  L->pk = (tu && tu->packed) ? 1 : 0;
  L->nth = (tu && tu->threads_per_cta > 0) ? tu->threads_per_cta : 256;
  L->minb = (tu && tu->ctas_per_sm == 2 && batched_shape_supported(L->fb, L->eb, L->bt, L->pk, 2, L->nth)) ? 2 : 1;
  int64_t chunk = (tu && tu->chunk_scatterers > 0) ? tu->chunk_scatterers : 32768;
  chunk = ((chunk + L->bt - 1) / L->bt) * L->bt;
  L->chunk = (int)chunk;
  const int E = probe->n_elements, U = probe->n_sub;
  size_t o = 0;
  L->off_src = o; o += a256((size_t)E * U * 16);
  L->off_rot = o; o += a256((size_t)E * 8);
  L->off_tau = o; o += a256((size_t)n_tx * E * 8);
  L->off_apod = o; o += a256((size_t)n_tx * E * 4);
  L->off_queue = o; o += 256;
  int items = 0;
  int64_t scat = 0;
  L->max_scat = 0;
  for (int p = 0; p < n_ph; ++p) {
    const int F = ph[p].plan.n_freq;
    L->n_bands[p] = (F + L->fb - 1) / L->fb;
    L->n_chunks[p] = ph[p].n_scat > 0 ? (int)((ph[p].n_scat + chunk - 1) / chunk) : 1;
    L->item0[p] = items;
    items += L->n_bands[p] * L->n_chunks[p];
    L->off_tab[p] = o;
    o += a256((size_t)F * (8 + 4 + 8 + 8 + 4));
    L->geo0[p] = scat;
    scat += ph[p].n_scat;
    if (ph[p].n_scat > L->max_scat) L->max_scat = ph[p].n_scat;
  }
  L->n_items = items;
  L->off_partial = o;
  o += a256((size_t)items * L->fb * kBTX * L->eb * 8);
  L->off_geo_a = o;
  o += a256((size_t)scat * E * U * 16);
  L->off_geo_b = o;
  o += a256((size_t)scat * E * U * 4);
  L->off_geo_c = o;
  if (ffd) o += a256((size_t)scat * E * U * 4);
  L->total = o;
  return FSG_OK;
}

int validate_batch(const FsgProbe* probe, const FsgMedium* medium, const FsgPhantom* ph, int n_ph,
                   const double* delays, int n_tx) {
  if (!probe || !medium || !ph) return set_error(FSG_EINVAL, "probe, medium and phantoms must be non-NULL");
  if (n_ph < 1 || n_ph > kMaxPhantoms) return set_error(FSG_EINVAL, "n_phantoms must be in [1, %d]", kMaxPhantoms);
  if (n_tx < 1 || n_tx > kBatchMaxTx) return set_error(FSG_EUNSUPPORTED, "n_tx must be in [1, %d]", kBatchMaxTx);
  if (probe->n_elements < 1 || probe->n_elements > kBatchMaxE)
    return set_error(FSG_EUNSUPPORTED, "batched sweep supports n_elements <= %d (got %d)", kBatchMaxE, probe->n_elements);
  if (probe->n_sub < 1 || probe->n_sub > 8) return set_error(FSG_EUNSUPPORTED, "n_sub must be in [1, 8]");
  if (!delays) return set_error(FSG_EINVAL, "delays must be non-NULL");
  if (!(medium->speed_of_sound > 0) || !(medium->attenuation >= 0))
    return set_error(FSG_EINVAL, "speed_of_sound must be > 0 and attenuation >= 0");
  for (int p = 0; p < n_ph; ++p) {
    const FsgFreqPlan& pl = ph[p].plan;
    if (ph[p].n_scat < 0) return set_error(FSG_EINVAL, "phantom %d: n_scat < 0", p);
    if (ph[p].n_scat > 0 && (!ph[p].scat_xz || !ph[p].rc)) return set_error(FSG_EINVAL, "phantom %d: NULL inputs", p);
    if (!ph[p].out) return set_error(FSG_EINVAL, "phantom %d: NULL output", p);
    if (pl.n_freq < 1 || !pl.pulse_spectrum || !pl.probe_spectrum)
      return set_error(FSG_EINVAL, "phantom %d: empty plan", p);
    if (pl.freq_idx_start < 0 || pl.freq_idx_start + pl.n_freq > pl.n_freq_full)
      return set_error(FSG_EINVAL, "phantom %d: selected band does not fit n_freq_full", p);
  }
  return FSG_OK;
}

}  // namespace

extern "C" size_t fsg_simus_batched_workspace_size(const FsgProbe* probe, const FsgPhantom* phantoms,
                                                   int32_t n_phantoms, int32_t n_tx,
                                                   int32_t full_frequency_directivity,
                                                   const FsgBatchTuning* tuning) {
  if (!probe || !phantoms || n_phantoms < 1 || n_phantoms > kMaxPhantoms || n_tx < 1) return 0;
  BatchPlanLayout L;
  plan_layout(probe, phantoms, n_phantoms, n_tx, tuning, &L, full_frequency_directivity ? 1 : 0);
  return L.total;
}

static int32_t simus_batched_impl(const FsgProbe* probe, const FsgMedium* medium, const FsgPhantom* phantoms,
                                  int32_t n_phantoms, const double* delays, const double* apod, int32_t n_tx, int ffd,
                                  const FsgBatchTuning* tuning, const float2* tx_in, void* workspace,
                                  size_t workspace_bytes, void* stream_ptr) {
  int st = validate_batch(probe, medium, phantoms, n_phantoms, delays, n_tx);
  if (st != FSG_OK) return st;
  {
    BatchPlanLayout T;
    plan_layout(probe, phantoms, n_phantoms, n_tx, tuning, &T, ffd);
    if (!batched_shape_supported(T.fb, T.eb, T.bt, T.pk, T.minb, T.nth))
      return set_error(FSG_EUNSUPPORTED,
                       "batched tile shape (freqs_per_item %d, elements tile %d, tile_scatterers %d, packed %d, "
                       "threads %d) is not compiled into this library",
                       T.fb, T.eb, T.bt, T.pk, T.nth);
  }
  if (ffd) {
    // the per-frequency directivity is a polynomial valid for |k_f seg / 2| <= 2 pi (as in the
    // plain sweep): sub-elements up to two wavelengths of the highest frequency wide
    for (int p = 0; p < n_phantoms; ++p) {
      const FsgFreqPlan& pl = phantoms[p].plan;
      const double f_max = pl.freq_start + (pl.n_freq - 1) * pl.freq_step;
      const double x_max = 2.0 * kPi * f_max / medium->speed_of_sound * pl.seg_length / 2.0;
      if (x_max > 2.0 * kPi)
        return set_error(FSG_EUNSUPPORTED,
                         "full_frequency_directivity with sub-elements wider than two wavelengths "
                         "(phantom %d: k_max seg / 2 = %.3f > 2 pi) is not supported by this library",
                         p, x_max);
    }
  }
  BatchPlanLayout L;
  plan_layout(probe, phantoms, n_phantoms, n_tx, tuning, &L, ffd);
  if (!workspace || workspace_bytes < L.total)
    return set_error(FSG_EWORKSPACE, "workspace of %zu bytes is smaller than the %zu bytes required", workspace_bytes,
                     L.total);
  int sms = 0;
  {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return check_cuda(e, "device query");
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream_ptr);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  const int E = probe->n_elements, U = probe->n_sub;

  // shared source tables (positions, element rotation) through the plain set-up kernel
  {
    SetupArgs a;
    memset(&a, 0, sizeof(a));
    a.E = E;
    a.U = U;
    a.F = 0;
    a.n_anchor = 0;
    a.pitch = probe->pitch;
    a.width = probe->element_width;
    a.radius = probe->radius;
    a.c = medium->speed_of_sound;
    a.seg = probe->element_width / U;
    a.delays = delays;
    a.t.src_pos = reinterpret_cast<float4*>(ws + L.off_src);
    a.t.rot_e = reinterpret_cast<float2*>(ws + L.off_rot);
    setup_tables<<<(E * U + 127) / 128, 128, 0, s>>>(a);
    if ((st = check_cuda(cudaGetLastError(), "setup_tables launch")) != FSG_OK) return st;
  }
  BatchPhantom bp[kMaxPhantoms];
  memset(bp, 0, sizeof(bp));
  int max_f = 0;
  for (int p = 0; p < n_phantoms; ++p) {
    const FsgPhantom& q = phantoms[p];
    BatchPhantom& b = bp[p];
    b.scat = q.scat_xz;
    b.rc = q.rc;
    b.n_scat = q.n_scat;
    b.n_freq = q.plan.n_freq;
    b.n_freq_full = q.plan.n_freq_full;
    b.freq_idx_start = q.plan.freq_idx_start;
    b.n_bands = L.n_bands[p];
    b.n_chunks = L.n_chunks[p];
    b.item0 = L.item0[p];
    b.geo0 = L.geo0[p];
    b.f0 = q.plan.freq_start;
    b.df = q.plan.freq_step;
    b.corr = (float)q.plan.correction_factor;
    {
      const SweepConst cp = make_sweep_const(probe, medium, &q.plan, 0);
      b.dk = cp.dk;
      b.dalpha = cp.dalpha;
    }
    b.pulse_src = q.plan.pulse_spectrum;
    b.probe_src = q.plan.probe_spectrum;
    unsigned char* tb = ws + L.off_tab[p];
    const int F = q.plan.n_freq;
    b.kf = reinterpret_cast<float2*>(tb);
    b.freq_hz = reinterpret_cast<float2*>(tb + (size_t)F * 8);
    b.pp = reinterpret_cast<float2*>(tb + (size_t)F * 16);
    b.af = reinterpret_cast<float*>(tb + (size_t)F * 24);
    b.probe = reinterpret_cast<float*>(tb + (size_t)F * 28);
    b.out = static_cast<float2*>(q.out);
    if (F > max_f) max_f = F;
  }
  float2* tau = reinterpret_cast<float2*>(ws + L.off_tau);
  float* apw = reinterpret_cast<float*>(ws + L.off_apod);
  {
    BatchSetupArgs a;
    memcpy(a.ph, bp, sizeof(bp));
    a.n_phantoms = n_phantoms;
    a.n_tx = n_tx;
    a.E = E;
    a.c = medium->speed_of_sound;
    a.att = medium->attenuation;
    a.delays = delays;
    a.apod_src = apod;
    a.tau = tau;
    a.apod = apw;
    int n = max_f > n_tx * E ? max_f : n_tx * E;
    batched_setup<<<dim3((n + 127) / 128, n_phantoms), 128, 0, s>>>(a);
    if ((st = check_cuda(cudaGetLastError(), "batched_setup launch")) != FSG_OK) return st;
  }
  int* queue = reinterpret_cast<int*>(ws + L.off_queue);
  if ((st = check_cuda(cudaMemsetAsync(queue, 0, sizeof(int), s), "queue reset")) != FSG_OK) return st;
  float2* partial = reinterpret_cast<float2*>(ws + L.off_partial);
  {
    BatchArgs A;
    memcpy(A.ph, bp, sizeof(bp));
    A.n_phantoms = n_phantoms;
    A.n_items = L.n_items;
    A.E = E;
    A.U = U;
    A.n_tx = n_tx;
    A.chunk = L.chunk;
    A.src_pos = reinterpret_cast<const float4*>(ws + L.off_src);
    A.rot_e = reinterpret_cast<const float2*>(ws + L.off_rot);
    A.tau = tau;
    A.apod = apw;
    FsgFreqPlan any = phantoms[0].plan;
    A.C = make_sweep_const(probe, medium, &any, ffd);
    convex_geometry(probe, &A.convex, &A.apex, &A.radius2);
    A.queue = queue;
    A.partial = partial;
    A.tx_in = tx_in;
    A.geo_a = reinterpret_cast<float4*>(ws + L.off_geo_a);
    A.geo_b = reinterpret_cast<float*>(ws + L.off_geo_b);
    A.geo_c = ffd ? reinterpret_cast<float*>(ws + L.off_geo_c) : nullptr;
    if (L.max_scat > 0) {
      const int spb = E * U >= kThreads ? 1 : kThreads / (E * U);
      const int64_t want = (L.max_scat + spb - 1) / spb, cap = (int64_t)sms * 8;
      batched_geometry_kernel<<<dim3((unsigned)(want < cap ? want : cap), n_phantoms), kThreads, 0, s>>>(A);
      if ((st = check_cuda(cudaGetLastError(), "batched_geometry_kernel launch")) != FSG_OK) return st;
    }
    const int per_sm = (tuning && tuning->ctas_per_sm > 0) ? tuning->ctas_per_sm : 1;
    int grid = sms * per_sm;
    if (grid > L.n_items) grid = L.n_items;
    if ((st = check_cuda(launch_batched(L.fb, L.eb, L.bt, L.pk, L.minb, L.nth, grid, A, s),
                         "batched_kernel launch")) != FSG_OK)
      return st;
  }
  {
    BatchReduceArgs a;
    memcpy(a.ph, bp, sizeof(bp));
    a.n_phantoms = n_phantoms;
    a.n_tx = n_tx;
    a.E = E;
    a.fb = L.fb;
    a.tx_pad = kBTX;
    a.e_pad = L.eb;
    a.apply_pp = 0;
    a.partial = partial;
    batched_reduce<<<dim3(2 * sms, n_phantoms), 256, 0, s>>>(a);
    if ((st = check_cuda(cudaGetLastError(), "batched_reduce launch")) != FSG_OK) return st;
  }
  return FSG_OK;
}

extern "C" int32_t fsg_simus_batched(const FsgProbe* probe, const FsgMedium* medium, const FsgPhantom* phantoms,
                                     int32_t n_phantoms, const double* delays, const double* apod, int32_t n_tx,
                                     int32_t full_frequency_directivity, const FsgBatchTuning* tuning,
                                     void* workspace, size_t workspace_bytes, void* stream) {
  return simus_batched_impl(probe, medium, phantoms, n_phantoms, delays, apod, n_tx,
                            full_frequency_directivity ? 1 : 0, tuning, nullptr, workspace, workspace_bytes, stream);
}

extern "C" int32_t fsg_simus_batched_rx(const FsgProbe* probe, const FsgMedium* medium, const FsgPhantom* phantom,
                                        const double* delays, int32_t n_tx, const void* tx_field,
                                        const FsgBatchTuning* tuning, void* workspace, size_t workspace_bytes,
                                        void* stream) {
  if (!tx_field) return fsg::set_error(FSG_EINVAL, "tx_field must be non-NULL");
  return simus_batched_impl(probe, medium, phantom, 1, delays, nullptr, n_tx, 0, tuning,
                            static_cast<const float2*>(tx_field), workspace, workspace_bytes, stream);
}

// Tensor-core (tcgen05) multi-transmit simus sweep: Green's tiles generated on chip in FP32,
// split into BF16 hi + lo, three-product complex GEMMs with FP32 accumulation in TMEM.
//
// Work item = (phantom, band of `fb` consecutive frequencies, scatterer chunk); one CTA of 256
// threads per SM pulls items from an atomic counter.  Per tile of 64 scatterers and frequency f:
//
//   generate   Gm[s][e] = mean_u G(s, e, u, f)            (FP32 recurrence, 32 states / thread)
//   TX  (MMA)  D_tx[(c,s)][(c',t)] = sum_e Gc[s][e] * Dc'[e][t]     M=128 N=64 per chunk K=64
//              with c, c' in {re, im}: rows [Gr; Gi], columns [Dr | Di] per chunk of 32
//              transmits (at most two chunks per MMA pass)
//              P = (D_tx[0,s][0,t] - D_tx[1,s][1,t]) + i (D_tx[0,s][1,t] + D_tx[1,s][0,t])
//   RX  (MMA)  D_rx[f][(c,e)][(c',t)] += sum_s Gc[s][e] * Qc'[s][t]  M=128 N=64 nc K=64
//              with rows [Gr^T; Gi^T] (the same BF16 words as the TX operand) and columns
//              [Qr | Qi], Q = rc_s P; Y = D_rx[0][0] - D_rx[1][1] + i (D_rx[0][1] + D_rx[1][0]) is
//              formed once per item, and the reduction multiplies it by pulse x probe.
//
// Each real GEMM is A_hi B_hi + A_hi B_lo + A_lo B_hi (three tcgen05.mma kind::f16 per K step).
// TX operands are K-major; RX operands are written MN-major so that no thread transposes data.
// Every wait on an mbarrier is bounded: on timeout the CTA records FSG_ETIMEOUT in the status
// word, skips the remaining work, frees its TMEM and exits.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "../../include/fsgb300.h"
#include "fsg_batched.h"
#include "fsg_common.cuh"
#include "fsg_internal.h"
#include "fsg_tc.cuh"

namespace fsg {

constexpr int kTcT = 64;        // scatterers per tile
constexpr int kTcE = 64;        // padded elements
constexpr int kTcTxChunk = 32;  // transmits per column chunk: an accumulator has N = 64 nc columns
constexpr int kTcMaxTx = 96;    // up to nc = 3 chunks
constexpr int kTcMaxFb = 7;     // TMEM: the TX accumulator + N per band frequency <= 512 columns
// The TX product is formed at most two chunks (128 columns) at a time, so TMEM keeps
// 64 min(nc, 2) TX columns; band frequencies per item that fit: 7, 3, 2.
__host__ __device__ constexpr int tc_tx_chunks(int nc) { return nc < 2 ? nc : 2; }
__host__ __device__ constexpr int tc_max_fb(int nc) { return (512 - 64 * tc_tx_chunks(nc)) / (64 * nc); }
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kWaitTries = 1u << 26;

struct TcArgs {
  BatchPhantom ph[kMaxPhantoms];
  int n_phantoms, n_items, E, U, n_tx, fb, convex;
  int nc;           // transmit chunks of 32: N = 64 nc accumulator columns
  int64_t chunk;
  const float4* src_pos;
  const float2* rot_e;
  const float2* tau;
  const float* apod;
  SweepConst C;
  double apex, radius2;
  int* queue;
  int* status;
  float2* partial;  // [n_items][fb][32 nc][kTcE]
  const float4* geo;  // per (tile, state, thread) geometry of all phantoms, see tc_geometry_kernel
};

// Geometry for the tensor-core path (accuracy target 1e-3), in plain FP32 and without
// branches: distance from one rsqrt, the lambda/2 clip, obliquity with the 1e-16 horizon floor
// and the centre-frequency sinc (_pfield_math.py:70-118, :165-199), and the MUFU recurrence
// step (its ~4e-7 error compounds over at most seven steps).  Computed once per
// (scatterer, source) by tc_geometry_kernel; returns (clipped r, amplitude, step).
__device__ __forceinline__ float4 tc_geometry(float xs, float zs, float4 sp, float2 rot, const SweepConst& C) {
  const float dx = __fsub_rn(__fsub_rn(xs, sp.x), sp.y);
  const float dz = __fsub_rn(__fsub_rn(zs, sp.z), sp.w);
  const float d2 = fmaf(dx, dx, dz * dz);
  const float rinv = rsqrtf(fmaxf(d2, 1e-30f));
  const float r = d2 * rinv;
  const float a = (d2 > 0.0f) ? fminf(1.0f, fmaxf(-1.0f, dx * rinv)) : 1.0f;
  const float ca = sqrtf(fmaxf(0.0f, (1.0f - a) * (1.0f + a)));
  const float sth = fmaf(a, rot.x, -ca * rot.y);
  const float cth = fmaf(ca, rot.x, a * rot.y);
  const float rc = fmaxf(r, C.min_dist.x);
  float ob = (C.baffle == 0) ? cth : ((C.baffle == 1) ? 1.0f : __fdividef(cth, cth + C.baffle_val));
  ob = (cth <= 0.0f) ? 1e-16f : ob;
  const float x = C.dir_coef * sth;
  const float dir = (fabsf(x) < 1e-4f) ? 1.0f : __fdividef(__sinf(x), x);
  const float amp = ob * dir * rsqrtf(rc) * C.inv_nsub;
  float sn, cs;
  __sincosf(C.dk.x * rc, &sn, &cs);
  const float mag = __expf(-C.dalpha * rc);
  return make_float4(rc, amp, mag * cs, mag * sn);
}

// Anchor value amp exp(-a0 r) exp(i k0 r) at a band's first frequency, with k0 r reduced
// mod 2 pi in FP32 (error ~1e-7 |k0 r|, below 1e-4 rad here).
__device__ __forceinline__ float2 tc_anchor(float rc, float amp, float2 k0, float a0) {
  const float p = k0.x * rc;
  const float n = rintf(p * kInvTwoPi);
  const float ph = fmaf(-n, kTwoPiLo, fmaf(-n, kTwoPiHi, p));
  float sn, cs;
  __sincosf(ph, &sn, &cs);
  const float m = amp * __expf(-a0 * rc);
  return make_float2(m * cs, m * sn);
}

// Generation mapping shared by the geometry pre-pass and the sweep: thread tid owns scatterer
// s_g of a 64-scatterer tile and elements [16 eg, 16 eg + 16).  The eight lanes of a
// quarter-warp share eg and take eight consecutive scatterers, so their 16-byte stores into
// the core-matrix operand layouts fill one contiguous 128-byte row of banks.
__device__ __forceinline__ int tc_sg(int tid) { return (tid >> 5) * 8 + (tid & 7); }
__device__ __forceinline__ int tc_eg(int tid) { return (tid >> 3) & 3; }

// SMEM layout (bytes).
constexpr uint32_t kOffAtxHi = 0;                 // K-major  128 x 64 bf16
constexpr uint32_t kOffAtxLo = 16384;
constexpr uint32_t kOffArxHi = 32768;             // MN-major 128 x 64 bf16
constexpr uint32_t kOffArxLo = 49152;
constexpr int kXPitch = 33;
// The rest depends on the transmit chunks nc (N = 64 nc): B_rx MN-major N (n) x 64 (k), hi
// then lo; the exchange buffer, 2 x 64 rows x 33 floats (padded: conflict-free); per band
// frequency B_tx K-major N x 64, hi then lo.
struct TcSmem {
  uint32_t brx_hi, brx_lo, x, btx, btx_bytes;
};
__host__ __device__ inline TcSmem tc_smem(int nc) {
  TcSmem L;
  L.brx_hi = 65536;
  L.brx_lo = 65536 + 8192u * nc;
  L.x = 65536 + 16384u * nc;
  L.btx = ((L.x + 2u * 64u * kXPitch * 4u + 1023u) / 1024u) * 1024u;
  L.btx_bytes = 16384u * nc;
  return L;
}
__host__ __device__ inline uint32_t tc_smem_bytes(int fb, int nc) {
  const TcSmem L = tc_smem(nc);
  return L.btx + (uint32_t)fb * L.btx_bytes + 1024;
}

// kSplitTx: the TX product is formed in passes of two chunks (three chunks, N = 192); else in
// one pass of all nc chunks.
template <int U, bool kSplitTx>
__global__ void __launch_bounds__(kThreads, 1) tc_kernel(const __grid_constant__ TcArgs A) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar_tx, mbar_rx;
  __shared__ uint32_t tmem_holder;
  __shared__ int s_item, s_fail;
  __shared__ float rcs[kTcT];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int fb = A.fb, E = A.E, T = A.n_tx;
  const int NC = A.nc, NT = kTcTxChunk * NC, N = 2 * NT;
  const int TXK = kSplitTx ? 2 : NC, TXC = 64 * TXK;  // chunks per TX pass, TX TMEM columns
  const int n_pass = kSplitTx ? (NC + 1) / 2 : 1;
  const TcSmem SL = tc_smem(NC);
  if (tid == 0) {
    tc::mbar_init(&mbar_tx, 1);
    tc::mbar_init(&mbar_rx, 1);
    tc::fence_mbar_init();
    s_fail = 0;
  }
  if (warp == 0) tc::tmem_alloc(&tmem_holder, kTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_holder;
  // mbarrier phases and the pending-RX flag are only used by thread 0
  uint32_t ph_tx = 0, ph_rx = 0;
  bool rx_pending = false;

  const uint32_t sbase = tc::smem_u32(sm);
  const uint32_t id_tx = tc::idesc_bf16(128, TXC, 0, 0);  // A K-major, B K-major (a full pass)
  const uint32_t id_rx = tc::idesc_bf16(128, N, 1, 1);  // A MN-major, B MN-major
  float* X = reinterpret_cast<float*>(sm + SL.x);

  const int s_g = tc_sg(tid), eg = tc_eg(tid);
  // TMEM read mapping: lane quarter q (rows 32q..32q+31), column half h
  const int q = warp & 3, h = warp >> 2;

  // thread 0 waits on an mbarrier (bounded); the result reaches every thread through s_fail
  // after the next __syncthreads, so all threads take the same branches.
  auto wait0 = [&](uint64_t* mb, uint32_t& ph) {
    if (tid == 0) {
      if (!tc::mbar_wait_bounded(mb, ph, kWaitTries)) s_fail = 1;
      ph ^= 1u;
    }
  };

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = s_fail ? A.n_items : atomicAdd(A.queue, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= A.n_items) break;
    int p = 0;
    while (p + 1 < A.n_phantoms && item >= A.ph[p + 1].item0) ++p;
    const BatchPhantom& P = A.ph[p];
    const int local = item - P.item0;
    const int band = local % P.n_bands, chunk = local / P.n_bands;
    const int f0 = band * fb;
    const int nf = min(fb, P.n_freq - f0);
    const int64_t s_begin = (int64_t)chunk * A.chunk;
    const int64_t s_end = min(P.n_scat, s_begin + A.chunk);
    SweepConst C = A.C;
    C.dk = P.dk;
    C.dalpha = P.dalpha;

    // ---- B_tx for the band: K-major rows n', K = e; value D_c'(e, t).  With split TX passes
    //      the rows are (chunk, c', t mod 32), so that each chunk of 32 transmits is 64
    //      contiguous rows; else (c', t). ----
    for (int i = tid; i < fb * N * 64; i += kThreads) {
      const int f = i / (N * 64), n = (i >> 6) % N, e = i & 63;
      // chunk-major rows when the TX product is formed in passes; else (c', t) order
      const int c = kSplitTx ? (n >> 5) & 1 : n / NT;
      const int t = kSplitTx ? kTcTxChunk * (n >> 6) + (n & 31) : n % NT;
      float v = 0.f;
      if (f < nf && e < E && t < T) {
        const float w = A.apod[t * E + e];
        if (w != 0.f) {
          const float2 tau = A.tau[t * E + e];
          const float2 fr = P.freq_hz[f0 + f];
          const float pr = __fmul_rn(fr.x, tau.x);
          float er = fmaf(fr.x, tau.x, -pr);
          er = fmaf(fr.x, tau.y, er);
          er = fmaf(fr.y, tau.x, er);
          const float x = __fadd_rn(__fsub_rn(pr, rintf(pr)), er);  // cycles, |x| <= 0.5
          float sn, cs;
          sincospif(2.0f * x, &sn, &cs);
          v = w * (c ? sn : cs);
        }
      }
      __nv_bfloat16 hi, lo;
      tc::split_bf16(v, hi, lo);
      unsigned char* bt = sm + SL.btx + f * SL.btx_bytes;
      const uint32_t off = tc::kmajor_off(n, e, 8);
      *reinterpret_cast<__nv_bfloat16*>(bt + off) = hi;
      *reinterpret_cast<__nv_bfloat16*>(bt + SL.btx_bytes / 2 + off) = lo;
    }
    const float2 k0 = P.kf[f0];
    const float a0 = P.af[f0];
    bool first_tile = true;

    if constexpr (!kSplitTx) {
      // Software-pipelined tile loop (one pass of the transmit product): the Green's values of
      // frequency f + 1 are formed while the receive MMAs of f run, written to the transmit A
      // operand as soon as the transmit MMAs of f are done, and to the receive A operand once
      // the receive MMAs of f are; the transmit MMAs of f + 1 queue right behind the receive
      // MMAs of f.  Order per frequency: wait TX(f) | epilogue(f) -> B_rx | issue RX(f) |
      // values(f + 1) -> A_tx | issue TX(f + 1) | wait RX(f) | values(f + 1) -> A_rx.
      for (int64_t t0 = s_begin; t0 < s_end; t0 += kTcT) {
        const int64_t s = t0 + s_g;
        const bool sval = s < s_end;
        if (eg == 0) {
          float w = 0.f;
          if (sval) {
            const double x = P.scat[2 * s], z = P.scat[2 * s + 1];
            bool out = z < 0.0;
            if (A.convex) out = out || (x * x + (z + A.apex) * (z + A.apex) <= A.radius2);
            w = out ? 0.f : (float)P.rc[s];
          }
          rcs[s_g] = w;
        }
        float2 G[16 * U], S[16 * U];
        {
          const float4* gp = A.geo + ((P.tile0 + t0 / kTcT) * (16 * U)) * kThreads + tid;
#pragma unroll
          for (int i = 0; i < 16 * U; ++i) {
            const float4 v = gp[(size_t)i * kThreads];
            G[i] = tc_anchor(v.x, v.y, k0, a0);
            S[i] = make_float2(v.z, v.w);
          }
        }
        // the BF16 hi/lo words of this thread's 16 Green's values at the current frequency
        // (both halves of 8 elements: re hi, re lo, im hi, im lo), then one recurrence step
        uint4 wv[2][4];
        auto gen_values = [&]() {
#pragma unroll
          for (int half = 0; half < 2; ++half) {
            float gr[8], gi[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const int jj = half * 8 + j;
              float2 acc = G[jj * U];
#pragma unroll
              for (int u = 1; u < U; ++u) acc = cadd(acc, G[jj * U + u]);
              gr[j] = acc.x;
              gi[j] = acc.y;
#pragma unroll
              for (int u = 0; u < U; ++u) G[jj * U + u] = cmul(G[jj * U + u], S[jj * U + u]);
            }
            tc::split8(gr, wv[half][0], wv[half][1]);
            tc::split8(gi, wv[half][2], wv[half][3]);
          }
        };
        auto store_tx = [&]() {
#pragma unroll
          for (int half = 0; half < 2; ++half) {
            const int e0 = eg * 16 + half * 8;
            const uint32_t o_re = tc::kmajor_off(s_g, e0, 8), o_im = tc::kmajor_off(64 + s_g, e0, 8);
            *reinterpret_cast<uint4*>(sm + kOffAtxHi + o_re) = wv[half][0];
            *reinterpret_cast<uint4*>(sm + kOffAtxLo + o_re) = wv[half][1];
            *reinterpret_cast<uint4*>(sm + kOffAtxHi + o_im) = wv[half][2];
            *reinterpret_cast<uint4*>(sm + kOffAtxLo + o_im) = wv[half][3];
          }
        };
        auto store_rx = [&]() {
#pragma unroll
          for (int half = 0; half < 2; ++half) {
            const int e0 = eg * 16 + half * 8;
            const uint32_t q_re = tc::mnmajor_off(e0, s_g, 16), q_im = tc::mnmajor_off(64 + e0, s_g, 16);
            *reinterpret_cast<uint4*>(sm + kOffArxHi + q_re) = wv[half][0];
            *reinterpret_cast<uint4*>(sm + kOffArxLo + q_re) = wv[half][1];
            *reinterpret_cast<uint4*>(sm + kOffArxHi + q_im) = wv[half][2];
            *reinterpret_cast<uint4*>(sm + kOffArxLo + q_im) = wv[half][3];
          }
        };
        auto issue_tx = [&](int f) {  // thread 0
          const uint32_t bt = sbase + SL.btx + f * SL.btx_bytes;
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
            const uint64_t ah = tc::sdesc(sbase + kOffAtxHi + ks * 256, 128, 1024);
            const uint64_t al = tc::sdesc(sbase + kOffAtxLo + ks * 256, 128, 1024);
            const uint64_t bh = tc::sdesc(bt + ks * 256, 128, 1024);
            const uint64_t bl = tc::sdesc(bt + SL.btx_bytes / 2 + ks * 256, 128, 1024);
            tc::mma_bf16(tmem, ah, bh, id_tx, ks > 0);
            tc::mma_bf16(tmem, ah, bl, id_tx, 1);
            tc::mma_bf16(tmem, al, bh, id_tx, 1);
          }
          tc::commit(&mbar_tx);
        };
        gen_values();
        // the previous receive MMAs read A_rx and B_rx: wait for them before the prologue writes
        if (tid == 0 && rx_pending) {
          wait0(&mbar_rx, ph_rx);
          rx_pending = false;
        }
        tc::fence_before_sync();
        __syncthreads();  // rcs visible, the previous receive product done
        tc::fence_after_sync();
        if (s_fail) break;
        store_tx();
        store_rx();
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) issue_tx(0);
        for (int f = 0; f < nf; ++f) {
          if (tid == 0) wait0(&mbar_tx, ph_tx);
          tc::fence_before_sync();
          __syncthreads();
          tc::fence_after_sync();
          if (s_fail) break;
          // ---- P = combine(D_tx); write B_rx (MN-major rows n' = (c', t), K = s), one chunk
          //      of 32 transmits at a time ----
          const int row = 32 * q + lane;  // (c, s) with c = row / 64
          for (int k = 0; k < NC; ++k) {
            float v[32];
            tc::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + h * NT + 32 * k, v);
            if (row >= 64) {
#pragma unroll
              for (int t = 0; t < 32; ++t) X[(h * 64 + (row - 64)) * kXPitch + t] = v[t];
            }
            __syncthreads();
            if (row < 64) {
              const float* x = X + ((1 - h) * 64 + row) * kXPitch;
              const float rw = rcs[row];
#pragma unroll
              for (int t = 0; t < 32; ++t) v[t] = rw * (h ? v[t] + x[t] : v[t] - x[t]);
#pragma unroll
              for (int c8 = 0; c8 < 4; ++c8) {
                uint4 hh, ll;
                tc::split8(v + 8 * c8, hh, ll);
                const uint32_t o = tc::mnmajor_off(h * NT + 32 * k + 8 * c8, row, N / 8);
                *reinterpret_cast<uint4*>(sm + SL.brx_hi + o) = hh;
                *reinterpret_cast<uint4*>(sm + SL.brx_lo + o) = ll;
              }
            }
            if (k + 1 < NC) __syncthreads();  // X is reused by the next chunk
          }
          tc::fence_proxy_async_smem();
          tc::fence_before_sync();
          __syncthreads();
          tc::fence_after_sync();
          // ---- RX MMAs into this frequency's accumulator ----
          if (tid == 0) {
            const uint32_t d = tmem + TXC + N * f;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              const uint64_t ah = tc::sdesc(sbase + kOffArxHi + ks * 2 * 2048, 2048, 128);
              const uint64_t al = tc::sdesc(sbase + kOffArxLo + ks * 2 * 2048, 2048, 128);
              const uint32_t lbo = 16u * N;  // N / 8 core matrices of 128 bytes per K group
              const uint64_t bh = tc::sdesc(sbase + SL.brx_hi + ks * 2 * lbo, lbo, 128);
              const uint64_t bl = tc::sdesc(sbase + SL.brx_lo + ks * 2 * lbo, lbo, 128);
              tc::mma_bf16(d, ah, bh, id_rx, (first_tile && ks == 0) ? 0u : 1u);
              tc::mma_bf16(d, ah, bl, id_rx, 1);
              tc::mma_bf16(d, al, bh, id_rx, 1);
            }
            tc::commit(&mbar_rx);
            rx_pending = true;
          }
          if (f + 1 < nf) {
            gen_values();
            store_tx();  // the transmit MMAs of f are done (waited above)
            tc::fence_proxy_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (tid == 0) {
              issue_tx(f + 1);
              wait0(&mbar_rx, ph_rx);
              rx_pending = false;
            }
            tc::fence_before_sync();
            __syncthreads();  // the receive MMAs of f are done: A_rx may be overwritten
            tc::fence_after_sync();
            if (s_fail) break;
            store_rx();
            tc::fence_proxy_async_smem();  // published by the barrier that opens the next frequency
          }
        }
        first_tile = false;
        if (s_fail) break;
      }
    } else {
      for (int64_t t0 = s_begin; t0 < s_end; t0 += kTcT) {
        const int64_t s = t0 + s_g;
        const bool sval = s < s_end;
        if (eg == 0) {
          float w = 0.f;
          if (sval) {
            const double x = P.scat[2 * s], z = P.scat[2 * s + 1];
            bool out = z < 0.0;
            if (A.convex) out = out || (x * x + (z + A.apex) * (z + A.apex) <= A.radius2);
            w = out ? 0.f : (float)P.rc[s];
          }
          rcs[s_g] = w;
        }
        // ---- the tile's cached geometry (16 elements x U sub-elements per thread) -> anchors ----
        float2 G[16 * U], S[16 * U];
        {
          const float4* gp = A.geo + ((P.tile0 + t0 / kTcT) * (16 * U)) * kThreads + tid;
  #pragma unroll
          for (int i = 0; i < 16 * U; ++i) {
            const float4 v = gp[(size_t)i * kThreads];
            G[i] = tc_anchor(v.x, v.y, k0, a0);
            S[i] = make_float2(v.z, v.w);
          }
        }
        __syncthreads();  // rcs visible

        for (int f = 0; f < nf; ++f) {
          // previous RX MMAs read A_rx / B_rx: wait before overwriting
          if (tid == 0 && rx_pending) {
            wait0(&mbar_rx, ph_rx);
            rx_pending = false;
          }
          tc::fence_before_sync();
          __syncthreads();
          tc::fence_after_sync();
          if (s_fail) break;
          // ---- Green's values at f; write A_tx (K-major rows (c, s), K = e) and
          //      A_rx (MN-major rows (c, e), K = s) in halves of 8 elements.  Both operands hold
          //      the same BF16 hi/lo words: eight consecutive elements of one scatterer are one
          //      16-byte core-matrix row in either layout.  The receive weights rc (real) go into
          //      B_rx and pulse x probe (one complex factor per frequency) into the reduction. ----
  #pragma unroll
          for (int half = 0; half < 2; ++half) {
            float gr[8], gi[8];
  #pragma unroll
            for (int j = 0; j < 8; ++j) {
              const int jj = half * 8 + j;
              float2 acc = G[jj * U];
  #pragma unroll
              for (int u = 1; u < U; ++u) acc = cadd(acc, G[jj * U + u]);
              gr[j] = acc.x;
              gi[j] = acc.y;
  #pragma unroll
              for (int u = 0; u < U; ++u) G[jj * U + u] = cmul(G[jj * U + u], S[jj * U + u]);
            }
            const int e0 = eg * 16 + half * 8;
            uint4 hr, lr, hi_, li_;
            tc::split8(gr, hr, lr);
            tc::split8(gi, hi_, li_);
            const uint32_t o_re = tc::kmajor_off(s_g, e0, 8), o_im = tc::kmajor_off(64 + s_g, e0, 8);
            *reinterpret_cast<uint4*>(sm + kOffAtxHi + o_re) = hr;
            *reinterpret_cast<uint4*>(sm + kOffAtxLo + o_re) = lr;
            *reinterpret_cast<uint4*>(sm + kOffAtxHi + o_im) = hi_;
            *reinterpret_cast<uint4*>(sm + kOffAtxLo + o_im) = li_;
            const uint32_t q_re = tc::mnmajor_off(e0, s_g, 16), q_im = tc::mnmajor_off(64 + e0, s_g, 16);
            *reinterpret_cast<uint4*>(sm + kOffArxHi + q_re) = hr;
            *reinterpret_cast<uint4*>(sm + kOffArxLo + q_re) = lr;
            *reinterpret_cast<uint4*>(sm + kOffArxHi + q_im) = hi_;
            *reinterpret_cast<uint4*>(sm + kOffArxLo + q_im) = li_;
          }
          tc::fence_proxy_async_smem();
          tc::fence_before_sync();
          __syncthreads();
          tc::fence_after_sync();
          if constexpr (!kSplitTx) {
            // ---- TX MMAs (one pass, N columns) ----
            if (tid == 0) {
              const uint32_t bt = sbase + SL.btx + f * SL.btx_bytes;
  #pragma unroll
              for (int ks = 0; ks < 4; ++ks) {
                const uint64_t ah = tc::sdesc(sbase + kOffAtxHi + ks * 256, 128, 1024);
                const uint64_t al = tc::sdesc(sbase + kOffAtxLo + ks * 256, 128, 1024);
                const uint64_t bh = tc::sdesc(bt + ks * 256, 128, 1024);
                const uint64_t bl = tc::sdesc(bt + SL.btx_bytes / 2 + ks * 256, 128, 1024);
                tc::mma_bf16(tmem, ah, bh, id_tx, ks > 0);
                tc::mma_bf16(tmem, ah, bl, id_tx, 1);
                tc::mma_bf16(tmem, al, bh, id_tx, 1);
              }
              tc::commit(&mbar_tx);
              wait0(&mbar_tx, ph_tx);
            }
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (s_fail) break;
            // ---- P = combine(D_tx); write B_rx (MN-major rows n' = (c', t), K = s), one chunk
            //      of 32 transmits at a time ----
            const int row = 32 * q + lane;  // (c, s) with c = row / 64
            for (int k = 0; k < NC; ++k) {
              float v[32];
              tc::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + h * NT + 32 * k, v);
              if (row >= 64) {
  #pragma unroll
                for (int t = 0; t < 32; ++t) X[(h * 64 + (row - 64)) * kXPitch + t] = v[t];
              }
              __syncthreads();
              if (row < 64) {
                // h = 0: Pr = D[0,s][0,t] - D[1,s][1,t];  h = 1: Pi = D[0,s][1,t] + D[1,s][0,t];
                // times the scatterer's reflectivity
                const float* x = X + ((1 - h) * 64 + row) * kXPitch;
                const float rw = rcs[row];
  #pragma unroll
                for (int t = 0; t < 32; ++t) v[t] = rw * (h ? v[t] + x[t] : v[t] - x[t]);
  #pragma unroll
                for (int c8 = 0; c8 < 4; ++c8) {
                  uint4 hh, ll;
                  tc::split8(v + 8 * c8, hh, ll);
                  const uint32_t o = tc::mnmajor_off(h * NT + 32 * k + 8 * c8, row, N / 8);
                  *reinterpret_cast<uint4*>(sm + SL.brx_hi + o) = hh;
                  *reinterpret_cast<uint4*>(sm + SL.brx_lo + o) = ll;
                }
              }
              if (k + 1 < NC) __syncthreads();  // X is reused by the next chunk
            }
          } else {
            // ---- TX MMAs, at most two chunks of 32 transmits per pass (columns [0, 64 chunks)),
            //      then P = combine(D_tx) -> B_rx (MN-major rows n' = (c', t), K = s) chunk by
            //      chunk ----
            const int row = 32 * q + lane;  // (c, s) with c = row / 64
            for (int pz = 0; pz < n_pass; ++pz) {
              const int k0 = pz * TXK, k1 = kSplitTx ? min(NC, k0 + 2) : NC;
              if (kSplitTx && pz > 0) {  // the previous pass's TMEM reads and exchange are done
                tc::fence_before_sync();
                __syncthreads();
                tc::fence_after_sync();
              }
              if (tid == 0) {
                const uint32_t bt = sbase + SL.btx + f * SL.btx_bytes + 8192u * k0;  // 64 rows per chunk
                const uint32_t idp = (!kSplitTx || k1 - k0 == TXK) ? id_tx : tc::idesc_bf16(128, 64 * (k1 - k0), 0, 0);
  #pragma unroll
                for (int ks = 0; ks < 4; ++ks) {
                  const uint64_t ah = tc::sdesc(sbase + kOffAtxHi + ks * 256, 128, 1024);
                  const uint64_t al = tc::sdesc(sbase + kOffAtxLo + ks * 256, 128, 1024);
                  const uint64_t bh = tc::sdesc(bt + ks * 256, 128, 1024);
                  const uint64_t bl = tc::sdesc(bt + SL.btx_bytes / 2 + ks * 256, 128, 1024);
                  tc::mma_bf16(tmem, ah, bh, idp, ks > 0);
                  tc::mma_bf16(tmem, ah, bl, idp, 1);
                  tc::mma_bf16(tmem, al, bh, idp, 1);
                }
                tc::commit(&mbar_tx);
                wait0(&mbar_tx, ph_tx);
              }
              tc::fence_before_sync();
              __syncthreads();
              tc::fence_after_sync();
              if (s_fail) break;
              for (int k = k0; k < k1; ++k) {
                float v[32];
                // split passes: chunk k occupies TX columns 64 (k - k0) + 32 c'; one pass: c' NT + 32 k
                const int col = kSplitTx ? 64 * (k - k0) + 32 * h : h * NT + 32 * k;
                tc::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + col, v);
                if (row >= 64) {
  #pragma unroll
                  for (int t = 0; t < 32; ++t) X[(h * 64 + (row - 64)) * kXPitch + t] = v[t];
                }
                __syncthreads();
                if (row < 64) {
                  // h = 0: Pr = D[0,s][0,t] - D[1,s][1,t];  h = 1: Pi = D[0,s][1,t] + D[1,s][0,t];
                  // times the scatterer's reflectivity
                  const float* x = X + ((1 - h) * 64 + row) * kXPitch;
                  const float rw = rcs[row];
  #pragma unroll
                  for (int t = 0; t < 32; ++t) v[t] = rw * (h ? v[t] + x[t] : v[t] - x[t]);
  #pragma unroll
                  for (int c8 = 0; c8 < 4; ++c8) {
                    uint4 hh, ll;
                    tc::split8(v + 8 * c8, hh, ll);
                    const uint32_t o = tc::mnmajor_off(h * NT + 32 * k + 8 * c8, row, N / 8);
                    *reinterpret_cast<uint4*>(sm + SL.brx_hi + o) = hh;
                    *reinterpret_cast<uint4*>(sm + SL.brx_lo + o) = ll;
                  }
                }
                if (k + 1 < k1) __syncthreads();  // X is reused by the next chunk
              }
            }
          }
          if (s_fail) break;
          tc::fence_proxy_async_smem();
          tc::fence_before_sync();
          __syncthreads();
          tc::fence_after_sync();
          // ---- RX MMAs into this frequency's accumulator ----
          if (tid == 0) {
            const uint32_t d = tmem + TXC + N * f;
  #pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              const uint64_t ah = tc::sdesc(sbase + kOffArxHi + ks * 2 * 2048, 2048, 128);
              const uint64_t al = tc::sdesc(sbase + kOffArxLo + ks * 2 * 2048, 2048, 128);
              const uint32_t lbo = 16u * N;  // N / 8 core matrices of 128 bytes per K group
              const uint64_t bh = tc::sdesc(sbase + SL.brx_hi + ks * 2 * lbo, lbo, 128);
              const uint64_t bl = tc::sdesc(sbase + SL.brx_lo + ks * 2 * lbo, lbo, 128);
              tc::mma_bf16(d, ah, bh, id_rx, (first_tile && ks == 0) ? 0u : 1u);
              tc::mma_bf16(d, ah, bl, id_rx, 1);
              tc::mma_bf16(d, al, bh, id_rx, 1);
            }
            tc::commit(&mbar_rx);
            rx_pending = true;
          }
        }
        first_tile = false;
        __syncthreads();
        if (s_fail) break;
      }
    }
    // ---- drain, then Y = combine(D_rx[f]) -> partial[item][f][t][e] ----
    if (tid == 0 && rx_pending) {
      wait0(&mbar_rx, ph_rx);
      rx_pending = false;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const bool fail = s_fail != 0;
    float2* out = A.partial + (size_t)item * fb * NT * kTcE;
    for (int f = 0; f < fb; ++f) {
      for (int k = 0; k < NC; ++k) {
        float v[32];
        const bool have = !first_tile && f < nf && !fail;
        if (have) tc::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + TXC + N * f + h * NT + 32 * k, v);
        const int row = 32 * q + lane;  // (c, e)
        if (row >= 64) {
#pragma unroll
          for (int t = 0; t < 32; ++t) X[(h * 64 + (row - 64)) * kXPitch + t] = have ? v[t] : 0.f;
        }
        __syncthreads();
        if (row < 64) {
          const float* x = X + ((1 - h) * 64 + row) * kXPitch;
#pragma unroll
          for (int t = 0; t < 32; ++t) {
            const float val = have ? (h ? v[t] + x[t] : v[t] - x[t]) : 0.f;
            float* o = reinterpret_cast<float*>(out + ((size_t)f * NT + 32 * k + t) * kTcE + row);
            o[h] = val;  // h = 0 real part, h = 1 imaginary part
          }
        }
        __syncthreads();
      }
    }
  }
  // ---- release TMEM ----
  tc::fence_before_sync();
  __syncthreads();
  if (s_fail && tid == 0) atomicExch(A.status, FSG_ETIMEOUT);
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// Single-tile check of the tcgen05 GEMM building block: D (128 x 64) = A (128 x 64) B^T, with
// A and B given row-major in FP32, split into BF16 hi/lo and laid out K-major or MN-major.
__global__ void __launch_bounds__(128, 1) tc_selftest_kernel(const float* Ag, const float* Bg, float* Dg, int a_mn,
                                                              int b_mn, int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_holder;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    tc::mbar_init(&mbar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(&tmem_holder, 64);
  // A: 32 KB region (hi at 0, lo at 16384); B: hi at 32768, lo at 40960
  for (int k = 0; k < 64; ++k) {
    __nv_bfloat16 hi, lo;
    tc::split_bf16(Ag[tid * 64 + k], hi, lo);
    const uint32_t o = a_mn ? tc::mnmajor_off(tid, k, 16) : tc::kmajor_off(tid, k, 8);
    *reinterpret_cast<__nv_bfloat16*>(sm + o) = hi;
    *reinterpret_cast<__nv_bfloat16*>(sm + 16384 + o) = lo;
    if (tid < 64) {
      tc::split_bf16(Bg[tid * 64 + k], hi, lo);
      const uint32_t ob = b_mn ? tc::mnmajor_off(tid, k, 8) : tc::kmajor_off(tid, k, 8);
      *reinterpret_cast<__nv_bfloat16*>(sm + 32768 + ob) = hi;
      *reinterpret_cast<__nv_bfloat16*>(sm + 40960 + ob) = lo;
    }
  }
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_holder;
  const uint32_t sb = tc::smem_u32(sm);
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, 64, a_mn, b_mn);
    for (int ks = 0; ks < 4; ++ks) {
      uint64_t ah, al, bh, bl;
      if (a_mn) {
        ah = tc::sdesc(sb + ks * 2 * 2048, 2048, 128);
        al = tc::sdesc(sb + 16384 + ks * 2 * 2048, 2048, 128);
      } else {
        ah = tc::sdesc(sb + ks * 256, 128, 1024);
        al = tc::sdesc(sb + 16384 + ks * 256, 128, 1024);
      }
      if (b_mn) {
        bh = tc::sdesc(sb + 32768 + ks * 2 * 1024, 1024, 128);
        bl = tc::sdesc(sb + 40960 + ks * 2 * 1024, 1024, 128);
      } else {
        bh = tc::sdesc(sb + 32768 + ks * 256, 128, 1024);
        bl = tc::sdesc(sb + 40960 + ks * 256, 128, 1024);
      }
      tc::mma_bf16(tmem, ah, bh, idesc, ks > 0);
      tc::mma_bf16(tmem, ah, bl, idesc, 1);
      tc::mma_bf16(tmem, al, bh, idesc, 1);
    }
    tc::commit(&mbar);
  }
  const bool ok = tc::mbar_wait_bounded(&mbar, 0, kWaitTries);
  tc::fence_after_sync();
  float v[32];
  if (ok) {
    tc::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16), v);
    for (int j = 0; j < 32; ++j) Dg[(32 * warp + lane) * 64 + j] = v[j];
    tc::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + 32, v);
    for (int j = 0; j < 32; ++j) Dg[(32 * warp + lane) * 64 + 32 + j] = v[j];
  } else if (tid == 0) {
    atomicExch(status, FSG_ETIMEOUT);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

// Geometry of every (scatterer, source) of every phantom, once per sweep: one CTA per
// (tile, phantom); thread tid writes its 16 U states (clipped r, amplitude, step) at
// geo[((tile0 + tile) 16U + i) 256 + tid], so that the sweep's loads are coalesced.  Sources
// of padded elements and scatterers past the end get zeros (no contribution).
template <int U>
__global__ void __launch_bounds__(kThreads) tc_geometry_kernel(const __grid_constant__ TcArgs A) {
  const BatchPhantom& P = A.ph[blockIdx.y];
  const int tid = threadIdx.x, s_g = tc_sg(tid), eg = tc_eg(tid);
  const int64_t n_tiles = (P.n_scat + kTcT - 1) / kTcT;
  SweepConst C = A.C;
  C.dk = P.dk;
  C.dalpha = P.dalpha;
  for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const int64_t s = t * kTcT + s_g;
    const bool sval = s < P.n_scat;
    const int64_t si = sval ? s : t * kTcT;
    const float xs = (float)P.scat[2 * si], zs = (float)P.scat[2 * si + 1];
    float4* gp = const_cast<float4*>(A.geo) + ((P.tile0 + t) * (16 * U)) * kThreads + tid;
#pragma unroll 4
    for (int i = 0; i < 16 * U; ++i) {
      const int e = eg * 16 + i / U, u = i % U;
      const int ec = e < A.E ? e : A.E - 1;
      const float4 v = tc_geometry(xs, zs, A.src_pos[ec * U + u], A.rot_e[ec], C);
      gp[(size_t)i * kThreads] = (sval && e < A.E) ? v : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

cudaError_t launch_tc_geometry(int U, int max_tiles, int sms, const TcArgs& A, cudaStream_t s) {
  const int gx = max_tiles < 4 * sms ? max_tiles : 4 * sms;
  const dim3 grid(gx > 0 ? gx : 1, A.n_phantoms);
  if (U == 1) tc_geometry_kernel<1><<<grid, kThreads, 0, s>>>(A);
  else tc_geometry_kernel<2><<<grid, kThreads, 0, s>>>(A);
  return cudaGetLastError();
}

template <int U, bool kSplitTx>
static cudaError_t launch_tc_t(int grid, const TcArgs& A, cudaStream_t s) {
  const uint32_t smem = tc_smem_bytes(A.fb, A.nc);
  cudaError_t e = cudaFuncSetAttribute(tc_kernel<U, kSplitTx>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  tc_kernel<U, kSplitTx><<<grid, kThreads, smem, s>>>(A);
  return cudaGetLastError();
}

cudaError_t launch_tc(int U, int grid, const TcArgs& A, cudaStream_t s) {
  const bool split = tc_tx_chunks(A.nc) < A.nc;
  if (U == 1) return split ? launch_tc_t<1, true>(grid, A, s) : launch_tc_t<1, false>(grid, A, s);
  return split ? launch_tc_t<2, true>(grid, A, s) : launch_tc_t<2, false>(grid, A, s);
}

}  // namespace fsg

// ------------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------------

namespace {

using namespace fsg;

size_t tc_a256(size_t v) { return (v + 255) & ~size_t(255); }

struct TcLayout {
  int fb, nc, chunk, n_items, max_tiles;
  int n_bands[kMaxPhantoms], n_chunks[kMaxPhantoms], item0[kMaxPhantoms];
  int64_t tile0[kMaxPhantoms];
  size_t off_src, off_rot, off_tau, off_apod, off_queue, off_tab[kMaxPhantoms], off_partial, off_geo, total;
};

void tc_layout(const FsgProbe* probe, const FsgPhantom* ph, int n_ph, int n_tx, const FsgBatchTuning* tu,
               TcLayout* L) {
  L->nc = (n_tx + kTcTxChunk - 1) / kTcTxChunk;
  int fb = (tu && tu->freqs_per_item > 0) ? tu->freqs_per_item : kTcMaxFb;
  if (fb > tc_max_fb(L->nc)) fb = tc_max_fb(L->nc);
  L->fb = fb;
  // the items of one chunk run side by side, so a chunk's geometry (16 KB per scatterer at
  // U = 2) should stay resident in L2: 16,384 scatterers by default
  int64_t chunk = (tu && tu->chunk_scatterers > 0) ? tu->chunk_scatterers : 16384;
  chunk = ((chunk + kTcT - 1) / kTcT) * kTcT;
  L->chunk = (int)chunk;
  const int E = probe->n_elements, U = probe->n_sub;
  size_t o = 0;
  L->off_src = o; o += tc_a256((size_t)E * U * 16);
  L->off_rot = o; o += tc_a256((size_t)E * 8);
  L->off_tau = o; o += tc_a256((size_t)n_tx * E * 8);
  L->off_apod = o; o += tc_a256((size_t)n_tx * E * 4);
  L->off_queue = o; o += 256;  // queue counter + status word
  int items = 0;
  int64_t tiles = 0;
  L->max_tiles = 0;
  for (int p = 0; p < n_ph; ++p) {
    const int F = ph[p].plan.n_freq;
    L->n_bands[p] = (F + fb - 1) / fb;
    L->n_chunks[p] = ph[p].n_scat > 0 ? (int)((ph[p].n_scat + chunk - 1) / chunk) : 1;
    L->item0[p] = items;
    items += L->n_bands[p] * L->n_chunks[p];
    L->off_tab[p] = o;
    o += tc_a256((size_t)F * (8 + 4 + 8 + 8 + 4));
    L->tile0[p] = tiles;
    const int64_t t = (ph[p].n_scat + kTcT - 1) / kTcT;
    tiles += t;
    if (t > L->max_tiles) L->max_tiles = (int)t;
  }
  L->n_items = items;
  L->off_partial = o;
  o += tc_a256((size_t)items * fb * kTcTxChunk * L->nc * kTcE * 8);
  L->off_geo = o;
  o += tc_a256((size_t)tiles * 16 * U * kThreads * 16);
  L->total = o;
}

}  // namespace

extern "C" size_t fsg_simus_batched_tc_workspace_size(const FsgProbe* probe, const FsgPhantom* phantoms,
                                                      int32_t n_phantoms, int32_t n_tx,
                                                      const FsgBatchTuning* tuning) {
  if (!probe || !phantoms || n_phantoms < 1 || n_phantoms > kMaxPhantoms || n_tx < 1) return 0;
  TcLayout L;
  tc_layout(probe, phantoms, n_phantoms, n_tx, tuning, &L);
  return L.total;
}

extern "C" int32_t fsg_simus_batched_tc(const FsgProbe* probe, const FsgMedium* medium, const FsgPhantom* phantoms,
                                        int32_t n_phantoms, const double* delays, const double* apod, int32_t n_tx,
                                        const FsgBatchTuning* tuning, void* workspace, size_t workspace_bytes,
                                        void* stream_ptr) {
  if (!probe || !medium || !phantoms || !delays) return set_error(FSG_EINVAL, "NULL argument");
  if (n_phantoms < 1 || n_phantoms > kMaxPhantoms) return set_error(FSG_EINVAL, "n_phantoms must be in [1, %d]", kMaxPhantoms);
  if (n_tx < 1 || n_tx > kTcMaxTx)
    return set_error(FSG_EUNSUPPORTED, "tensor-core sweep supports n_tx <= %d", kTcMaxTx);
  if (probe->n_elements < 1 || probe->n_elements > kTcE)
    return set_error(FSG_EUNSUPPORTED, "tensor-core sweep supports n_elements <= %d", kTcE);
  if (probe->n_sub < 1 || probe->n_sub > 2) return set_error(FSG_EUNSUPPORTED, "tensor-core sweep supports n_sub <= 2");
  if (!(medium->speed_of_sound > 0) || !(medium->attenuation >= 0)) return set_error(FSG_EINVAL, "bad medium");
  for (int p = 0; p < n_phantoms; ++p) {
    const FsgFreqPlan& pl = phantoms[p].plan;
    if (phantoms[p].n_scat < 0 || (phantoms[p].n_scat > 0 && (!phantoms[p].scat_xz || !phantoms[p].rc)) ||
        !phantoms[p].out)
      return set_error(FSG_EINVAL, "phantom %d: bad inputs", p);
    if (pl.n_freq < 1 || !pl.pulse_spectrum || !pl.probe_spectrum || pl.freq_idx_start < 0 ||
        pl.freq_idx_start + pl.n_freq > pl.n_freq_full)
      return set_error(FSG_EINVAL, "phantom %d: bad plan", p);
  }
  TcLayout L;
  tc_layout(probe, phantoms, n_phantoms, n_tx, tuning, &L);
  if (!workspace || workspace_bytes < L.total)
    return set_error(FSG_EWORKSPACE, "workspace of %zu bytes is smaller than the %zu bytes required", workspace_bytes,
                     L.total);
  int sms = 0, dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (ce != cudaSuccess) return check_cuda(ce, "device query");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream_ptr);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  const int E = probe->n_elements, U = probe->n_sub;
  int st;
  {
    SetupArgs a;
    memset(&a, 0, sizeof(a));
    a.E = E;
    a.U = U;
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
    b.tile0 = L.tile0[p];
    b.f0 = q.plan.freq_start;
    b.df = q.plan.freq_step;
    b.corr = (float)q.plan.correction_factor;
    const SweepConst cp = make_sweep_const(probe, medium, &q.plan, 0);
    b.dk = cp.dk;
    b.dalpha = cp.dalpha;
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
    const int n = max_f > n_tx * E ? max_f : n_tx * E;
    batched_setup<<<dim3((n + 127) / 128, n_phantoms), 128, 0, s>>>(a);
    if ((st = check_cuda(cudaGetLastError(), "batched_setup launch")) != FSG_OK) return st;
  }
  int* queue = reinterpret_cast<int*>(ws + L.off_queue);
  if ((st = check_cuda(cudaMemsetAsync(queue, 0, 2 * sizeof(int), s), "queue reset")) != FSG_OK) return st;
  float2* partial = reinterpret_cast<float2*>(ws + L.off_partial);
  {
    TcArgs A;
    memcpy(A.ph, bp, sizeof(bp));
    A.n_phantoms = n_phantoms;
    A.n_items = L.n_items;
    A.E = E;
    A.U = U;
    A.n_tx = n_tx;
    A.fb = L.fb;
    A.nc = L.nc;
    A.chunk = L.chunk;
    A.src_pos = reinterpret_cast<const float4*>(ws + L.off_src);
    A.rot_e = reinterpret_cast<const float2*>(ws + L.off_rot);
    A.tau = tau;
    A.apod = apw;
    A.C = make_sweep_const(probe, medium, &phantoms[0].plan, 0);
    convex_geometry(probe, &A.convex, &A.apex, &A.radius2);
    A.queue = queue;
    A.status = queue + 1;
    A.partial = partial;
    A.geo = reinterpret_cast<const float4*>(ws + L.off_geo);
    if ((st = check_cuda(launch_tc_geometry(U, L.max_tiles, sms, A, s), "tc_geometry_kernel launch")) != FSG_OK)
      return st;
    int grid = sms;
    if (grid > L.n_items) grid = L.n_items;
    if ((st = check_cuda(launch_tc(U, grid, A, s), "tc_kernel launch")) != FSG_OK) return st;
  }
  {
    BatchReduceArgs a;
    memcpy(a.ph, bp, sizeof(bp));
    a.n_phantoms = n_phantoms;
    a.n_tx = n_tx;
    a.E = E;
    a.fb = L.fb;
    a.tx_pad = kTcTxChunk * L.nc;
    a.e_pad = kTcE;
    a.apply_pp = 1;  // the tensor-core partials carry rc but not pulse x probe
    a.partial = partial;
    batched_reduce<<<dim3(2 * sms, n_phantoms), 256, 0, s>>>(a);
    if ((st = check_cuda(cudaGetLastError(), "batched_reduce launch")) != FSG_OK) return st;
  }
  return FSG_OK;
}

extern "C" int32_t fsg_simus_batched_tc_status(const void* workspace, const FsgProbe* probe,
                                               const FsgPhantom* phantoms, int32_t n_phantoms, int32_t n_tx,
                                               const FsgBatchTuning* tuning, int32_t* status_out, void* stream) {
  if (!workspace || !probe || !phantoms || !status_out) return set_error(FSG_EINVAL, "NULL argument");
  TcLayout L;
  tc_layout(probe, phantoms, n_phantoms, n_tx, tuning, &L);
  const int* dev_status = reinterpret_cast<const int*>(static_cast<const unsigned char*>(workspace) + L.off_queue) + 1;
  cudaError_t e = cudaMemcpyAsync(status_out, dev_status, sizeof(int), cudaMemcpyDeviceToHost,
                                  reinterpret_cast<cudaStream_t>(stream));
  if (e == cudaSuccess) e = cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream));
  return check_cuda(e, "status read");
}

extern "C" int32_t fsg_tc_selftest(const float* a, const float* b, float* d, int32_t a_mn_major, int32_t b_mn_major,
                                   int32_t* status, void* stream) {
  if (!a || !b || !d || !status) return set_error(FSG_EINVAL, "NULL argument");
  const int smem = 96 * 1024;
  cudaError_t e = cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(tc_selftest_kernel)");
  tc_selftest_kernel<<<1, 128, smem, reinterpret_cast<cudaStream_t>(stream)>>>(a, b, d, a_mn_major, b_mn_major, status);
  return check_cuda(cudaGetLastError(), "tc_selftest launch");
}

// The plain simus sweep with one Green's-function recurrence per (scatterer, element,
// frequency): simus_stash_kernel.  Instantiated by fsg_sweep_stash.cu (without full-frequency
// directivity) and fsg_sweep_stash_ffd.cu (with it), compiled in parallel.
//
// Work split, geometry cache and slots are those of simus_band_kernel: one CTA of 256 threads
// per SM sweeps its share of a chunk's (band, tile) units; each tile's geometry block comes in
// by TMA from the L2-resident cache.  What differs is the receive side.  simus_band_kernel
// re-generates every Green's term for the receive contraction; here the transmit lanes write
// each term once into a shared-memory stash, per sub-block of kStashFreqs frequencies, and the
// receive contraction reads it back:
//
//   anchors    lane (point s, g) owns elements e = g + GN k and all their sub-elements; exact
//              double-float anchor at the band's first frequency times exp(i 2 pi f tau_e),
//              and the recurrence step times exp(i 2 pi df tau_e)
//   transmit   per frequency f of the sub-block: m(s, e, f) = sum_u G(s, e, u, f) e^{i 2 pi f tau_e}
//              -> stash[s][f][e];  P(s, f) = sum_e apod_e m(s, e, f) (reduce-scatter over the
//              GN lanes) -> W[s][f] = rc_s pulse_f probe_f P(s, f)
//   receive    thread (e, frequencies): Y'(e, f) += sum_s stash[s][f][e] W[s][f]
//
// The receive sums carry the transmit delay phase exp(i 2 pi f tau_e) of every term;
// simus_reduce multiplies it out, once per (f, e).  The stash overlays the tile's geometry
// block, which the anchors have consumed by then.  FP32-pipe work per (scatterer, element,
// frequency) at two sub-elements: 8 (two recurrences) + 2 (sub-element sum) + 2 (transmit
// sum) + 4 (receive MAC), against 26 in simus_band_kernel.
#pragma once

#include "fsg_sweep_kernels.cuh"

namespace fsg {

// Source slots per element of a lane: 1, 2, 4 (U = 3 and 4) or 8 (U = 5 to 8, the kernels
// instantiated with U = 8 and the runtime count).
__host__ __device__ constexpr int stash_spe(int U) { return U == 1 ? 1 : (U == 2 ? 2 : (U <= 4 ? 4 : 8)); }

// Receive over one stash sub-block: Ys[sb FS + j][e] += sum_s stash[s][j][e] W[s][j] for the
// NJ frequencies j of each item (e, j0).  A warp takes consecutive elements: the stash reads
// are contiguous and the W reads are broadcasts.
template <int ST, int NJ>
__device__ __forceinline__ void stash_receive(const float2* __restrict__ stash, const float2* __restrict__ W,
                                              float2* __restrict__ Ys, int E, int ep, int sb) {
  constexpr int FS = kStashFreqs;
  const int items = E * (FS / NJ);
  for (int it = threadIdx.x; it < items; it += kThreads) {
    const int e = it % E, j0 = (it / E) * NJ;
    float2 acc[NJ];
#pragma unroll
    for (int j = 0; j < NJ; ++j) acc[j] = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int s = 0; s < ST; ++s) {
      float2 wv[NJ];
      if constexpr (NJ >= 2) {
#pragma unroll
        for (int q = 0; q < NJ / 2; ++q) {
          const float4 w4 = reinterpret_cast<const float4*>(W + s * FS + j0)[q];
          wv[2 * q] = make_float2(w4.x, w4.y);
          wv[2 * q + 1] = make_float2(w4.z, w4.w);
        }
      } else {
        wv[0] = W[s * FS + j0];
      }
#pragma unroll
      for (int j = 0; j < NJ; ++j) acc[j] = cfma(stash[(s * FS + j0 + j) * ep + e], wv[j], acc[j]);
    }
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      float2* y = Ys + (size_t)(sb * FS + j0 + j) * E + e;
      *y = cadd(*y, acc[j]);
    }
  }
}

// Transmit half of one stash sub-block for one lane (point sl, lane g of GN): FS recurrence
// steps of the lane's 16 source slots (packed in 8 FP32x2 pairs), with every element's
// sub-element sum m(s, e, f) written to stash_row[f ep + e] (stash_row = the point's row block)
// and accumulated, times the element's transmit apodization, into the point's source sum.
// The sums are then reduced over the GN lanes: halving exchanges while a lane holds more than
// one frequency, all-reduce over the lanes left sharing one.  On return v[r] (r < R) holds
// the full sum of sub-block frequency R (g / SH) + r, SH = max(1, GN / FS) lanes holding each.
// GUARD: the lanes' element slots may run past E (no stash write for those).
template <int U, int GN, bool FFD, bool GUARD>
__device__ __forceinline__ void stash_transmit(float2 (&Gr)[kSrcPerThread / 2], float2 (&Gi)[kSrcPerThread / 2],
                                               const float2 (&Sr)[kSrcPerThread / 2],
                                               const float2 (&Si)[kSrcPerThread / 2],
                                               const float2 (&Sn)[kSrcPerThread / 2],
                                               const float2 (&Dh)[FFD ? kSrcPerThread / 2 : 1],
                                               const float (&wk)[kSrcPerThread / stash_spe(U)],
                                               float2* __restrict__ stash_row, int ep, int g, int E,
                                               const float* __restrict__ kb_sb, float2 (&v)[kStashFreqs]) {
  constexpr int SPE = stash_spe(U);
  constexpr int EPL = kSrcPerThread / SPE;
  constexpr int kPairs = kSrcPerThread / 2;
  constexpr int FS = kStashFreqs;
  constexpr int SH = GN >= FS ? GN / FS : 1;
#pragma unroll
  for (int j = 0; j < FS; ++j) {
    float2 kk = make_float2(0.f, 0.f);
    if constexpr (FFD) {
      const float k = kb_sb[j];
      kk = make_float2(k, k);
    }
    v[j] = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < EPL; ++k) {
      float2 m;
      if constexpr (U == 1) {
        const int p = k >> 1;
        if constexpr (FFD) {
          const float2 d = sinc_poly2(__fmul2_rn(Dh[p], kk));
          m = (k & 1) ? make_float2(Gr[p].y * d.y, Gi[p].y * d.y) : make_float2(Gr[p].x * d.x, Gi[p].x * d.x);
        } else {
          m = (k & 1) ? make_float2(Gr[p].y, Gi[p].y) : make_float2(Gr[p].x, Gi[p].x);
        }
      } else if constexpr (U == 2) {
        if constexpr (FFD) {
          const float2 d = sinc_poly2(__fmul2_rn(Dh[k], kk));
          const float2 tr = __fmul2_rn(Gr[k], d), ti = __fmul2_rn(Gi[k], d);
          m = make_float2(tr.x + tr.y, ti.x + ti.y);
        } else {
          m = make_float2(Gr[k].x + Gr[k].y, Gi[k].x + Gi[k].y);
        }
      } else {
        // SPE / 2 pairs per element (the slots past the element's sub-elements hold zeros)
        constexpr int PPE = SPE / 2;
        float2 tr, ti;
        if constexpr (FFD) {
          const float2 d0 = sinc_poly2(__fmul2_rn(Dh[PPE * k], kk));
          tr = __fmul2_rn(Gr[PPE * k], d0);
          ti = __fmul2_rn(Gi[PPE * k], d0);
#pragma unroll
          for (int q = 1; q < PPE; ++q) {
            const float2 d = sinc_poly2(__fmul2_rn(Dh[PPE * k + q], kk));
            tr = __ffma2_rn(Gr[PPE * k + q], d, tr);
            ti = __ffma2_rn(Gi[PPE * k + q], d, ti);
          }
        } else {
          tr = Gr[PPE * k];
          ti = Gi[PPE * k];
#pragma unroll
          for (int q = 1; q < PPE; ++q) {
            tr = __fadd2_rn(tr, Gr[PPE * k + q]);
            ti = __fadd2_rn(ti, Gi[PPE * k + q]);
          }
        }
        m = make_float2(tr.x + tr.y, ti.x + ti.y);
      }
      const int e = g + GN * k;
      if (!GUARD || e < E) stash_row[j * ep + e] = m;
      v[j] = __ffma2_rn(m, make_float2(wk[k], wk[k]), v[j]);
    }
#pragma unroll
    for (int p = 0; p < kPairs; ++p) cstep2(Gr[p], Gi[p], Sr[p], Si[p], Sn[p]);
  }
#pragma unroll
  for (int h = GN / 2; h >= SH; h >>= 1) {
    const int half = FS * h / GN;
    const bool up = (g & h) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float2 send = up ? v[i] : v[i + half];
      const float2 keep = up ? v[i + half] : v[i];
      v[i].x = keep.x + __shfl_xor_sync(0xffffffffu, send.x, h);
      v[i].y = keep.y + __shfl_xor_sync(0xffffffffu, send.y, h);
    }
  }
#pragma unroll
  for (int h = SH / 2; h >= 1; h >>= 1) {
    v[0].x += __shfl_xor_sync(0xffffffffu, v[0].x, h);
    v[0].y += __shfl_xor_sync(0xffffffffu, v[0].y, h);
  }
}

template <int U, int GN, bool FFD>
__global__ void __launch_bounds__(kThreads, 1) simus_stash_kernel(const BandArgs A) {
  constexpr int SPE = stash_spe(U);  // source slots per element (U = 3 pads one, U = 5..7 pad to 8)
  constexpr int EPL = kSrcPerThread / SPE;             // element slots per lane
  constexpr int kPairs = kSrcPerThread / 2;
  constexpr int FS = kStashFreqs;
  constexpr int R = GN >= FS ? 1 : FS / GN;  // frequencies a lane holds after the reduce-scatter
  constexpr int ST = kThreads / GN;          // tile points
  extern __shared__ __align__(16) unsigned char sm[];
  const StashLayout L = stash_layout(ST, A.fb, A.E, A.U, A.plane_pad, FFD);
  __shared__ uint64_t s_mbar;
  __shared__ int s_fail;
  const int tid = threadIdx.x;
  if (tid == 0) {
    tc::mbar_init(&s_mbar, 1);
    tc::fence_mbar_init();
    s_fail = 0;
  }
  const int g = tid % GN;
  const int sl = tid / GN;
  const int E = A.E, fb = A.fb, ep = L.ep;

  const float* b_rhi = reinterpret_cast<const float*>(sm + L.g.off_rhi);
  const float* b_rlo = reinterpret_cast<const float*>(sm + L.g.off_rlo);
  const float* b_amp = reinterpret_cast<const float*>(sm + L.g.off_amp);
  const float2* b_st = reinterpret_cast<const float2*>(sm + L.g.off_step);
  const float* b_dir = reinterpret_cast<const float*>(sm + L.g.off_dir);
  float2* stash = reinterpret_cast<float2*>(sm);  // region 0, once the anchors are taken
  float2* W = reinterpret_cast<float2*>(sm + L.off_w);
  float2* pp = reinterpret_cast<float2*>(sm + L.off_pp);
  float* kb = reinterpret_cast<float*>(sm + L.off_kb);
  float2* dph = reinterpret_cast<float2*>(sm + L.off_dph);
  float2* dstep = reinterpret_cast<float2*>(sm + L.off_dstep);
  float2* Ys = reinterpret_cast<float2*>(sm + L.off_y);  // running receive sums [f][e] of the band

  float wk[EPL];  // transmit apodization of my elements
#pragma unroll
  for (int k = 0; k < EPL; ++k) {
    const int e = g + GN * k;
    wk[k] = e < E ? A.t.wtx[e] : 0.f;
  }
  for (int i = tid; i < E; i += kThreads) dstep[i] = A.t.dstep[i];

  const int64_t units = (int64_t)A.n_bands * A.chunk_tiles;
  const int64_t u_end = (int64_t)(blockIdx.x + 1) * units / A.grid;
  const int64_t s_stop = min(A.n_pts, A.chunk_s0 + A.chunk_tiles * ST);
  uint32_t phase = 0;
  for (int64_t u = (int64_t)blockIdx.x * units / A.grid; u < u_end;) {
    const int band = (int)(u / A.chunk_tiles);
    const int64_t t_lo = u - (int64_t)band * A.chunk_tiles;
    const int64_t t_hi = min(A.chunk_tiles, t_lo + (u_end - u));
    u += t_hi - t_lo;
    const int slot = (int)blockIdx.x - cta_of_unit((int64_t)band * A.chunk_tiles, units, A.grid);
    const int f_b0 = band * fb;
    // band tables (their previous readers finished at the barrier that closed the last tile)
    for (int i = tid; i < fb; i += kThreads) {
      const int f = f_b0 + i;
      pp[i] = (f < A.F) ? A.t.pp[f] : make_float2(0.f, 0.f);
      if (FFD) kb[i] = A.t.kf[min(f, A.F - 1)].x;
    }
    for (int i = tid; i < E; i += kThreads) dph[i] = A.t.dph[(f_b0 / kAnchor) * E + i];
    for (int i = tid; i < fb * E; i += kThreads) Ys[i] = make_float2(0.f, 0.f);
    __syncthreads();
    const float2 k0 = A.t.kf[f_b0];
    const float a0 = A.t.af[f_b0];

    for (int64_t tile = t_lo; tile < t_hi; ++tile) {
      const int64_t t0 = A.chunk_s0 + tile * ST;
      // ---------------- geometry: TMA bulk copy of the tile's block into region 0 ----------------
      // The previous tile's stash reads finished at the barrier that closed it; the proxy fence
      // orders them before the asynchronous writes.
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
      float w = 0.f;  // rc of my point (0 when out of field or padding)
      {
        const int64_t s = t0 + sl;
        if (s < s_stop) {
          const double x = A.pts[2 * s], z = A.pts[2 * s + 1];
          bool out = z < 0.0;
          if (A.convex) out = out || (x * x + (z + A.apex) * (z + A.apex) <= A.radius2);
          w = out ? 0.f : (float)A.rc[s];
        }
      }
      // ---------------- anchors: slots 2p, 2p + 1 share one packed FP32x2 lane pair ----------------
      float2 Gr[kPairs], Gi[kPairs], Sr[kPairs], Si[kPairs], Sn[kPairs];
      float2 Dh[FFD ? kPairs : 1];
#pragma unroll
      for (int p = 0; p < kPairs; ++p) {
        float2 gv[2], sv[2];
        float dv[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int slot = 2 * p + h, k = slot / SPE, uu = slot % SPE;
          const int e = g + GN * k;
          gv[h] = make_float2(0.f, 0.f);
          sv[h] = make_float2(0.f, 0.f);
          dv[h] = 0.f;
          if (uu < (U == 8 ? A.U : U) && e < E) {
            const int idx = uu * L.g.plane + e * L.g.pitch + sl;
            gv[h] = cmul(anchor_value(b_rhi[idx], b_rlo[idx], b_amp[idx], k0, a0), dph[e]);
            sv[h] = cmul(b_st[idx], dstep[e]);
            if (FFD) dv[h] = b_dir[idx];
          }
        }
        Gr[p] = make_float2(gv[0].x, gv[1].x);
        Gi[p] = make_float2(gv[0].y, gv[1].y);
        Sr[p] = make_float2(sv[0].x, sv[1].x);
        Si[p] = make_float2(sv[0].y, sv[1].y);
        Sn[p] = make_float2(-sv[0].y, -sv[1].y);
        if constexpr (FFD) Dh[p] = make_float2(dv[0], dv[1]);
      }
      __syncthreads();  // every geometry read is done: region 0 becomes the stash

#pragma unroll 1
      for (int sb = 0; sb < fb / FS; ++sb) {
        // ---------------- transmit: FS recurrence steps, stash writes, source sums ----------------
        float2 v[FS];
        stash_transmit<U, GN, FFD, true>(Gr, Gi, Sr, Si, Sn, Dh, wk, stash + sl * FS * ep, ep, g, E,
                                         FFD ? kb + sb * FS : nullptr, v);
        if (g % (GN >= FS ? GN / FS : 1) == 0) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const int fj = R * (g / (GN >= FS ? GN / FS : 1)) + r;
            const float2 pv = cmul(pp[sb * FS + fj], v[r]);
            W[sl * FS + fj] = make_float2(w * pv.x, w * pv.y);
          }
        }
        __syncthreads();
        // ---------------- receive from the stash ----------------
        if (E >= 128) {
          stash_receive<ST, 4>(stash, W, Ys, E, ep, sb);
        } else if (E >= 64) {
          stash_receive<ST, 2>(stash, W, Ys, E, ep, sb);
        } else {
          stash_receive<ST, 1>(stash, W, Ys, E, ep, sb);
        }
        __syncthreads();
      }
    }
    if (s_fail) break;
    if (slot >= A.n_slots) {  // cannot happen for the host's slot count; fail loudly if it does
      if (tid == 0) atomicExch(A.status, FSG_EINVAL);
      break;
    }
    float2* out = reinterpret_cast<float2*>(A.partial) + (size_t)slot * A.F * E;
    for (int i = tid; i < fb * E; i += kThreads) {
      const int f = f_b0 + i / E;
      if (f < A.F) {
        float2* o = out + (size_t)f * E + (i % E);
        *o = cadd(*o, Ys[i]);
      }
    }
  }
  if (tid == 0 && s_fail) atomicExch(A.status, FSG_ETIMEOUT);
}

// ---------------------------------------------------------------------------------------------
// simus_ws_kernel: the same sweep with the two halves on separate warps, for probes of EC = 64,
// 128 or 256 elements.  Warps 0-3 (transmit) run the recurrences of STX = 128 / GN points and
// fill stash buffer b while warps 4-7 (receive) contract buffer 1 - b, so the FP32 work of the
// transmit side runs under the shared-memory traffic of the receive side.  The hand-over is
// two pairs of named barriers (full[b]: transmit arrives, receive waits; empty[b]: receive
// arrives, transmit waits), and both sides walk the same sequence of sub-blocks, n = 0, 1, ...,
// N - 1 with buffer b = n mod 2; transmit waits on empty[b] from n = 2 on and receive releases
// it up to n = N - 3, so every barrier phase has its 256 threads.  No thread leaves the
// sequence early: a geometry copy that timed out is recorded in the status word, the
// remaining copies are skipped and the output of the call becomes NaN (simus_reduce).
// The receive sums of a band stay in the receive threads' registers (thread = element, and a
// share of each sub-block's frequencies for EC < 128, or two elements for EC = 256) and go to
// the band's slot when its run of tiles ends.  The geometry block of the next tile is copied
// in (TMA) as soon as the transmit warps have taken the current tile's anchors.
template <int EC, int U>
struct WsShape {
  static constexpr int SPE = (U == 1) ? 1 : (U == 2 ? 2 : 4);
  static constexpr int GN0 = EC * SPE / kSrcPerThread;
  static constexpr int GN = GN0 < 4 ? 4 : GN0;          // lanes per point
  static constexpr int STX = 128 / GN;                   // points per tile
  static constexpr int FB = EC > 128 ? 32 : 64;          // band
  static constexpr int EPT = EC > 128 ? EC / 128 : 1;    // receive elements per thread
  static constexpr int NJ = EC >= 128 ? kStashFreqs : kStashFreqs * EC / 128;  // receive frequencies per sub-block
};

constexpr uint32_t kBarFull = 1;   // + b
constexpr uint32_t kBarEmpty = 3;  // + b
constexpr uint32_t kBarTx = 5;

template <int EC, int U, bool FFD>
__global__ void __launch_bounds__(kThreads, 1) simus_ws_kernel(const BandArgs A) {
  using SH_ = WsShape<EC, U>;
  constexpr int SPE = SH_::SPE, GN = SH_::GN, STX = SH_::STX, FB = SH_::FB, EPT = SH_::EPT, NJ = SH_::NJ;
  constexpr int EPL = kSrcPerThread / SPE;
  constexpr int kPairs = kSrcPerThread / 2;
  constexpr int FS = kStashFreqs;
  constexpr int NSB = FB / FS;
  constexpr int R = GN >= FS ? 1 : FS / GN;
  constexpr int SHL = GN >= FS ? GN / FS : 1;
  static_assert(GN <= 32 && GN * EPL == EC, "every element slot of every lane is a real element");
  static_assert(NSB % 2 == 0, "buffer parity of a sub-block is fixed within a tile");
  extern __shared__ __align__(16) unsigned char sm[];
  const WsLayout L = ws_layout(STX, FB, EC, A.U, A.plane_pad, FFD);
  constexpr int EP = EC | 1;
  constexpr size_t kStashWords = (size_t)STX * FS * EP;  // float2 per buffer
  __shared__ uint64_t s_mbar;
  __shared__ int s_fail;
  const int tid = threadIdx.x;
  if (tid == 0) {
    tc::mbar_init(&s_mbar, 1);
    tc::fence_mbar_init();
    s_fail = 0;
  }
  float2* stash = reinterpret_cast<float2*>(sm + L.off_stash);
  float2* Wb = reinterpret_cast<float2*>(sm + L.off_w);
  float2* pp = reinterpret_cast<float2*>(sm + L.off_pp);
  float* kb = reinterpret_cast<float*>(sm + L.off_kb);
  float2* dph = reinterpret_cast<float2*>(sm + L.off_dph);
  float2* dstep = reinterpret_cast<float2*>(sm + L.off_dstep);
  for (int i = tid; i < EC; i += kThreads) dstep[i] = A.t.dstep[i];
  __syncthreads();

  const int64_t units = (int64_t)A.n_bands * A.chunk_tiles;
  const int64_t u_begin = (int64_t)blockIdx.x * units / A.grid;
  const int64_t u_end = (int64_t)(blockIdx.x + 1) * units / A.grid;
  const int64_t n_total = (u_end - u_begin) * NSB;
  const int64_t s_stop = min(A.n_pts, A.chunk_s0 + A.chunk_tiles * STX);

  if (tid < 128) {
    // =============================== transmit warps ===============================
    const int g = tid % GN, sl = tid / GN;
    const float* b_rhi = reinterpret_cast<const float*>(sm + L.g.off_rhi);
    const float* b_rlo = reinterpret_cast<const float*>(sm + L.g.off_rlo);
    const float* b_amp = reinterpret_cast<const float*>(sm + L.g.off_amp);
    const float2* b_st = reinterpret_cast<const float2*>(sm + L.g.off_step);
    const float* b_dir = reinterpret_cast<const float*>(sm + L.g.off_dir);
    float wk[EPL];
#pragma unroll
    for (int k = 0; k < EPL; ++k) wk[k] = A.t.wtx[g + GN * k];
    // geometry copies: thread 0 issues the copy of a unit's tile block and waits for it; one is
    // in flight at a time (inflight), phases alternate
    uint32_t phase = 0;
    bool inflight = false;
    auto issue = [&](int64_t unit) {
      const unsigned char* src = A.geo + (unit % A.chunk_tiles) * A.geo_bytes;
      tc::fence_proxy_async_smem();
      tc::mbar_arrive_expect_tx(&s_mbar, (uint32_t)A.geo_bytes);
      for (size_t off = 0; off < A.geo_bytes; off += kBulkPiece)
        tc::bulk_g2s(sm + off, src + off, (uint32_t)min(kBulkPiece, A.geo_bytes - off), &s_mbar);
      inflight = true;
    };
    if (tid == 0 && u_begin < u_end) issue(u_begin);
    int64_t n = 0;
    for (int64_t u = u_begin; u < u_end;) {
      const int band = (int)(u / A.chunk_tiles);
      const int64_t t_lo = u - (int64_t)band * A.chunk_tiles;
      const int64_t t_hi = min(A.chunk_tiles, t_lo + (u_end - u));
      const int f_b0 = band * FB;
      tc::bar_sync(kBarTx, 128);  // the previous band's table readers are done
      for (int i = tid; i < FB; i += 128) {
        const int f = f_b0 + i;
        pp[i] = (f < A.F) ? A.t.pp[f] : make_float2(0.f, 0.f);
        if (FFD) kb[i] = A.t.kf[min(f, A.F - 1)].x;
      }
      for (int i = tid; i < EC; i += 128) dph[i] = A.t.dph[(f_b0 / kAnchor) * EC + i];
      const float2 k0 = A.t.kf[f_b0];
      const float a0 = A.t.af[f_b0];
      for (int64_t tile = t_lo; tile < t_hi; ++tile, ++u) {
        if (tid == 0 && inflight && !s_fail) {
          if (tc::mbar_wait_bounded(&s_mbar, phase, kBulkWaitTries)) {
            inflight = false;
            phase ^= 1u;
          } else {
            s_fail = 1;
          }
        }
        tc::bar_sync(kBarTx, 128);  // the block (and the band tables) are visible
        float w = 0.f;
        {
          const int64_t s = A.chunk_s0 + tile * STX + sl;
          if (s < s_stop) {
            const double x = A.pts[2 * s], z = A.pts[2 * s + 1];
            bool out = z < 0.0;
            if (A.convex) out = out || (x * x + (z + A.apex) * (z + A.apex) <= A.radius2);
            w = out ? 0.f : (float)A.rc[s];
          }
        }
        float2 Gr[kPairs], Gi[kPairs], Sr[kPairs], Si[kPairs], Sn[kPairs];
        float2 Dh[FFD ? kPairs : 1];
#pragma unroll
        for (int p = 0; p < kPairs; ++p) {
          float2 gv[2], sv[2];
          float dv[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int slot = 2 * p + h, k = slot / SPE, uu = slot % SPE;
            const int e = g + GN * k;
            gv[h] = make_float2(0.f, 0.f);
            sv[h] = make_float2(0.f, 0.f);
            dv[h] = 0.f;
            if (uu < U) {
              const int idx = uu * L.g.plane + e * L.g.pitch + sl;
              gv[h] = cmul(anchor_value(b_rhi[idx], b_rlo[idx], b_amp[idx], k0, a0), dph[e]);
              sv[h] = cmul(b_st[idx], dstep[e]);
              if (FFD) dv[h] = b_dir[idx];
            }
          }
          Gr[p] = make_float2(gv[0].x, gv[1].x);
          Gi[p] = make_float2(gv[0].y, gv[1].y);
          Sr[p] = make_float2(sv[0].x, sv[1].x);
          Si[p] = make_float2(sv[0].y, sv[1].y);
          Sn[p] = make_float2(-sv[0].y, -sv[1].y);
          if constexpr (FFD) Dh[p] = make_float2(dv[0], dv[1]);
        }
        tc::bar_sync(kBarTx, 128);  // the block is consumed: copy the next tile's in
        if (tid == 0 && !s_fail && u + 1 < u_end) issue(u + 1);
#pragma unroll 1
        for (int sb = 0; sb < NSB; ++sb, ++n) {
          const int b = sb & 1;
          if (n >= 2) tc::bar_sync(kBarEmpty + b, 256);
          float2 v[FS];
          stash_transmit<U, GN, FFD, false>(Gr, Gi, Sr, Si, Sn, Dh, wk, stash + b * kStashWords + sl * FS * EP, EP,
                                            g, EC, FFD ? kb + sb * FS : nullptr, v);
          if (g % SHL == 0) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
              const int fj = R * (g / SHL) + r;
              const float2 pv = cmul(pp[sb * FS + fj], v[r]);
              Wb[(b * STX + sl) * FS + fj] = make_float2(w * pv.x, w * pv.y);
            }
          }
          tc::bar_arrive(kBarFull + b, 256);
        }
      }
    }
    if (tid == 0) {
      // a copy that gave up: wait (bounded) until it lands before the CTA's memory goes away
      if (inflight) tc::mbar_wait_bounded(&s_mbar, phase, kBulkWaitTries);
      if (s_fail) atomicExch(A.status, FSG_ETIMEOUT);
    }
  } else {
    // =============================== receive warps ===============================
    const int r = tid - 128;
    const int e0 = (EC >= 128) ? r : r % EC;
    const int j0 = (EC >= 128) ? 0 : (r / EC) * NJ;
    int64_t n = 0;
    for (int64_t u = u_begin; u < u_end;) {
      const int band = (int)(u / A.chunk_tiles);
      const int64_t t_lo = u - (int64_t)band * A.chunk_tiles;
      const int64_t t_hi = min(A.chunk_tiles, t_lo + (u_end - u));
      const int slot = (int)blockIdx.x - cta_of_unit((int64_t)band * A.chunk_tiles, units, A.grid);
      u += t_hi - t_lo;
      float2 Y[NSB][EPT][NJ];
#pragma unroll
      for (int sb = 0; sb < NSB; ++sb)
#pragma unroll
        for (int i = 0; i < EPT; ++i)
#pragma unroll
          for (int j = 0; j < NJ; ++j) Y[sb][i][j] = make_float2(0.f, 0.f);
      for (int64_t tile = t_lo; tile < t_hi; ++tile) {
#pragma unroll
        for (int sb = 0; sb < NSB; ++sb) {
          const int b = sb & 1;
          tc::bar_sync(kBarFull + b, 256);
          const float2* st_b = stash + b * kStashWords;
          const float2* w_b = Wb + b * STX * FS;
#pragma unroll 2
          for (int s = 0; s < STX; ++s) {
            float2 wv[NJ];
#pragma unroll
            for (int q = 0; q < NJ / 2; ++q) {
              const float4 w4 = reinterpret_cast<const float4*>(w_b + s * FS + j0)[q];
              wv[2 * q] = make_float2(w4.x, w4.y);
              wv[2 * q + 1] = make_float2(w4.z, w4.w);
            }
#pragma unroll
            for (int i = 0; i < EPT; ++i)
#pragma unroll
              for (int j = 0; j < NJ; ++j)
                Y[sb][i][j] = cfma(st_b[(s * FS + j0 + j) * EP + e0 + 128 * i], wv[j], Y[sb][i][j]);
          }
          if (n + sb + 2 < n_total) tc::bar_arrive(kBarEmpty + b, 256);
        }
        n += NSB;
      }
      // the band's receive sums into its slot (the host sizes the slots; a bad slot is recorded)
      if (slot < A.n_slots) {
        float2* out = reinterpret_cast<float2*>(A.partial) + (size_t)slot * A.F * EC;
#pragma unroll
        for (int sb = 0; sb < NSB; ++sb)
#pragma unroll
          for (int i = 0; i < EPT; ++i)
#pragma unroll
            for (int j = 0; j < NJ; ++j) {
              const int f = band * FB + sb * FS + j0 + j;
              if (f < A.F) {
                float2* o = out + (size_t)f * EC + e0 + 128 * i;
                *o = cadd(*o, Y[sb][i][j]);
              }
            }
      } else if (r == 0) {
        atomicExch(A.status, FSG_EINVAL);
      }
    }
  }
}

template <int U, int GN, bool FFD>
static cudaError_t launch_simus_stash(const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  cudaError_t e =
      cudaFuncSetAttribute(simus_stash_kernel<U, GN, FFD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  if (e != cudaSuccess) return e;
  simus_stash_kernel<U, GN, FFD><<<A.grid, kThreads, c.smem, s>>>(A);
  return cudaGetLastError();
}

template <int U, bool FFD>
static cudaError_t launch_simus_stash_gn(const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  switch (c.gn) {
    case 4: return launch_simus_stash<U, 4, FFD>(c, A, s);
    case 8: return launch_simus_stash<U, 8, FFD>(c, A, s);
    case 16: return launch_simus_stash<U, 16, FFD>(c, A, s);
    case 32: return launch_simus_stash<U, 32, FFD>(c, A, s);
    default: return cudaErrorInvalidValue;
  }
}

template <bool FFD>
static cudaError_t launch_simus_stash_u(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  switch (U) {
    case 1: return launch_simus_stash_gn<1, FFD>(c, A, s);
    case 2: return launch_simus_stash_gn<2, FFD>(c, A, s);
    case 3: return launch_simus_stash_gn<3, FFD>(c, A, s);
    case 4: return launch_simus_stash_gn<4, FFD>(c, A, s);
    case 5:
    case 6:
    case 7:
    case 8: return launch_simus_stash_gn<8, FFD>(c, A, s);  // the runtime count pads to 8 slots
    default: return cudaErrorInvalidValue;
  }
}

template <int EC, int U, bool FFD>
static cudaError_t launch_simus_ws(const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  cudaError_t e =
      cudaFuncSetAttribute(simus_ws_kernel<EC, U, FFD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  if (e != cudaSuccess) return e;
  simus_ws_kernel<EC, U, FFD><<<A.grid, kThreads, c.smem, s>>>(A);
  return cudaGetLastError();
}

// Warp-specialised sweep for E = 64, 128 (U = 1..4) and 256 (U = 1, 2).
template <bool FFD>
static cudaError_t launch_simus_ws_any(int U, const SweepConfig& c, const BandArgs& A, cudaStream_t s) {
  switch (A.E * 8 + U) {
    case 64 * 8 + 1: return launch_simus_ws<64, 1, FFD>(c, A, s);
    case 64 * 8 + 2: return launch_simus_ws<64, 2, FFD>(c, A, s);
    case 64 * 8 + 3: return launch_simus_ws<64, 3, FFD>(c, A, s);
    case 64 * 8 + 4: return launch_simus_ws<64, 4, FFD>(c, A, s);
    case 128 * 8 + 1: return launch_simus_ws<128, 1, FFD>(c, A, s);
    case 128 * 8 + 2: return launch_simus_ws<128, 2, FFD>(c, A, s);
    case 128 * 8 + 3: return launch_simus_ws<128, 3, FFD>(c, A, s);
    case 128 * 8 + 4: return launch_simus_ws<128, 4, FFD>(c, A, s);
    case 256 * 8 + 1: return launch_simus_ws<256, 1, FFD>(c, A, s);
    case 256 * 8 + 2: return launch_simus_ws<256, 2, FFD>(c, A, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace fsg

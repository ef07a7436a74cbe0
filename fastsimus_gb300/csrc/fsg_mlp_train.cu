// Tensor-core training of the transmit-field surrogate network (tcgen05, BF16 operands, FP32
// accumulation in TMEM): one optimiser step is three launches, with no host synchronisation.
//
// Network: 64 random Fourier features [sin(2 pi B u), cos(2 pi B u)] of the normalised inputs
// u = (x, z, f, theta), four hidden layers of 256 with SiLU, a linear head of n_out = 2 n_c
// outputs: the complex amplitudes a_j of n_c <= 5 analytic carriers c_j (the plane wave of the
// firing, the two edge waves of the aperture and the two grating lobes), so that the field is
//     p(u) = sum_j (o_{2j} + i o_{2j+1}) c_j(u).
// Loss: mean over the batch of |p - y|^2 (y: the exact field, scaled).
//
//   mlp_train_fb_kernel    per tile of 128 sampled rows (one CTA per SM, persistent): gather
//                          the rows (a counter-based hash of (seed, step, row) picks them, so a
//                          step needs no host input), Fourier features, the forward pass
//                          (D = A_hi W^T + A_lo W^T per layer: hi + lo BF16 activations keep
//                          FP32-class precision), the head and loss on the CUDA cores, then the
//                          backward pass dA_l = dZ_l W_l on the tensor cores (BF16 dZ).  The
//                          weights stream through two 32 KB shared-memory buffers by TMA bulk
//                          copies.  Activations A_l, gradients dZ_l and SiLU derivatives go to
//                          a global stash in the layouts that the next kernels read.
//   mlp_train_dw_kernel    weight gradients dW_l = dZ_l^T A_l (M = 256 outputs in two halves,
//                          N = inputs, K = the batch rows split over CTAs), bias gradients from
//                          an all-ones operand column, and the head's dW_h^T = A_4^T dOut; both
//                          operands MN-major, streamed by bulk copies through four stages.
//   mlp_train_adam_kernel  sums the split partials in a fixed order, applies Adam with the
//                          step's warm-up/cosine learning rate (read from the device step
//                          counter), writes the FP32 master weights and both packed BF16 copies
//                          (K-major for the forward pass, MN-major for the backward pass), and
//                          records the step's loss; the last block advances the counter.
// Every mbarrier wait is bounded: on timeout the CTA records FSG_ETIMEOUT in the status word,
// frees its TMEM and returns.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/fsgb300.h"
#include "fsg_internal.h"
#include "fsg_tc.cuh"

namespace fsg {
namespace mlpt {

constexpr int kRows = 128;                            // rows per tile (MMA M)
constexpr int kW = 256;                               // hidden width
constexpr int kFeat = 128;                            // 2 x 64 Fourier features
constexpr int kMaxOut = 10;                           // head outputs (2 per carrier, <= 5 carriers)
constexpr int kAux = 12;                              // per row: carriers c_0..c_4, target y (complex)
constexpr int kHO = 16;                               // head width padded for the weight-gradient MMA
constexpr int kPart = kHO + 1;                        // per-tile partials: head-bias gradients, loss
// Packed weights (global): chunks of 64 inputs (forward, K-major) or 64 outputs (backward,
// MN-major), 32 KB each, core matrices k-group-major so that each half chunk of 32 K columns is
// a contiguous 16 KB piece.  The kernels stream 16 KB pieces through kBufs buffers.
constexpr int kChunkK = 64;                           // K columns per packed chunk
constexpr uint32_t kChunkBytes = kW * kChunkK * 2;    // 32 KB
constexpr int kPieceK = 64;                           // K columns per streamed piece (32 or 64)
constexpr uint32_t kPieceBytes = kW * kPieceK * 2;    // 16 KB
constexpr int kBufs = kPieceK == 32 ? 5 : 2;          // streamed pieces in shared memory
constexpr uint32_t kABytes = kRows * kW * 2;          // one BF16 copy of a 128 x 256 operand
constexpr uint32_t kOffAHi = 0, kOffALo = kABytes, kOffB = 2 * kABytes;
constexpr uint32_t kFbSmem = kOffB + kBufs * kPieceBytes;
// The head's packed weights: W_h hi and lo (K-major, 16 rows x 256, row-group-major cores; the
// forward MMA N = 16), one 16 KB piece, then W_h as the MN-major B operand of dA_4 = dOut W_h
// (K = 16), an 8 KB piece.
constexpr uint32_t kHeadHi = 0, kHeadLo = 8192, kHeadBwd = 16384, kHeadBytes = 24576;
// Pieces of one tile: forward (layer 0: P0, layers 1..3: P1 each), the head's two, backward
// (P1 per layer).
constexpr int kP0 = kFeat / kPieceK, kP1 = kW / kPieceK;
constexpr int kHeadPiece = kP0 + 3 * kP1;
constexpr int kPiecesPerTile = kHeadPiece + 2 + 3 * kP1;
constexpr uint32_t kWaitTries = 1u << 26;

// Byte offset of (row n, input k) inside a 64-input packed chunk, k-group-major: core
// (k / 8, n / 8) at ((k / 8) * 32 + n / 8) * 128.  MMA descriptor: LBO (K) 4096, SBO (N) 128.
__host__ __device__ inline uint32_t wpack_off(int n, int k) {
  return ((uint32_t)(((k >> 3) << 5) + (n >> 3)) << 7) + ((uint32_t)(n & 7) << 4) + ((uint32_t)(k & 7) << 1);
}

// Global stash, per 64-row chunk q of the batch.  "A-role" tensors feed the weight-gradient
// MMA as its A operand (M = feature): two 16 KB halves of 128 features, each MN-major core
// matrices [row / 8][feature / 8].  "B-role" tensors feed it as B (N = feature): MN-major core
// matrices [row / 8][feature / 8] over the whole width.
__host__ __device__ inline uint32_t arole_off(int r, int m) {
  return (uint32_t)(m >> 7) * 16384u + ((uint32_t)((((r >> 3) << 4) + ((m & 127) >> 3)) << 7)) +
         ((uint32_t)(r & 7) << 4) + ((uint32_t)(m & 7) << 1);
}
__host__ __device__ inline uint32_t brole_off(int r, int n, int wd) {
  return ((uint32_t)(((r >> 3) * (wd >> 3)) + (n >> 3)) << 7) + ((uint32_t)(r & 7) << 4) + ((uint32_t)(n & 7) << 1);
}

struct Stash {
  unsigned char* act[5];   // [0]: features, B-role width 128; [1..3]: B-role 256; [4]: A-role 256
  unsigned char* dz[4];    // A-role 256
  unsigned char* dout;     // B-role 16
  unsigned char* gate[3];  // SiLU'(z_l), per tile [8 column blocks][128 rows][32] BF16
};

__host__ __device__ inline size_t act_chunk_bytes(int l) { return l == 0 ? 64 * 128 * 2 : 64 * 256 * 2; }
constexpr size_t kDzChunk = 64 * 256 * 2;
constexpr size_t kDoutChunk = 64 * kHO * 2;
constexpr size_t kGateTile = 128 * 256 * 2;

struct Net {
  const float* bmat;       // [64][4]
  const void* wf[4];       // forward-packed BF16 (K-major chunks of 64 inputs)
  const void* wb[4];       // backward-packed BF16 (MN-major chunks of 64 outputs), [1..3]
  const float* bias[4];
  const void* whead;       // packed head weights (kHeadBytes)
  const float* bhead;      // [n_out]
  int n_out;
};

struct FbArgs {
  const float* u;          // [n_data][4]
  const float* aux;        // [n_data][kAux]: carriers c_0..c_4 (complex), target y (complex)
  int64_t n_data;
  uint64_t seed;
  const int* step;
  Net net;
  float inv_batch;
  Stash st;
  float* tile_part;        // [n_tiles][kPart]
  int n_tiles;
  int* rows_out;           // optional [n_tiles * 128]: the sampled data rows
  int* status;
};

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ float sigmoid_f(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }

// 8 floats -> 8 BF16 in one 16-byte vector (element 0 at the lowest address).
__device__ __forceinline__ uint4 pack8(const float* x) {
  uint32_t h[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const __nv_bfloat162 b = __floats2bfloat162_rn(x[2 * i], x[2 * i + 1]);
    h[i] = *reinterpret_cast<const uint32_t*>(&b);
  }
  return make_uint4(h[0], h[1], h[2], h[3]);
}

__device__ __forceinline__ void unpack8(uint4 v, float* x) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[i]));
    x[2 * i] = f.x;
    x[2 * i + 1] = f.y;
  }
}

// Row R of tile t lies in 64-row chunk (t * 128 + R) / 64 at row R % 64.
__device__ __forceinline__ unsigned char* chunk_ptr(unsigned char* base, size_t chunk_bytes, int tile, int R) {
  return base + (size_t)(tile * 2 + (R >> 6)) * chunk_bytes;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(256, 1) mlp_train_fb_kernel(const __grid_constant__ FbArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar_full[kBufs], mbar_free[kBufs], mbar_mma;
  __shared__ uint32_t tmem_holder;
  __shared__ int s_fail;
  __shared__ int s_step;
  __shared__ float s_bmat[256];
  __shared__ float s_bias[4][kW];
  __shared__ float s_bh[kMaxOut];
  __shared__ float4 s_u[kRows];
  __shared__ float s_aux[kRows][kAux];
  __shared__ float s_red[4][kPart];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nout = a.net.n_out;
  for (int i = tid; i < 256; i += blockDim.x) s_bmat[i] = a.net.bmat[i];
  for (int i = tid; i < 4 * kW; i += blockDim.x) s_bias[i / kW][i % kW] = a.net.bias[i / kW][i % kW];
  if (tid < kMaxOut) s_bh[tid] = tid < nout ? a.net.bhead[tid] : 0.f;
  if (tid == 0) {
    for (int b = 0; b < kBufs; ++b) {
      tc::mbar_init(&mbar_full[b], 1);
      tc::mbar_init(&mbar_free[b], 1);
    }
    tc::mbar_init(&mbar_mma, 1);
    tc::fence_mbar_init();
    s_fail = 0;
    s_step = *a.step;
  }
  // TMEM: columns [0, 256) the layer accumulator; [256, 272) the head's outputs, then
  // [256, 512) dA_4 = dOut W_h
  if (warp == 0) tc::tmem_alloc(&tmem_holder, 2 * kW);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_holder;
  const uint32_t sbase = tc::smem_u32(sm);
  const uint32_t id_fwd = tc::idesc_bf16(kRows, kW, 0, 0);  // A K-major, B K-major
  const uint32_t id_bwd = tc::idesc_bf16(kRows, kW, 0, 1);  // A K-major, B MN-major
  const uint32_t id_head = tc::idesc_bf16(kRows, kHO, 0, 0); // head: N = 16
  const uint64_t step_key = (uint64_t)(uint32_t)s_step << 32;

  // Weight pieces as one sequence over all tiles: piece g of a tile is j = g % kPiecesPerTile,
  // held in buffer g % kBufs; up to kBufs pieces are in flight.
  uint32_t ph_full[kBufs] = {}, ph_free[kBufs] = {}, ph_mma = 0u;
  int64_t next_load = 0, consumed = 0;  // pieces copied / pieces whose copy was waited for
  const int64_t my_tiles = (a.n_tiles - (int64_t)blockIdx.x + gridDim.x - 1) / gridDim.x;
  const int64_t total_pieces = my_tiles * kPiecesPerTile;
  // Copies piece g into buffer g % kBufs.  The buffer's previous piece (g - kBufs) must be
  // released by its MMAs: with `block` the call waits for that (bounded); without, it returns
  // false at once (nothing issued) if the release has not happened yet.
  auto load = [&](int64_t g, bool block, bool& failed) -> bool {
    const int b = (int)(g % kBufs);
    if (g >= kBufs) {
      if (block) {
        if (!tc::mbar_wait_bounded(&mbar_free[b], ph_free[b], kWaitTries)) {
          failed = true;
          return false;
        }
      } else if (!tc::mbar_test(&mbar_free[b], ph_free[b])) {
        return false;
      }
      ph_free[b] ^= 1u;
    }
    const int j = (int)(g % kPiecesPerTile);
    const unsigned char* src;
    uint32_t bytes = kPieceBytes;
    if (j < kP0) {
      src = static_cast<const unsigned char*>(a.net.wf[0]) + (size_t)j * kPieceBytes;
    } else if (j < kHeadPiece) {
      src = static_cast<const unsigned char*>(a.net.wf[1 + (j - kP0) / kP1]) + (size_t)((j - kP0) % kP1) * kPieceBytes;
    } else if (j == kHeadPiece) {
      src = static_cast<const unsigned char*>(a.net.whead) + kHeadHi;  // hi and lo, 16 KB
    } else if (j == kHeadPiece + 1) {
      src = static_cast<const unsigned char*>(a.net.whead) + kHeadBwd;
      bytes = kHeadBytes - kHeadBwd;
    } else {
      const int q = j - kHeadPiece - 2;
      src = static_cast<const unsigned char*>(a.net.wb[3 - q / kP1]) + (size_t)(q % kP1) * kPieceBytes;
    }
    tc::mbar_arrive_expect_tx(&mbar_full[b], bytes);
    tc::bulk_g2s(sm + kOffB + b * kPieceBytes, src, bytes, &mbar_full[b]);
    return true;
  };
  // Wait for piece g (loading ahead up to kBufs pieces); returns its buffer's shared address.
  // Look-ahead copies never wait for the MMAs of the pieces just issued (that would drain the
  // tensor pipe between pieces): only the piece needed now may block.
  auto acquire = [&](int64_t g, uint32_t& addr) -> bool {
    bool failed = false;
    while (next_load < g + kBufs && next_load < total_pieces) {
      if (!load(next_load, next_load <= g, failed)) {
        if (failed) return false;
        break;
      }
      ++next_load;
    }
    const int b = (int)(g % kBufs);
    if (!tc::mbar_wait_bounded(&mbar_full[b], ph_full[b], kWaitTries)) return false;
    ph_full[b] ^= 1u;
    ++consumed;
    tc::fence_after_sync();
    addr = sbase + kOffB + b * kPieceBytes;
    return true;
  };
  auto finish = [&]() -> bool {  // wait for all issued MMAs
    tc::commit(&mbar_mma);
    if (!tc::mbar_wait_bounded(&mbar_mma, ph_mma, kWaitTries)) return false;
    ph_mma ^= 1u;
    return true;
  };
  // One GEMM of the tile on the tensor cores (thread 0): np pieces of 2 K-steps of 16.
  // Forward: D = A_hi W^T + A_lo W^T; backward: D = dZ W (dZ in the A_hi region).
  auto gemm = [&](int64_t piece0, int np, bool bwd) -> bool {
    for (int c = 0; c < np; ++c) {
      const int64_t g = piece0 + c;
      uint32_t bb;
      if (!acquire(g, bb)) return false;
#pragma unroll
      for (int ks = 0; ks < kPieceK / 16; ++ks) {
        const int kk = c * (kPieceK / 16) + ks;
        const uint64_t ah = tc::sdesc(sbase + kOffAHi + kk * 256, 128, 32 * 128);
        const uint64_t bd = tc::sdesc(bb + ks * 2 * 4096, 4096, 128);  // both packings: K stride 4096, N stride 128
        if (!bwd) {
          const uint64_t al = tc::sdesc(sbase + kOffALo + kk * 256, 128, 32 * 128);
          tc::mma_bf16(tmem, ah, bd, id_fwd, kk > 0);
          tc::mma_bf16(tmem, al, bd, id_fwd, 1);
        } else {
          tc::mma_bf16(tmem, ah, bd, id_bwd, kk > 0);
        }
      }
      tc::commit(&mbar_free[(int)(g % kBufs)]);
    }
    if (!finish()) return false;
    // every buffer is free now: start the next pieces so they land during the epilogue
    bool failed = false;
    while (next_load < piece0 + np + kBufs && next_load < total_pieces) {
      if (!load(next_load, true, failed)) return false;
      ++next_load;
    }
    return true;
  };
  // The head's forward MMA (thread 0): O = A_4 W_h^T in TMEM columns [256, 272), three products
  // A_hi W_hi + A_lo W_hi + A_hi W_lo over K = 256.
  auto head_fwd = [&](int64_t g) -> bool {
    uint32_t hb;
    if (!acquire(g, hb)) return false;
#pragma unroll
    for (int kk = 0; kk < kW / 16; ++kk) {
      const uint64_t ah = tc::sdesc(sbase + kOffAHi + kk * 256, 128, 32 * 128);
      const uint64_t al = tc::sdesc(sbase + kOffALo + kk * 256, 128, 32 * 128);
      const uint64_t bh = tc::sdesc(hb + kHeadHi + kk * 256, 128, 32 * 128);
      const uint64_t bl = tc::sdesc(hb + kHeadLo + kk * 256, 128, 32 * 128);
      tc::mma_bf16(tmem + kW, ah, bh, id_head, kk > 0);
      tc::mma_bf16(tmem + kW, al, bh, id_head, 1);
      tc::mma_bf16(tmem + kW, ah, bl, id_head, 1);
    }
    tc::commit(&mbar_free[(int)(g % kBufs)]);
    return finish();
  };
  // dA_4 = dOut W_h (K = 16; dOut as BF16 in the A_lo region, K-major [128][16]) into TMEM
  // columns [256, 512).
  auto head_bwd = [&](int64_t g) -> bool {
    uint32_t hb;
    if (!acquire(g, hb)) return false;
    const uint64_t ad = tc::sdesc(sbase + kOffALo, 128, 2 * 128);
    const uint64_t bd = tc::sdesc(hb, 32 * 128, 128);
    tc::mma_bf16(tmem + kW, ad, bd, id_bwd, 0u);
    tc::commit(&mbar_free[(int)(g % kBufs)]);
    return finish();
  };
  auto sync_all = [&]() {
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  };

  const int row = 32 * (warp & 3) + lane, chalf = warp >> 2;
  const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
  int64_t tile_iter = 0;
  for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x, ++tile_iter) {
    const int64_t chunk_base = tile_iter * kPiecesPerTile;
    // ---- gather the tile's rows ----
    if (tid < kRows) {
      const uint64_t h = mix64(a.seed ^ (step_key + (uint64_t)tile * kRows + tid));
      const int64_t idx = (int64_t)(h % (uint64_t)a.n_data);
      if (a.rows_out) a.rows_out[tile * kRows + tid] = (int)idx;
      s_u[tid] = reinterpret_cast<const float4*>(a.u)[idx];
      const float4* ax = reinterpret_cast<const float4*>(a.aux + idx * kAux);
#pragma unroll
      for (int i = 0; i < kAux / 4; ++i) {
        const float4 x = ax[i];
        s_aux[tid][4 * i] = x.x;
        s_aux[tid][4 * i + 1] = x.y;
        s_aux[tid][4 * i + 2] = x.z;
        s_aux[tid][4 * i + 3] = x.w;
      }
    }
    __syncthreads();
    // ---- Fourier features -> A (hi + lo, K-major) and the stash (B-role, width 128) ----
    {
      const int r = tid & (kRows - 1), half = tid >> 7;
      const float4 uv = s_u[r];
      unsigned char* g0 = chunk_ptr(a.st.act[0], act_chunk_bytes(0), tile, r);
#pragma unroll
      for (int blk = 0; blk < 4; ++blk) {
        float sv[8], cv[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int j = 32 * half + 8 * blk + i;
          const float t = s_bmat[4 * j] * uv.x + s_bmat[4 * j + 1] * uv.y + s_bmat[4 * j + 2] * uv.z +
                          s_bmat[4 * j + 3] * uv.w;
          sincospif(2.0f * t, &sv[i], &cv[i]);
        }
        const int k0 = 32 * half + 8 * blk;
        uint4 hi, lo;
        tc::split8(sv, hi, lo);
        *reinterpret_cast<uint4*>(sm + kOffAHi + tc::kmajor_off(r, k0, 32)) = hi;
        *reinterpret_cast<uint4*>(sm + kOffALo + tc::kmajor_off(r, k0, 32)) = lo;
        *reinterpret_cast<uint4*>(g0 + brole_off(r & 63, k0, kFeat)) = hi;
        tc::split8(cv, hi, lo);
        *reinterpret_cast<uint4*>(sm + kOffAHi + tc::kmajor_off(r, 64 + k0, 32)) = hi;
        *reinterpret_cast<uint4*>(sm + kOffALo + tc::kmajor_off(r, 64 + k0, 32)) = lo;
        *reinterpret_cast<uint4*>(g0 + brole_off(r & 63, 64 + k0, kFeat)) = hi;
      }
    }
    tc::fence_proxy_async_smem();
    sync_all();

    // ---- forward ----
    int64_t ch = chunk_base;
    for (int l = 0; l < 4; ++l) {
      const int np = l == 0 ? kP0 : kP1;
      if (tid == 0 && !s_fail)
        if (!gemm(ch, np, false)) s_fail = 1;
      ch += np;
      sync_all();
      if (s_fail) break;
      unsigned char* gact = chunk_ptr(a.st.act[l + 1], act_chunk_bytes(l + 1), tile, row);
      unsigned char* ggate = l < 3 ? a.st.gate[l] + (size_t)tile * kGateTile : nullptr;
#pragma unroll 1
      for (int cb = 0; cb < 4; ++cb) {
        const int col0 = 128 * chalf + 32 * cb;
        float v[32], gt[32];
        tc::tmem_ld32(trow + col0, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float z = v[i] + s_bias[l][col0 + i];
          const float s = sigmoid_f(z);
          v[i] = z * s;
          gt[i] = s * fmaf(z, 1.0f - s, 1.0f);
        }
#pragma unroll
        for (int g8 = 0; g8 < 4; ++g8) {
          const int c8 = col0 + 8 * g8;
          uint4 hi, lo;
          tc::split8(v + 8 * g8, hi, lo);
          // the next MMA's A operand (the last layer's output feeds the head)
          *reinterpret_cast<uint4*>(sm + kOffAHi + tc::kmajor_off(row, c8, 32)) = hi;
          *reinterpret_cast<uint4*>(sm + kOffALo + tc::kmajor_off(row, c8, 32)) = lo;
          if (l < 3) {
            *reinterpret_cast<uint4*>(gact + brole_off(row & 63, c8, kW)) = hi;
            *reinterpret_cast<uint4*>(ggate + ((size_t)(col0 >> 5) * kRows + row) * 64 + 16 * g8) = pack8(gt + 8 * g8);
          } else {
            *reinterpret_cast<uint4*>(gact + arole_off(row & 63, c8)) = hi;
          }
        }
      }
      tc::fence_proxy_async_smem();
      sync_all();
    }
    if (s_fail) break;

    // ---- head on the tensor cores, loss and the head's output gradient ----
    if (tid == 0 && !s_fail)
      if (!head_fwd(ch)) s_fail = 1;
    ch += 1;
    sync_all();
    if (s_fail) break;
    if (chalf == 0) {
      float o[kHO], d[kMaxOut];
      tmem_ld16(trow + kW, o);
#pragma unroll
      for (int j = 0; j < kMaxOut; ++j) o[j] += s_bh[j];
      float pr = 0.f, pi = 0.f;
#pragma unroll
      for (int c = 0; c < kMaxOut / 2; ++c) {
        if (2 * c < nout) {
          const float cr = s_aux[row][2 * c], ci = s_aux[row][2 * c + 1];
          pr = fmaf(o[2 * c], cr, fmaf(-o[2 * c + 1], ci, pr));
          pi = fmaf(o[2 * c], ci, fmaf(o[2 * c + 1], cr, pi));
        }
      }
      const float er = pr - s_aux[row][kAux - 2], ei = pi - s_aux[row][kAux - 1];
      const float loss = fmaf(er, er, ei * ei);
      const float k2 = 2.0f * a.inv_batch;
#pragma unroll
      for (int c = 0; c < kMaxOut / 2; ++c) {
        const float cr = s_aux[row][2 * c], ci = s_aux[row][2 * c + 1];
        const bool on = 2 * c < nout;
        d[2 * c] = on ? k2 * fmaf(er, cr, ei * ci) : 0.f;           //  2 Re(conj(err) c) / B
        d[2 * c + 1] = on ? -k2 * fmaf(er, ci, -ei * cr) : 0.f;     // -2 Im(conj(err) c) / B
      }
      float d16[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) d16[j] = j < kMaxOut ? d[j] : 0.f;
      const uint4 p0 = pack8(d16), p1 = pack8(d16 + 8);
      unsigned char* gd = chunk_ptr(a.st.dout, kDoutChunk, tile, row);
      *reinterpret_cast<uint4*>(gd + brole_off(row & 63, 0, kHO)) = p0;
      *reinterpret_cast<uint4*>(gd + brole_off(row & 63, 8, kHO)) = p1;
      // dOut as the A operand of dA_4 = dOut W_h: K-major [128][16] in the A_lo region
      *reinterpret_cast<uint4*>(sm + kOffALo + tc::kmajor_off(row, 0, 2)) = p0;
      *reinterpret_cast<uint4*>(sm + kOffALo + tc::kmajor_off(row, 8, 2)) = p1;
      // tile partials: head-bias gradient (sum of d) and the loss, reduced over the 128 rows
      float red[kMaxOut + 1];
#pragma unroll
      for (int j = 0; j < kMaxOut; ++j) red[j] = d[j];
      red[kMaxOut] = loss;
#pragma unroll
      for (int j = 0; j <= kMaxOut; ++j) {
        float x = red[j];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
        red[j] = x;
      }
      if (lane == 0) {
#pragma unroll
        for (int j = 0; j < kPart; ++j) s_red[warp][j] = 0.f;
#pragma unroll
        for (int j = 0; j < kMaxOut; ++j) s_red[warp][j] = red[j];
        s_red[warp][kHO] = red[kMaxOut];
      }
    }
    tc::fence_proxy_async_smem();
    sync_all();
    if (tid == 0 && !s_fail)
      if (!head_bwd(ch)) s_fail = 1;
    ch += 1;
    if (tid < kPart) a.tile_part[(size_t)tile * kPart + tid] = s_red[0][tid] + s_red[1][tid] + s_red[2][tid] + s_red[3][tid];
    sync_all();
    if (s_fail) break;

    // ---- dZ_3 = dA_4 * SiLU'(z_3); z_3 and dA_4 are in TMEM ----
    {
      unsigned char* gdz = chunk_ptr(a.st.dz[3], kDzChunk, tile, row);
#pragma unroll 1
      for (int cb = 0; cb < 4; ++cb) {
        const int col0 = 128 * chalf + 32 * cb;
        float v[32], da[32];
        tc::tmem_ld32(trow + col0, v);
        tc::tmem_ld32(trow + kW + col0, da);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float z = v[i] + s_bias[3][col0 + i];
          const float s = sigmoid_f(z);
          v[i] = da[i] * s * fmaf(z, 1.0f - s, 1.0f);
        }
#pragma unroll
        for (int g8 = 0; g8 < 4; ++g8) {
          const int c8 = col0 + 8 * g8;
          const uint4 p = pack8(v + 8 * g8);
          *reinterpret_cast<uint4*>(sm + kOffAHi + tc::kmajor_off(row, c8, 32)) = p;
          *reinterpret_cast<uint4*>(gdz + arole_off(row & 63, c8)) = p;
        }
      }
    }
    tc::fence_proxy_async_smem();
    sync_all();

    // ---- backward: dA_l = dZ_l W_l, dZ_{l-1} = dA_l * SiLU'(z_{l-1}) ----
    for (int l = 3; l >= 1; --l) {
      // this thread's SiLU derivatives for the epilogue, loaded while the MMAs run
      const unsigned char* ggate = a.st.gate[l - 1] + (size_t)tile * kGateTile;
      uint4 graw[16];
#pragma unroll
      for (int cb = 0; cb < 4; ++cb) {
        const uint4* gp = reinterpret_cast<const uint4*>(ggate + ((size_t)(4 * chalf + cb) * kRows + row) * 64);
#pragma unroll
        for (int g8 = 0; g8 < 4; ++g8) graw[4 * cb + g8] = gp[g8];
      }
      if (tid == 0 && !s_fail)
        if (!gemm(ch, kP1, true)) s_fail = 1;
      ch += kP1;
      sync_all();
      if (s_fail) break;
      unsigned char* gdz = chunk_ptr(a.st.dz[l - 1], kDzChunk, tile, row);
#pragma unroll
      for (int cb = 0; cb < 4; ++cb) {
        const int col0 = 128 * chalf + 32 * cb;
        float v[32];
        tc::tmem_ld32(trow + col0, v);
#pragma unroll
        for (int g8 = 0; g8 < 4; ++g8) {
          float gt[8];
          unpack8(graw[4 * cb + g8], gt);
#pragma unroll
          for (int i = 0; i < 8; ++i) v[8 * g8 + i] *= gt[i];
          const int c8 = col0 + 8 * g8;
          const uint4 p = pack8(v + 8 * g8);
          if (l > 1) *reinterpret_cast<uint4*>(sm + kOffAHi + tc::kmajor_off(row, c8, 32)) = p;
          *reinterpret_cast<uint4*>(gdz + arole_off(row & 63, c8)) = p;
        }
      }
      tc::fence_proxy_async_smem();
      sync_all();
    }
    if (s_fail) break;
  }
  if (s_fail && tid == 0) {
    // let the copies still in flight land (bounded) before the CTA's shared memory goes away
    for (int64_t g = consumed; g < next_load; ++g) {
      const int b = (int)(g % kBufs);
      if (!tc::mbar_wait_bounded(&mbar_full[b], ph_full[b], kWaitTries)) break;
      ph_full[b] ^= 1u;
    }
    atomicExch(a.status, FSG_ETIMEOUT);
  }
  sync_all();
  if (warp == 0) tc::tmem_dealloc(tmem, 2 * kW);
}

// ------------------------------------------------------------------------------------------
// Weight gradients.  CTA (job, split): job < 8 is hidden layer job / 2, output half job % 2
// (dW[m][n] = sum_rows dZ[row][m] A[row][n], plus db[m] = sum_rows dZ[row][m] from an
// all-ones B column); jobs 8, 9 are the head, feature half job - 8 (dW_h^T[k][j] =
// sum_rows A_4[row][k] dOut[row][j]).  The split takes 64-row chunks [s C / S, (s + 1) C / S).
// ------------------------------------------------------------------------------------------
constexpr int kDwStages = 4;
constexpr uint32_t kDwG = 16384;                  // G half chunk: 64 rows x 128 features
constexpr uint32_t kDwH = 32768;                  // H chunk: up to 64 rows x 256
constexpr uint32_t kDwStage = kDwG + kDwH;
constexpr uint32_t kDwOnes = kDwStages * kDwStage;
constexpr uint32_t kDwSmem = kDwOnes + 512 + 1024;
constexpr int kDwJobs = 10;

// The CTAs of the weight-gradient launch: CTAs [off[j], off[j + 1]) split job j's rows, n_split
// CTAs per job.  A CTA's time is set by its number of 64-row chunks (each chunk's copy has to
// arrive from the stash, which does not stay in L2), so every job gets the same split.
struct SplitMap {
  int off[kDwJobs + 1];
};

__host__ __device__ inline SplitMap split_map(int n_split) {
  SplitMap m;
  m.off[0] = 0;
  for (int j = 0; j < kDwJobs; ++j) {
    const int n = n_split;
    m.off[j + 1] = m.off[j] + n;
  }
  return m;
}

struct DwArgs {
  Stash st;
  int n_chunks;            // 64-row chunks in the batch
  SplitMap map;
  float* dw_part;          // [CTA][128][256]
  float* db_part;          // [CTA][128]
  int* status;
};

__global__ void __launch_bounds__(128, 1) mlp_train_dw_kernel(const __grid_constant__ DwArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar_full[kDwStages], mbar_free[kDwStages], mbar_done;
  __shared__ uint32_t tmem_holder;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  int job = 0;
  while (job + 1 < kDwJobs && (int)blockIdx.x >= a.map.off[job + 1]) ++job;
  const int split = (int)blockIdx.x - a.map.off[job], n_split = a.map.off[job + 1] - a.map.off[job];
  const bool head = job >= 8;
  const int layer = head ? 4 : job / 2, half = head ? job - 8 : job % 2;
  const int wd = head ? kHO : (layer == 0 ? kFeat : kW);
  const unsigned char* gsrc = head ? a.st.act[4] : a.st.dz[layer];
  const unsigned char* hsrc = head ? a.st.dout : a.st.act[layer];
  const size_t g_chunk = kDzChunk;  // A-role tensors are 256 wide
  const size_t h_chunk = (size_t)64 * wd * 2;
  const int c0 = (int)((int64_t)split * a.n_chunks / n_split);
  const int c1 = (int)((int64_t)(split + 1) * a.n_chunks / n_split);

  if (tid == 0) {
    for (int s = 0; s < kDwStages; ++s) {
      tc::mbar_init(&mbar_full[s], 1);
      tc::mbar_init(&mbar_free[s], 1);
    }
    tc::mbar_init(&mbar_done, 1);
    tc::fence_mbar_init();
    s_fail = 0;
  }
  // the all-ones B column (N = 16, K = 16, MN-major): B[n][k] = (n == 0)
  {
    __nv_bfloat16* ones = reinterpret_cast<__nv_bfloat16*>(sm + kDwOnes);
    for (int i = tid; i < 256; i += blockDim.x) {
      const int n = i % 16, k = i / 16;
      const uint32_t off = tc::mnmajor_off(n, k, 2);
      ones[off / 2] = __float2bfloat16_rn(n == 0 ? 1.0f : 0.0f);
    }
  }
  tc::fence_proxy_async_smem();
  if (warp == 0) tc::tmem_alloc(&tmem_holder, 512);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_holder;
  const uint32_t sbase = tc::smem_u32(sm);

  if (tid == 0) {
    const uint32_t idw = tc::idesc_bf16(128, wd, 1, 1);
    const uint32_t idb = tc::idesc_bf16(128, 16, 1, 1);
    const uint64_t dones = tc::sdesc(sbase + kDwOnes, 2 * 128, 128);
    const int n = c1 - c0;
    uint32_t ph_full[kDwStages] = {}, ph_free[kDwStages] = {};
    bool ok = true;
    int next = 0, consumed = 0;
    // Copies chunk i into stage i % kDwStages once the stage's previous chunk is released by its
    // MMAs: blocking (bounded; `failed` on timeout) or, for look-ahead copies, only if the release
    // has already happened, so the MMAs of consecutive chunks stay queued back to back.
    bool failed = false;
    auto issue = [&](int i, bool block) -> bool {
      const int s = i % kDwStages;
      if (i >= kDwStages) {
        if (block) {
          if (!tc::mbar_wait_bounded(&mbar_free[s], ph_free[s], kWaitTries)) {
            failed = true;
            return false;
          }
        } else if (!tc::mbar_test(&mbar_free[s], ph_free[s])) {
          return false;
        }
        ph_free[s] ^= 1u;
      }
      unsigned char* dst = sm + s * kDwStage;
      const int q = c0 + i;
      tc::mbar_arrive_expect_tx(&mbar_full[s], kDwG + (uint32_t)h_chunk);
      tc::bulk_g2s(dst, gsrc + (size_t)q * g_chunk + (size_t)half * kDwG, kDwG, &mbar_full[s]);
      tc::bulk_g2s(dst + kDwG, hsrc + (size_t)q * h_chunk, (uint32_t)h_chunk, &mbar_full[s]);
      return true;
    };
    for (int i = 0; i < n && ok; ++i) {
      while (next < n && next < i + kDwStages) {
        if (!issue(next, next <= i)) break;
        ++next;
      }
      if (failed) { ok = false; break; }
      const int s = i % kDwStages;
      if (!tc::mbar_wait_bounded(&mbar_full[s], ph_full[s], kWaitTries)) { ok = false; break; }
      ph_full[s] ^= 1u;
      ++consumed;
      tc::fence_after_sync();
      const uint32_t gb = sbase + s * kDwStage, hb = gb + kDwG;
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
        const uint64_t ad = tc::sdesc(gb + ks * 2 * 2048, 2048, 128);
        const uint64_t bd = tc::sdesc(hb + ks * 2 * (wd / 8) * 128, (wd / 8) * 128, 128);
        tc::mma_bf16(tmem, ad, bd, idw, (i > 0 || ks > 0) ? 1u : 0u);
        if (!head) tc::mma_bf16(tmem + 256, ad, dones, idb, (i > 0 || ks > 0) ? 1u : 0u);
      }
      tc::commit(&mbar_free[s]);
    }
    if (ok) {
      tc::commit(&mbar_done);
      ok = tc::mbar_wait_bounded(&mbar_done, 0, kWaitTries);
    }
    if (!ok) {
      s_fail = 1;
      // let the copies still in flight land (bounded) before the CTA's shared memory goes away
      for (int i = consumed; i < next; ++i) {
        const int s = i % kDwStages;
        if (!tc::mbar_wait_bounded(&mbar_full[s], ph_full[s], kWaitTries)) break;
        ph_full[s] ^= 1u;
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const int m = 32 * warp + (tid & 31);  // TMEM lane = output row of this half
  float* out = a.dw_part + ((size_t)blockIdx.x * 128 + m) * 256;
  const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
  if (!s_fail) {
    if (c1 > c0) {
      for (int c = 0; c < wd; c += 16) {
        float v[16];
        tmem_ld16(trow + c, v);
#pragma unroll
        for (int i = 0; i < 16; i += 4) *reinterpret_cast<float4*>(out + c + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
      }
      if (!head) {
        float v[16];
        tmem_ld16(trow + 256, v);
        a.db_part[(size_t)blockIdx.x * 128 + m] = v[0];
      }
    } else {  // an empty split contributes zeros
      for (int c = 0; c < wd; ++c) out[c] = 0.f;
      if (!head) a.db_part[(size_t)blockIdx.x * 128 + m] = 0.f;
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (s_fail && tid == 0) atomicExch(a.status, FSG_ETIMEOUT);
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------------------------------------------
// Gradient reduction + Adam.  Parameter p over [W_0 | W_1 | W_2 | W_3 | b_0..b_3 | W_h | b_h].
// ------------------------------------------------------------------------------------------
struct AdamArgs {
  float* w[4];
  float* mw[4];
  float* vw[4];
  void* wf[4];
  void* wb[4];
  float* b[4];
  float* mb[4];
  float* vb[4];
  float* wh;
  float* mwh;
  float* vwh;
  void* head_packed;
  float* bh;
  float* mbh;
  float* vbh;
  const float* dw_part;
  const float* db_part;
  const float* tile_part;
  SplitMap map;
  int n_tiles, n_out;
  int* step;
  float* loss_hist;
  int hist_len;
  float lr, lr_min, b1, b2, eps;
  int total_steps, warmup;
  float inv_batch;
  unsigned int* done;
  float* grads_out;        // if non-NULL: the reduced gradient of every parameter, in order
  int apply;               // 0: only reduce into grads_out (the step counter is left alone)
};

__host__ __device__ inline int64_t n_params(int n_out) {
  return (int64_t)kW * kFeat + 3LL * kW * kW + 4LL * kW + (int64_t)n_out * kW + n_out;
}

__device__ __forceinline__ float adam_step(float g, float w, float& m1, float& m2, float lr, float b1, float b2,
                                           float eps, float bc1, float bc2) {
  m1 = b1 * m1 + (1.f - b1) * g;
  m2 = b2 * m2 + (1.f - b2) * g * g;
  return w - lr * (m1 / bc1) / (sqrtf(m2 / bc2) + eps);
}

// One thread per parameter: the gradient is the fixed-order sum of its job's split partials.
__global__ void __launch_bounds__(256) mlp_train_adam_kernel(const __grid_constant__ AdamArgs a) {
  const int64_t total = n_params(a.n_out);
  const int t = *reinterpret_cast<volatile const int*>(a.step);  // advanced only by the last block
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < total) {
    float g = 0.f;
    float *w, *m1, *m2;
    int layer = -1, mrow = 0, ncol = 0, hj = -1, hk = 0;
    const int64_t nw0 = (int64_t)kW * kFeat, nw = (int64_t)kW * kW;
    const int64_t off_b = nw0 + 3 * nw, off_h = off_b + 4 * kW, off_bh = off_h + (int64_t)a.n_out * kW;
    if (p < off_b) {
      int64_t q;
      if (p < nw0) { layer = 0; q = p; } else { layer = 1 + (int)((p - nw0) / nw); q = (p - nw0) % nw; }
      const int K = layer == 0 ? kFeat : kW;
      mrow = (int)(q / K);
      ncol = (int)(q % K);
      const int job = 2 * layer + mrow / 128;
#pragma unroll 8
      for (int s = a.map.off[job]; s < a.map.off[job + 1]; ++s)
        g += a.dw_part[((size_t)s * 128 + (mrow & 127)) * 256 + ncol];
      w = a.w[layer] + q; m1 = a.mw[layer] + q; m2 = a.vw[layer] + q;
    } else if (p < off_h) {
      const int l = (int)((p - off_b) / kW), mm = (int)((p - off_b) % kW);
      const int job = 2 * l + mm / 128;
#pragma unroll 8
      for (int s = a.map.off[job]; s < a.map.off[job + 1]; ++s) g += a.db_part[(size_t)s * 128 + (mm & 127)];
      w = a.b[l] + mm; m1 = a.mb[l] + mm; m2 = a.vb[l] + mm;
    } else if (p < off_bh) {
      const int64_t q = p - off_h;
      hj = (int)(q / kW);
      hk = (int)(q % kW);
      const int job = 8 + hk / 128;
#pragma unroll 8
      for (int s = a.map.off[job]; s < a.map.off[job + 1]; ++s)
        g += a.dw_part[((size_t)s * 128 + (hk & 127)) * 256 + hj];
      w = a.wh + q; m1 = a.mwh + q; m2 = a.vwh + q;
    } else {
      const int j = (int)(p - off_bh);
      for (int s = 0; s < a.n_tiles; ++s) g += a.tile_part[(size_t)s * kPart + j];
      w = a.bh + j; m1 = a.mbh + j; m2 = a.vbh + j;
    }
    if (a.grads_out) a.grads_out[p] = g;
    if (a.apply) {
      const int tt = t + 1;
      float lr;
      if (tt <= a.warmup) {
        lr = a.lr * (float)tt / (float)max(1, a.warmup);
      } else {
        const float prog = fminf(1.0f, (float)(tt - a.warmup) / (float)max(1, a.total_steps - a.warmup));
        lr = a.lr_min + (a.lr - a.lr_min) * 0.5f * (1.0f + cospif(prog));
      }
      const float bc1 = 1.0f - powf(a.b1, (float)tt), bc2 = 1.0f - powf(a.b2, (float)tt);
      float mv = *m1, vv = *m2;
      const float nwv = adam_step(g, *w, mv, vv, lr, a.b1, a.b2, a.eps, bc1, bc2);
      *m1 = mv;
      *m2 = vv;
      *w = nwv;
      if (hj >= 0) {  // the head's packed chunk: hi and lo (forward), hi (backward)
        const __nv_bfloat16 hi = __float2bfloat16_rn(nwv);
        __nv_bfloat16* o = static_cast<__nv_bfloat16*>(a.head_packed);
        o[(kHeadHi + tc::kmajor_off(hj, hk, kW / 8)) / 2] = hi;
        o[(kHeadLo + tc::kmajor_off(hj, hk, kW / 8)) / 2] = __float2bfloat16_rn(nwv - __bfloat162float(hi));
        o[(kHeadBwd + tc::mnmajor_off(hk, hj, kW / 8)) / 2] = hi;
      }
      if (layer >= 0) {
        const __nv_bfloat16 hb = __float2bfloat16_rn(nwv);
        __nv_bfloat16* f = static_cast<__nv_bfloat16*>(a.wf[layer]);
        f[(size_t)(ncol / kChunkK) * (kChunkBytes / 2) + wpack_off(mrow, ncol % kChunkK) / 2] = hb;
        if (layer > 0) {
          __nv_bfloat16* b = static_cast<__nv_bfloat16*>(a.wb[layer]);
          b[(size_t)(mrow / kChunkK) * (kChunkBytes / 2) + tc::mnmajor_off(ncol, mrow % kChunkK, kW / 8) / 2] = hb;
        }
      }
    }
  }
  if (!a.apply) return;
  // the last block to finish records the step's loss and advances the step counter
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(a.done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  if (threadIdx.x == 0) {
    float loss = 0.f;
    for (int s = 0; s < a.n_tiles; ++s) loss += a.tile_part[(size_t)s * kPart + kHO];
    if (a.loss_hist && t < a.hist_len) a.loss_hist[t] = loss * a.inv_batch;
    *a.done = 0u;
    __threadfence();
    *a.step = t + 1;
  }
}

// Writes the packed BF16 copies of hidden layer l from its FP32 master weights.
// Writes the packed head chunk: entry (region r, output j, feature k) of W_h, zero for j >= n_out.
__global__ void mlp_train_pack_head_kernel(const float* __restrict__ wh, int n_out, void* packed) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * kHO * kW) return;
  const int r = t / (kHO * kW), j = (t / kW) % kHO, k = t % kW;
  float v = 0.f;
  if (j < n_out) {
    const float w = wh[j * kW + k];
    const __nv_bfloat16 hi = __float2bfloat16_rn(w);
    v = r == 1 ? w - __bfloat162float(hi) : w;
  }
  __nv_bfloat16* o = static_cast<__nv_bfloat16*>(packed);
  const uint32_t off = r == 2 ? kHeadBwd + tc::mnmajor_off(k, j, kW / 8) : (r ? kHeadLo : kHeadHi) + tc::kmajor_off(j, k, kW / 8);
  o[off / 2] = __float2bfloat16_rn(v);
}

__global__ void mlp_train_pack_kernel(const float* __restrict__ w, int layer, void* wf, void* wb) {
  const int K = layer == 0 ? kFeat : kW;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kW * K) return;
  const int m = i / K, n = i % K;
  const __nv_bfloat16 hb = __float2bfloat16_rn(w[i]);
  static_cast<__nv_bfloat16*>(wf)[(size_t)(n / kChunkK) * (kChunkBytes / 2) + wpack_off(m, n % kChunkK) / 2] = hb;
  if (layer > 0 && wb)
    static_cast<__nv_bfloat16*>(wb)[(size_t)(m / kChunkK) * (kChunkBytes / 2) + tc::mnmajor_off(n, m % kChunkK, 32) / 2] =
        hb;
}

}  // namespace mlpt
}  // namespace fsg

using namespace fsg;
using namespace fsg::mlpt;

namespace {

size_t stash_bytes_for(int n_tiles) {
  const size_t chunks = (size_t)n_tiles * 2;
  size_t b = chunks * (act_chunk_bytes(0) + 4 * act_chunk_bytes(1) + 4 * kDzChunk + kDoutChunk);
  b += (size_t)n_tiles * 3 * kGateTile;
  return b;
}

Stash carve_stash(unsigned char* base, int n_tiles) {
  const size_t chunks = (size_t)n_tiles * 2;
  Stash s;
  size_t o = 0;
  for (int l = 0; l < 5; ++l) {
    s.act[l] = base + o;
    o += chunks * act_chunk_bytes(l);
  }
  for (int l = 0; l < 4; ++l) {
    s.dz[l] = base + o;
    o += chunks * kDzChunk;
  }
  s.dout = base + o;
  o += chunks * kDoutChunk;
  for (int l = 0; l < 3; ++l) {
    s.gate[l] = base + o;
    o += (size_t)n_tiles * kGateTile;
  }
  return s;
}

size_t part_bytes(int n_split, int n_tiles) {
  const size_t ctas = (size_t)split_map(n_split).off[kDwJobs];
  return ctas * 128 * 256 * 4 + ctas * 128 * 4 + (size_t)n_tiles * kPart * 4 + 256;
}

int validate_train(const FsgMlpTrain* t) {
  if (!t) return set_error(FSG_EINVAL, "NULL training descriptor");
  if (t->n_tiles < 1) return set_error(FSG_EINVAL, "n_tiles must be >= 1 (batch = 128 n_tiles rows)");
  if (t->n_out < 2 || t->n_out > kMaxOut || t->n_out % 2)
    return set_error(FSG_EUNSUPPORTED, "n_out must be even and in [2, %d] (got %d)", kMaxOut, t->n_out);
  if (t->n_data < 1 || !t->u || !t->aux) return set_error(FSG_EINVAL, "empty training set");
  if (t->n_split < 1 || t->n_split > 64) return set_error(FSG_EINVAL, "n_split must be in [1, 64]");
  for (int l = 0; l < 4; ++l)
    if (!t->w[l] || !t->m_w[l] || !t->v_w[l] || !t->packed_fwd[l] || !t->b[l] || !t->m_b[l] || !t->v_b[l] ||
        (l > 0 && !t->packed_bwd[l]))
      return set_error(FSG_EINVAL, "layer %d parameters missing", l);
  if (!t->w_head || !t->m_w_head || !t->v_w_head || !t->b_head || !t->m_b_head || !t->v_b_head || !t->bmat ||
      !t->packed_head)
    return set_error(FSG_EINVAL, "head or feature parameters missing");
  if (!t->step || !t->status || !t->workspace) return set_error(FSG_EINVAL, "step counter, status or workspace missing");
  if (t->workspace_bytes < fsg_mlp_train_workspace_size(t->n_tiles, t->n_split))
    return set_error(FSG_EWORKSPACE, "training workspace of %zu bytes is smaller than the %zu bytes required",
                     t->workspace_bytes, fsg_mlp_train_workspace_size(t->n_tiles, t->n_split));
  return FSG_OK;
}

int launch_step(const FsgMlpTrain* t, int apply, float* grads_out, int* rows_out, cudaStream_t s) {
  static bool attr_done[64] = {};
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return check_cuda(e, "device query");
  if (dev >= 0 && dev < 64 && !attr_done[dev]) {
    e = cudaFuncSetAttribute(mlp_train_fb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFbSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(mlp_train_dw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDwSmem);
    if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute (training kernels)");
    attr_done[dev] = true;
  }
  unsigned char* ws = static_cast<unsigned char*>(t->workspace);
  Stash st = carve_stash(ws, t->n_tiles);
  unsigned char* pb = ws + stash_bytes_for(t->n_tiles);
  float* dw_part = reinterpret_cast<float*>(pb);
  const SplitMap map = split_map(t->n_split);
  const int dw_ctas = map.off[kDwJobs];
  float* db_part = dw_part + (size_t)dw_ctas * 128 * 256;
  float* tile_part = db_part + (size_t)dw_ctas * 128;
  unsigned int* done = reinterpret_cast<unsigned int*>(tile_part + (size_t)t->n_tiles * kPart);

  FbArgs fa;
  fa.u = t->u;
  fa.aux = t->aux;
  fa.n_data = t->n_data;
  fa.seed = t->seed;
  fa.step = t->step;
  fa.net.bmat = t->bmat;
  for (int l = 0; l < 4; ++l) {
    fa.net.wf[l] = t->packed_fwd[l];
    fa.net.wb[l] = t->packed_bwd[l];
    fa.net.bias[l] = t->b[l];
  }
  fa.net.whead = t->packed_head;
  fa.net.bhead = t->b_head;
  fa.net.n_out = t->n_out;
  fa.inv_batch = 1.0f / (float)(t->n_tiles * kRows);
  fa.st = st;
  fa.tile_part = tile_part;
  fa.n_tiles = t->n_tiles;
  fa.rows_out = rows_out;
  fa.status = t->status;
  const int grid = t->n_tiles < sms ? t->n_tiles : sms;
  mlp_train_fb_kernel<<<grid, 256, kFbSmem, s>>>(fa);
  int st_ = check_cuda(cudaGetLastError(), "mlp_train_fb_kernel launch");
  if (st_ != FSG_OK) return st_;

  DwArgs da;
  da.st = st;
  da.n_chunks = t->n_tiles * 2;
  da.map = map;
  da.dw_part = dw_part;
  da.db_part = db_part;
  da.status = t->status;
  mlp_train_dw_kernel<<<dw_ctas, 128, kDwSmem, s>>>(da);
  if ((st_ = check_cuda(cudaGetLastError(), "mlp_train_dw_kernel launch")) != FSG_OK) return st_;

  AdamArgs aa;
  for (int l = 0; l < 4; ++l) {
    aa.w[l] = t->w[l];
    aa.mw[l] = t->m_w[l];
    aa.vw[l] = t->v_w[l];
    aa.wf[l] = t->packed_fwd[l];
    aa.wb[l] = t->packed_bwd[l];
    aa.b[l] = t->b[l];
    aa.mb[l] = t->m_b[l];
    aa.vb[l] = t->v_b[l];
  }
  aa.wh = t->w_head;
  aa.mwh = t->m_w_head;
  aa.vwh = t->v_w_head;
  aa.head_packed = t->packed_head;
  aa.bh = t->b_head;
  aa.mbh = t->m_b_head;
  aa.vbh = t->v_b_head;
  aa.dw_part = dw_part;
  aa.db_part = db_part;
  aa.tile_part = tile_part;
  aa.map = map;
  aa.n_tiles = t->n_tiles;
  aa.n_out = t->n_out;
  aa.step = t->step;
  aa.loss_hist = t->loss_hist;
  aa.hist_len = t->loss_hist_len;
  aa.lr = t->lr;
  aa.lr_min = t->lr_min;
  aa.b1 = t->beta1;
  aa.b2 = t->beta2;
  aa.eps = t->eps;
  aa.total_steps = t->total_steps;
  aa.warmup = t->warmup_steps;
  aa.inv_batch = fa.inv_batch;
  aa.done = done;
  aa.grads_out = grads_out;
  aa.apply = apply;
  const int64_t np = n_params(t->n_out);
  mlp_train_adam_kernel<<<(unsigned)((np + 255) / 256), 256, 0, s>>>(aa);
  return check_cuda(cudaGetLastError(), "mlp_train_adam_kernel launch");
}

}  // namespace

extern "C" size_t fsg_mlp_train_workspace_size(int32_t n_tiles, int32_t n_split) {
  if (n_tiles < 1 || n_split < 1) return 0;
  return stash_bytes_for(n_tiles) + part_bytes(n_split, n_tiles);
}

extern "C" int64_t fsg_mlp_train_n_params(int32_t n_out) { return n_params(n_out); }

extern "C" int32_t fsg_mlp_train_init(const FsgMlpTrain* t, void* stream) {
  int st = validate_train(t);
  if (st != FSG_OK) return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  for (int l = 0; l < 4; ++l) {
    const int K = l == 0 ? kFeat : kW;
    mlp_train_pack_kernel<<<(kW * K + 255) / 256, 256, 0, s>>>(t->w[l], l, t->packed_fwd[l], t->packed_bwd[l]);
    if ((st = check_cuda(cudaGetLastError(), "mlp_train_pack_kernel launch")) != FSG_OK) return st;
  }
  mlp_train_pack_head_kernel<<<(3 * kHO * kW + 255) / 256, 256, 0, s>>>(t->w_head, t->n_out, t->packed_head);
  if ((st = check_cuda(cudaGetLastError(), "mlp_train_pack_head_kernel launch")) != FSG_OK) return st;
  unsigned char* ws = static_cast<unsigned char*>(t->workspace);
  unsigned char* done = ws + fsg_mlp_train_workspace_size(t->n_tiles, t->n_split) - 256;
  return check_cuda(cudaMemsetAsync(done, 0, 256, s), "training counter reset");
}

extern "C" int32_t fsg_mlp_train_steps(const FsgMlpTrain* t, int32_t n_steps, void* stream) {
  int st = validate_train(t);
  if (st != FSG_OK) return st;
  if (n_steps < 0) return set_error(FSG_EINVAL, "n_steps must be >= 0");
  for (int i = 0; i < n_steps; ++i)
    if ((st = launch_step(t, 1, nullptr, nullptr, reinterpret_cast<cudaStream_t>(stream))) != FSG_OK) return st;
  return FSG_OK;
}

extern "C" int32_t fsg_mlp_train_gradients(const FsgMlpTrain* t, float* grads_out, int32_t* rows_out, void* stream) {
  int st = validate_train(t);
  if (st != FSG_OK) return st;
  if (!grads_out || !rows_out) return set_error(FSG_EINVAL, "grads_out and rows_out must be non-NULL");
  return launch_step(t, 0, grads_out, rows_out, reinterpret_cast<cudaStream_t>(stream));
}

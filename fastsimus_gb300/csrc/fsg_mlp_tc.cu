// Fused tcgen05 forward pass of the transmit-field surrogate network (inference).
//
// Network: 64 random Fourier features [sin(2 pi B u), cos(2 pi B u)] of the normalised
// inputs, four hidden layers of 256 with SiLU, a linear head of n_out <= 10 outputs (the same
// network that the training kernels of fsg_mlp_train.cu train, with the same SiLU).  A persistent CTA takes 128 queries at a time and keeps everything on
// chip:
//   features -> A (shared memory, BF16 hi + lo, K-major core matrices)
//   per hidden layer: D (TMEM, 128 x 256 FP32) = A_hi W^T + A_lo W^T, two tcgen05.mma
//   kind::f16 per K step of 16, the layer's BF16 weights streamed through two 32 KB
//   shared-memory buffers by TMA bulk copies (64 input columns per copy);
//   epilogue: D + bias -> SiLU -> next layer's A (hi + lo), or, after the last hidden layer,
//   the 256 -> n_out head on the CUDA cores.
// The weights are BF16 (as in training) and multiply exactly; splitting the activations into
// hi + lo BF16 keeps them at FP32-class precision (~1e-5 relative), as in the training forward
// pass.  Every mbarrier wait is bounded: on timeout the CTA
// records FSG_ETIMEOUT in the status word, frees its TMEM and returns.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/fsgb300.h"
#include "fsg_internal.h"
#include "fsg_tc.cuh"

namespace fsg {

constexpr int kMlpRows = 128;      // queries per tile (MMA M)
constexpr int kMlpWidth = 256;     // hidden width (MMA N)
constexpr int kMlpFeat = 128;      // 2 x 64 Fourier features
constexpr int kMlpChunkK = 64;     // input columns per weight copy
constexpr uint32_t kMlpChunkBytes = kMlpWidth * kMlpChunkK * 2;  // 32 KB
constexpr uint32_t kMlpKGroups = kMlpWidth / 8;                 // A operand: 32 core matrices along K
constexpr uint32_t kMlpABytes = kMlpRows * kMlpWidth * 2;       // 64 KB per hi / lo
constexpr uint32_t kOffAHi = 0;
constexpr uint32_t kOffALo = kMlpABytes;
constexpr uint32_t kOffB0 = 2 * kMlpABytes;
constexpr uint32_t kOffB1 = kOffB0 + kMlpChunkBytes;
constexpr uint32_t kMlpSmem = kOffB1 + kMlpChunkBytes + 1024;
constexpr uint32_t kMlpWaitTries = 1u << 26;
constexpr int kMlpMaxOut = 10;

// SiLU z * sigmoid(z) with the fast exponential and reciprocal, evaluated exactly as the
// training kernels evaluate it.
__device__ __forceinline__ float mlp_silu(float z) { return z * __fdividef(1.0f, 1.0f + __expf(-z)); }

// Writes 8 consecutive activations (row r, columns k..k+7) as hi and lo BF16 into the K-major
// A operand.
__device__ __forceinline__ void store_a8(unsigned char* sm, int r, int k, const float* v) {
  uint4 hi, lo;
  tc::split8(v, hi, lo);
  const uint32_t off = tc::kmajor_off(r, k, kMlpKGroups);
  *reinterpret_cast<uint4*>(sm + kOffAHi + off) = hi;
  *reinterpret_cast<uint4*>(sm + kOffALo + off) = lo;
}

__global__ void __launch_bounds__(256, 1) mlp_tc_forward_kernel(const __grid_constant__ FsgMlpWeights W,
                                                                 const float* __restrict__ u, int64_t n,
                                                                 float* __restrict__ out, int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar_full[2], mbar_free[2], mbar_layer;
  __shared__ uint32_t tmem_holder;
  __shared__ int s_fail;
  __shared__ float bmat[64 * 4];
  __shared__ float whead[kMlpMaxOut][kMlpWidth];
  __shared__ float bias_s[4][kMlpWidth];
  __shared__ float hsum[kMlpRows][kMlpMaxOut];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nout = W.n_out;
  for (int i = tid; i < 64 * 4; i += blockDim.x) bmat[i] = W.bmat[i];
  for (int i = tid; i < kMlpMaxOut * kMlpWidth; i += blockDim.x)
    whead[i / kMlpWidth][i % kMlpWidth] = (i / kMlpWidth < nout) ? W.w_head[i] : 0.f;
  for (int i = tid; i < 4 * kMlpWidth; i += blockDim.x) bias_s[i / kMlpWidth][i % kMlpWidth] = W.bias[i / kMlpWidth][i % kMlpWidth];
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&mbar_full[b], 1);
      tc::mbar_init(&mbar_free[b], 1);
    }
    tc::mbar_init(&mbar_layer, 1);
    tc::fence_mbar_init();
    s_fail = 0;
  }
  if (warp == 0) tc::tmem_alloc(&tmem_holder, kMlpWidth);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_holder;
  const uint32_t sbase = tc::smem_u32(sm);
  const uint32_t idesc = tc::idesc_bf16(kMlpRows, kMlpWidth, 0, 0);
  // Thread 0 streams the weights as one sequence of 32 KB chunks over all layers and tiles
  // (kChunksPerTile per tile), keeping up to two in flight; chunk g goes to buffer g & 1.
  constexpr int kChunksPerTile = kMlpFeat / kMlpChunkK + 3 * (kMlpWidth / kMlpChunkK);
  uint32_t ph_full[2] = {0u, 0u}, ph_free[2] = {0u, 0u}, ph_layer = 0u;
  int64_t next_load = 0;  // next chunk to copy
  const int64_t my_tiles = ((n + kMlpRows - 1) / kMlpRows - blockIdx.x + gridDim.x - 1) / gridDim.x;
  const int64_t total_chunks = my_tiles * kChunksPerTile;
  // issue the copy of chunk g; before reusing a buffer, wait for the MMAs of chunk g - 2
  auto load = [&](int64_t g) -> bool {
    const int b = (int)(g & 1);
    if (g >= 2) {
      if (!tc::mbar_wait_bounded(&mbar_free[b], ph_free[b], kMlpWaitTries)) return false;
      ph_free[b] ^= 1u;
    }
    const int j = (int)(g % kChunksPerTile);
    const int layer = j < 2 ? 0 : 1 + (j - 2) / 4, c = j < 2 ? j : (j - 2) % 4;
    tc::mbar_arrive_expect_tx(&mbar_full[b], kMlpChunkBytes);
    tc::bulk_g2s(sm + (b ? kOffB1 : kOffB0),
                 static_cast<const unsigned char*>(W.packed[layer]) + (size_t)c * kMlpChunkBytes, kMlpChunkBytes,
                 &mbar_full[b]);
    return true;
  };
  int64_t tile_iter = 0;

  // TMEM read mapping: row = 32 (warp % 4) + lane, columns [128 (warp / 4), +128)
  const int row = 32 * (warp & 3) + lane, chalf = warp >> 2;
  const int64_t n_tiles = (n + kMlpRows - 1) / kMlpRows;

  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    // ---- features of the tile's queries -> A (K = 128) ----
    {
      const int r = tid & (kMlpRows - 1), half = tid >> 7;
      const int64_t q = tile * kMlpRows + r;
      float4 uv = make_float4(0.f, 0.f, 0.f, 0.f);
      if (q < n) uv = make_float4(u[4 * q], u[4 * q + 1], u[4 * q + 2], u[4 * q + 3]);
#pragma unroll
      for (int blk = 0; blk < 4; ++blk) {
        float sv[8], cv[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int j = 32 * half + 8 * blk + i;
          const float t = bmat[4 * j] * uv.x + bmat[4 * j + 1] * uv.y + bmat[4 * j + 2] * uv.z + bmat[4 * j + 3] * uv.w;
          sincospif(2.0f * t, &sv[i], &cv[i]);
        }
        store_a8(sm, r, 32 * half + 8 * blk, sv);
        store_a8(sm, r, 64 + 32 * half + 8 * blk, cv);
      }
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();

    float head[kMlpMaxOut];
#pragma unroll
    for (int j = 0; j < kMlpMaxOut; ++j) head[j] = 0.f;
    int64_t chunk0 = tile_iter * kChunksPerTile;  // global index of this layer's first chunk
    for (int layer = 0; layer < 4; ++layer) {
      const int K = layer == 0 ? kMlpFeat : kMlpWidth;
      const int nch = K / kMlpChunkK;
      // ---- MMAs: thread 0 keeps two weight chunks in flight and issues the products ----
      if (tid == 0 && !s_fail) {
        bool ok = true;
        for (int c = 0; c < nch && ok; ++c) {
          const int64_t g = chunk0 + c;
          const int b = (int)(g & 1);
          // the look-ahead copy (chunk g + 1) reuses chunk g - 1's buffer: issue it only if that
          // chunk's MMAs are done, so that the MMAs of consecutive chunks stay queued back to back
          while (ok && next_load < g + 2 && next_load < total_chunks) {
            if (next_load > g && next_load >= 2 &&
                !tc::mbar_test(&mbar_free[next_load & 1], ph_free[next_load & 1]))
              break;
            ok = load(next_load++);
          }
          if (!ok) break;
          if (!tc::mbar_wait_bounded(&mbar_full[b], ph_full[b], kMlpWaitTries)) { ok = false; break; }
          ph_full[b] ^= 1u;
          tc::fence_after_sync();
          const uint32_t bb = sbase + (b ? kOffB1 : kOffB0);
#pragma unroll
          for (int ks = 0; ks < kMlpChunkK / 16; ++ks) {
            const int kk = c * (kMlpChunkK / 16) + ks;  // K step of 16 within the layer
            const uint64_t ah = tc::sdesc(sbase + kOffAHi + kk * 256, 128, kMlpKGroups * 128);
            const uint64_t al = tc::sdesc(sbase + kOffALo + kk * 256, 128, kMlpKGroups * 128);
            // k-group-major packed chunk: K stride 4096 bytes, N stride 128
            const uint64_t bd = tc::sdesc(bb + ks * 2 * 4096, 4096, 128);
            tc::mma_bf16(tmem, ah, bd, idesc, kk > 0);
            tc::mma_bf16(tmem, al, bd, idesc, 1);
          }
          tc::commit(&mbar_free[b]);
        }
        if (ok) {
          tc::commit(&mbar_layer);
          ok = tc::mbar_wait_bounded(&mbar_layer, ph_layer, kMlpWaitTries);
          ph_layer ^= 1u;
        }
        // the layer's products are done and both buffers are free: start the next two
        // copies now, so that they land while the epilogue runs
        while (ok && next_load < chunk0 + nch + 2 && next_load < total_chunks) ok = load(next_load++);
        if (!ok) s_fail = 1;
      }
      chunk0 += nch;
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      if (s_fail) break;
      // ---- epilogue: bias + SiLU -> next A, or the head ----
      const float* bias = bias_s[layer];
#pragma unroll 1
      for (int cb = 0; cb < 4; ++cb) {
        const int col0 = 128 * chalf + 32 * cb;
        float v[32];
        tc::tmem_ld32(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + col0, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = mlp_silu(v[i] + bias[col0 + i]);
        if (layer < 3) {
#pragma unroll
          for (int g8 = 0; g8 < 4; ++g8) store_a8(sm, row, col0 + 8 * g8, v + 8 * g8);
        } else {
#pragma unroll
          for (int j = 0; j < kMlpMaxOut; ++j) {
            float acc = head[j];
#pragma unroll
            for (int i = 0; i < 32; ++i) acc = fmaf(v[i], whead[j][col0 + i], acc);
            head[j] = acc;
          }
        }
      }
      tc::fence_proxy_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
    }
    if (s_fail) break;
    // ---- head: combine the two column halves of each row ----
    if (chalf == 1) {
#pragma unroll
      for (int j = 0; j < kMlpMaxOut; ++j) hsum[row][j] = head[j];
    }
    __syncthreads();
    if (chalf == 0) {
      const int64_t q = tile * kMlpRows + row;
      if (q < n) {
        for (int j = 0; j < nout; ++j) out[q * nout + j] = head[j] + hsum[row][j] + W.b_head[j];
      }
    }
    __syncthreads();
    ++tile_iter;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (s_fail && tid == 0) atomicExch(status, FSG_ETIMEOUT);
  if (warp == 0) tc::tmem_dealloc(tmem, kMlpWidth);
}

// Packs a row-major [256][K] BF16 weight matrix into K/64 chunks of the K-major no-swizzle
// core-matrix layout that the forward kernel copies into shared memory as the B operand.
__global__ void mlp_pack_kernel(const __nv_bfloat16* __restrict__ w, int K, __nv_bfloat16* __restrict__ packed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kMlpWidth * K) return;
  const int n = i / K, k = i % K;
  const int c = k / kMlpChunkK, kk = k % kMlpChunkK;
  // bytes within the chunk: core (kk / 8, n / 8) at ((kk / 8) * 32 + n / 8) * 128 (k-group-major)
  const uint32_t off = ((uint32_t)(((kk >> 3) << 5) + (n >> 3)) << 7) + ((uint32_t)(n & 7) << 4) + ((uint32_t)(kk & 7) << 1);
  packed[(size_t)c * (kMlpChunkBytes / 2) + off / 2] = w[i];
}

}  // namespace fsg

using namespace fsg;

extern "C" size_t fsg_mlp_tc_packed_bytes(int32_t n_in) {
  if (n_in < kMlpChunkK || n_in % kMlpChunkK) return 0;
  return (size_t)kMlpWidth * n_in * 2;
}

extern "C" int32_t fsg_mlp_tc_pack(const void* w_bf16, int32_t n_out, int32_t n_in, void* packed, void* stream) {
  if (!w_bf16 || !packed) return set_error(FSG_EINVAL, "NULL argument");
  if (n_out != kMlpWidth || n_in < kMlpChunkK || n_in % kMlpChunkK)
    return set_error(FSG_EUNSUPPORTED, "tensor-core MLP layers are %d x K with K a multiple of %d (got %d x %d)",
                     kMlpWidth, kMlpChunkK, n_out, n_in);
  const int total = n_out * n_in;
  mlp_pack_kernel<<<(total + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(w_bf16), n_in, static_cast<__nv_bfloat16*>(packed));
  return check_cuda(cudaGetLastError(), "mlp_pack_kernel launch");
}

extern "C" int32_t fsg_mlp_tc_forward(const FsgMlpWeights* weights, const float* u, int64_t n, float* out, int32_t* status,
                                      void* stream_ptr) {
  if (!weights || !u || !out || !status || n < 0) return set_error(FSG_EINVAL, "NULL argument or n < 0");
  for (int l = 0; l < 4; ++l)
    if (!weights->packed[l] || !weights->bias[l]) return set_error(FSG_EINVAL, "layer %d weights or bias missing", l);
  if (!weights->w_head || !weights->b_head || !weights->bmat) return set_error(FSG_EINVAL, "head or features missing");
  if (weights->n_out < 1 || weights->n_out > kMlpMaxOut)
    return set_error(FSG_EUNSUPPORTED, "n_out must be in [1, %d] (got %d)", kMlpMaxOut, weights->n_out);
  if (n == 0) return FSG_OK;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return check_cuda(e, "device query");
  e = cudaFuncSetAttribute(mlp_tc_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMlpSmem);
  if (e != cudaSuccess) return check_cuda(e, "cudaFuncSetAttribute(mlp_tc_forward_kernel)");
  const int64_t tiles = (n + kMlpRows - 1) / kMlpRows;
  const int grid = (int)(tiles < sms ? tiles : sms);
  mlp_tc_forward_kernel<<<grid, 256, kMlpSmem, reinterpret_cast<cudaStream_t>(stream_ptr)>>>(*weights, u, n, out,
                                                                                               status);
  return check_cuda(cudaGetLastError(), "mlp_tc_forward_kernel launch");
}

// The learned correction's network on the tensor cores: training (forward,
// backward, weight gradients) and inference with tcgen05.mma, bf16 operands and
// fp32 accumulators in tensor memory.
//
// One CTA of 128 threads owns tiles of 128 samples; thread t holds sample t of
// the tile, which is also tensor-memory lane t of every accumulator, so the
// epilogues (bias, SiLU, its derivative, the loss) are per-thread register work
// between MMAs. Activations go back to shared memory in the canonical K-major
// layout as the next MMA's A operand. The weight gradients need the batch as
// the reduction dimension: each thread also scatters its activations and
// deltas as column t of transposed tiles, and two MMA groups accumulate
//   [H2^T ; dZ2^T] (128 x batch) * [dY^T ; H1^T]^T  ->  dW3^T (rows 0-63, cols 0-15)
//                                                      dW2   (rows 64-127, cols 16-79)
//   [dZ2^T ; dZ1^T] (128 x batch) * X                ->  dW1   (rows 64-127)
// in tensor memory over all tiles of the CTA. Bias gradients and the loss are
// warp-shuffle sums in a fixed order. Every CTA writes one partial gradient;
// one block adds the partials in CTA order (deterministic) and takes the Adam
// step. Training runs as CUDA graphs of whole chunks of steps; the step counter
// lives on the device.
#include <cuda_bf16.h>
#include <stdlib.h>
#include <string.h>
#include "pstep_internal.cuh"
#include "pstep_mlp.h"
#include "tc05.cuh"

namespace pmlp {

constexpr int kIn = PMLP_IN, kInP = 16, kHid = PMLP_HIDDEN, kOut = PMLP_OUT, kOutP = 16;
constexpr int kRows = 128;  // samples per tile = threads per CTA = tensor-memory lanes
constexpr int OW1 = 0, OB1 = OW1 + kHid * kInP, OW2 = OB1 + kHid, OB2 = OW2 + kHid * kHid, OW3 = OB2 + kHid,
              OB3 = OW3 + kOutP * kHid, kNParam = OB3 + kOutP;
static_assert(kNParam == PMLP_NPARAM, "parameter layout");
constexpr int kPartial = kNParam + 4;  // + loss
constexpr uint32_t kWaitLimit = 1u << 22;  // bounded polls of an MMA completion

// shared memory of the training kernel (bytes)
constexpr uint32_t S_XA = 0;                        // X     [128 x 16]
constexpr uint32_t S_H1A = S_XA + kRows * kInP * 2;  // H1    [128 x 64]
constexpr uint32_t S_H2A = S_H1A + kRows * kHid * 2;
constexpr uint32_t S_DYA = S_H2A + kRows * kHid * 2;  // dY    [128 x 16]
constexpr uint32_t S_DZ2A = S_DYA + kRows * kOutP * 2;  // dZ2  [128 x 64]
constexpr uint32_t S_W1 = S_DZ2A + kRows * kHid * 2;  // W1    [64 x 16]
constexpr uint32_t S_W2 = S_W1 + kHid * kInP * 2;      // W2    [64 x 64]
constexpr uint32_t S_W3 = S_W2 + kHid * kHid * 2;      // W3    [16 x 64]
constexpr uint32_t S_W3T = S_W3 + kOutP * kHid * 2;    // W3^T  [64 x 16]
constexpr uint32_t S_W2T = S_W3T + kHid * kOutP * 2;   // W2^T  [64 x 64]
constexpr uint32_t S_AT = S_W2T + kHid * kHid * 2;     // [H2^T ; dZ2^T ; dZ1^T] [192 x 128]
constexpr uint32_t S_BT1 = S_AT + 192 * kRows * 2;     // [dY^T ; H1^T] [80 x 128]
constexpr uint32_t S_BT2 = S_BT1 + 80 * kRows * 2;     // X^T [16 x 128]
constexpr uint32_t S_BIAS = S_BT2 + kInP * kRows * 2;  // b1, b2, b3 (fp32)
constexpr int kRedW = 136;                             // per warp: db1[64] db2[64] db3[4] loss
constexpr uint32_t S_RED = S_BIAS + (kHid + kHid + kOutP) * 4;
constexpr uint32_t S_DS1 = S_RED + 4 * kRedW * 4;    // SiLU'(z1) [64][128] fp32, sample index fastest
constexpr uint32_t S_MISC = S_DS1 + kHid * kRows * 4;
constexpr uint32_t kTrainSmem = S_MISC + 64;

// shared memory of the inference kernel
constexpr uint32_t I_XA = 0, I_H1A = I_XA + kRows * kInP * 2, I_H2A = I_H1A + kRows * kHid * 2,
                   I_W1 = I_H2A + kRows * kHid * 2, I_W2 = I_W1 + kHid * kInP * 2, I_W3 = I_W2 + kHid * kHid * 2,
                   I_BIAS = I_W3 + kOutP * kHid * 2, I_MISC = I_BIAS + (kHid + kHid + kOutP) * 4,
                   kInferSmem = I_MISC + 64;
// at most 4 inference CTAs fit on an SM (228 KB of shared memory, 1 KB reserved
// per CTA), so their 4 x 128 tensor-memory columns never exceed the 512 an SM
// has and no allocation waits
constexpr uint32_t kInferSmemAlloc = 52 * 1024;
static_assert(kInferSmem <= kInferSmemAlloc, "inference smem");

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ void st_bf16(uint8_t *tile, uint32_t off, float v) {
  *reinterpret_cast<__nv_bfloat16 *>(tile + off) = __float2bfloat16_rn(v);
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
  __nv_bfloat162 p = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&p);
}

// row r of a K-major tile with C columns from C fp32 values (C a multiple of 8)
template <int C>
__device__ __forceinline__ void st_row(uint8_t *tile, int r, const float *v) {
#pragma unroll
  for (int cb = 0; cb < C / 8; ++cb) {
    uint4 q;
    q.x = pack2(v[cb * 8 + 0], v[cb * 8 + 1]);
    q.y = pack2(v[cb * 8 + 2], v[cb * 8 + 3]);
    q.z = pack2(v[cb * 8 + 4], v[cb * 8 + 5]);
    q.w = pack2(v[cb * 8 + 6], v[cb * 8 + 7]);
    *reinterpret_cast<uint4 *>(tile + tc05::tile_off(r, cb * 8, C)) = q;
  }
}

__device__ __forceinline__ float sigmoid_(float z) { return 1.f / (1.f + expf(-z)); }

// generic-proxy smem writes -> tensor cores, tensor-memory reads -> next MMA
__device__ __forceinline__ void sync_for_mma() {
  tc05::fence_smem_async();
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
}

// CTA-uniform bounded wait for the next completion of the CTA's MMA barrier
// (on a timeout the phase is left pending, so the caller can wait for it again
// before it frees the tensor memory)
__device__ __forceinline__ bool wait_mma(uint64_t *mbar, uint32_t &phase) {
  const bool ok = tc05::mbar_wait(mbar, phase, kWaitLimit);
  tc05::fence_after();
  const bool all = __syncthreads_and(ok ? 1 : 0) != 0;
  if (all) phase ^= 1u;
  return all;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct TrainArgs {
  const float *params;
  const float *x, *y;
  int64_t n;
  float *partials;     // [gridDim.x][kPartial]
  const int64_t *step;  // Adam steps taken
  uint64_t seed;
  int ntiles, tiles_per_cta;
  int random_rows;  // 1: rows drawn by hash; 0: rows tile*128 + t
  float inv_count;  // 1 / (batch * kOut)
  int32_t *err;
};

__global__ void __launch_bounds__(kRows, 1) k_train(TrainArgs a) {
  extern __shared__ __align__(1024) uint8_t sm[];
  using namespace tc05;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint8_t *XA = sm + S_XA, *H1A = sm + S_H1A, *H2A = sm + S_H2A, *DYA = sm + S_DYA, *DZ2A = sm + S_DZ2A;
  uint8_t *W1 = sm + S_W1, *W2 = sm + S_W2, *W3 = sm + S_W3, *W3T = sm + S_W3T, *W2T = sm + S_W2T;
  uint8_t *AT = sm + S_AT, *BT1 = sm + S_BT1, *BT2 = sm + S_BT2;
  float *b1 = reinterpret_cast<float *>(sm + S_BIAS), *b2 = b1 + kHid, *b3 = b2 + kHid;
  float *red = reinterpret_cast<float *>(sm + S_RED);
  float *ds1 = reinterpret_cast<float *>(sm + S_DS1);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + S_MISC);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + S_MISC + 8);
  const float *P = a.params;

  // weights -> bf16 operand tiles (forward and transposed for the backward pass)
  for (int e = tid; e < kHid * kInP; e += kRows) st_bf16(W1, tile_off(e / kInP, e % kInP, kInP), P[OW1 + e]);
  for (int e = tid; e < kHid * kHid; e += kRows) {
    const int o = e / kHid, i = e % kHid;
    const float w = P[OW2 + e];
    st_bf16(W2, tile_off(o, i, kHid), w);
    st_bf16(W2T, tile_off(i, o, kHid), w);
  }
  for (int e = tid; e < kOutP * kHid; e += kRows) {
    const int o = e / kHid, h = e % kHid;
    const float w = P[OW3 + e];
    st_bf16(W3, tile_off(o, h, kHid), w);
    st_bf16(W3T, tile_off(h, o, kOutP), w);
  }
  if (tid < kHid) { b1[tid] = P[OB1 + tid]; b2[tid] = P[OB2 + tid]; }
  if (tid < kOutP) b3[tid] = P[OB3 + tid];
  for (int e = tid; e < 4 * kRedW; e += kRows) red[e] = 0.f;
  if (tid == 0) mbar_init(mbar, 1);
  if (warp == 0) tmem_alloc(tslot, 256);
  sync_for_mma();
  const uint32_t tm = *tslot;
  // tensor-memory columns: [0,64) D1 then dH1, [64,128) D2 then dH2, [128,144) D3,
  // [144,224) weight gradients W3^T | W2, [224,240) W1
  const uint32_t tl = tm + ((uint32_t)(warp * 32) << 16);  // this warp's lane quadrant
  uint32_t phase = 0;
  bool ok = true;
  const int64_t step = *a.step;
  const uint32_t id64 = idesc_bf16(128, 64), id16 = idesc_bf16(128, 16), id80 = idesc_bf16(128, 80);
  const uint32_t sXA = smem_u32(XA), sH1A = smem_u32(H1A), sH2A = smem_u32(H2A), sDYA = smem_u32(DYA),
                 sDZ2A = smem_u32(DZ2A), sW1 = smem_u32(W1), sW2 = smem_u32(W2), sW3 = smem_u32(W3),
                 sW3T = smem_u32(W3T), sW2T = smem_u32(W2T), sAT = smem_u32(AT), sBT1 = smem_u32(BT1),
                 sBT2 = smem_u32(BT2);
  float* rw = red + warp * kRedW;

  for (int it = 0; it < a.tiles_per_cta && ok; ++it) {
    const int tile = blockIdx.x * a.tiles_per_cta + it;
    if (tile >= a.ntiles) break;
    const int64_t slot = (int64_t)tile * kRows + tid;
    const int64_t row =
        a.random_rows ? (int64_t)(mix64(a.seed ^ mix64((uint64_t)step * 0x100000001ull + (uint64_t)slot)) %
                                  (uint64_t)a.n)
                      : slot;
    float x[kInP], t[kOut];
#pragma unroll
    for (int j = 0; j < kInP; ++j) x[j] = j < kIn ? a.x[row * kIn + j] : 0.f;
#pragma unroll
    for (int o = 0; o < kOut; ++o) t[o] = a.y[row * kOut + o];
    st_row<kInP>(XA, tid, x);
#pragma unroll
    for (int j = 0; j < kInP; ++j) st_bf16(BT2, tile_off(j, tid, kRows), x[j]);
    sync_for_mma();

    // layer 1: D1 = X W1^T
    if (tid == 0) {
      mma_bf16(tm + 0, tile_desc(sXA, kInP, 0, 0), tile_desc(sW1, kInP, 0, 0), id64, 0);
      commit(mbar);
    }
    ok = wait_mma(mbar, phase);
    if (!ok) break;
    float z2[kHid];
    {
      float h[kHid];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float v[16];
        tmem_ld16(tl + 0 + c * 16, v);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const float z = v[q] + b1[c * 16 + q], sg = sigmoid_(z);
          h[c * 16 + q] = z * sg;
          ds1[(c * 16 + q) * kRows + tid] = sg * (1.f + z * (1.f - sg));
        }
      }
      st_row<kHid>(H1A, tid, h);
#pragma unroll
      for (int i = 0; i < kHid; ++i) st_bf16(BT1, tile_off(16 + i, tid, kRows), h[i]);
    }
    sync_for_mma();
    // layer 2: D2 = H1 W2^T
    if (tid == 0) {
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) mma_bf16(tm + 64, tile_desc(sH1A, kHid, 0, ks), tile_desc(sW2, kHid, 0, ks), id64, ks);
      commit(mbar);
    }
    ok = wait_mma(mbar, phase);
    if (!ok) break;
    {
      float h[kHid];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float v[16];
        tmem_ld16(tl + 64 + c * 16, v);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          z2[c * 16 + q] = v[q] + b2[c * 16 + q];
          h[c * 16 + q] = z2[c * 16 + q] * sigmoid_(z2[c * 16 + q]);
        }
      }
      st_row<kHid>(H2A, tid, h);
#pragma unroll
      for (int i = 0; i < kHid; ++i) st_bf16(AT, tile_off(i, tid, kRows), h[i]);
    }
    sync_for_mma();
    // layer 3: D3 = H2 W3^T
    if (tid == 0) {
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) mma_bf16(tm + 128, tile_desc(sH2A, kHid, 0, ks), tile_desc(sW3, kHid, 0, ks), id16, ks);
      commit(mbar);
    }
    ok = wait_mma(mbar, phase);
    if (!ok) break;
    {
      float v[16], dy[kOutP];
      tmem_ld16(tl + 128, v);
      float l2 = 0.f;
#pragma unroll
      for (int o = 0; o < kOutP; ++o) {
        if (o < kOut) {
          const float r = v[o] + b3[o] - t[o];
          l2 += r * r;
          dy[o] = 2.f * r * a.inv_count;
        } else {
          dy[o] = 0.f;
        }
      }
      st_row<kOutP>(DYA, tid, dy);
#pragma unroll
      for (int o = 0; o < kOutP; ++o) st_bf16(BT1, tile_off(o, tid, kRows), dy[o]);
      // bias gradient of layer 3 and the loss (fixed-order warp sums)
#pragma unroll
      for (int o = 0; o < kOut; ++o) {
        const float s = warp_sum(dy[o]);
        if (lane == 0) rw[128 + o] += s;
      }
      const float s = warp_sum(l2);
      if (lane == 0) rw[132] += s;
    }
    sync_for_mma();
    // dH2 = dY W3
    if (tid == 0) {
      mma_bf16(tm + 64, tile_desc(sDYA, kOutP, 0, 0), tile_desc(sW3T, kOutP, 0, 0), id64, 0);
      commit(mbar);
    }
    ok = wait_mma(mbar, phase);
    if (!ok) break;
    {
      float dz[kHid];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float v[16];
        tmem_ld16(tl + 64 + c * 16, v);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const float z = z2[c * 16 + q], sg = sigmoid_(z);
          dz[c * 16 + q] = v[q] * sg * (1.f + z * (1.f - sg));
        }
      }
      st_row<kHid>(DZ2A, tid, dz);
#pragma unroll
      for (int i = 0; i < kHid; ++i) st_bf16(AT, tile_off(64 + i, tid, kRows), dz[i]);
#pragma unroll
      for (int i = 0; i < kHid; ++i) {
        const float s = warp_sum(dz[i]);
        if (lane == 0) rw[64 + i] += s;
      }
    }
    sync_for_mma();
    // dH1 = dZ2 W2
    if (tid == 0) {
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) mma_bf16(tm + 0, tile_desc(sDZ2A, kHid, 0, ks), tile_desc(sW2T, kHid, 0, ks), id64, ks);
      commit(mbar);
    }
    ok = wait_mma(mbar, phase);
    if (!ok) break;
    {
      float dz[kHid];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float v[16];
        tmem_ld16(tl + 0 + c * 16, v);
#pragma unroll
        for (int q = 0; q < 16; ++q) dz[c * 16 + q] = v[q] * ds1[(c * 16 + q) * kRows + tid];
      }
#pragma unroll
      for (int i = 0; i < kHid; ++i) st_bf16(AT, tile_off(128 + i, tid, kRows), dz[i]);
#pragma unroll
      for (int i = 0; i < kHid; ++i) {
        const float s = warp_sum(dz[i]);
        if (lane == 0) rw[i] += s;
      }
    }
    sync_for_mma();
    // weight gradients, accumulated over the CTA's tiles (K = the 128 samples)
    if (tid == 0) {
#pragma unroll
      for (int ks = 0; ks < 8; ++ks)
        mma_bf16(tm + 144, tile_desc(sAT, kRows, 0, ks), tile_desc(sBT1, kRows, 0, ks), id80, (it > 0 || ks > 0) ? 1u : 0u);
#pragma unroll
      for (int ks = 0; ks < 8; ++ks)
        mma_bf16(tm + 224, tile_desc(sAT, kRows, 64, ks), tile_desc(sBT2, kRows, 0, ks), id16, (it > 0 || ks > 0) ? 1u : 0u);
      commit(mbar);
    }
    ok = wait_mma(mbar, phase);  // the operand tiles are rewritten by the next tile
  }

  if (ok) {
    float *out = a.partials + (size_t)blockIdx.x * kPartial;
    float v[16];
    if (warp < 2) {  // lanes 0-63: dW3^T[h][o]
      tmem_ld16(tl + 144, v);
#pragma unroll
      for (int o = 0; o < kOutP; ++o) out[OW3 + o * kHid + tid] = o < kOut ? v[o] : 0.f;
    } else {  // lanes 64-127: dW2[o][*], dW1[o][*]
      const int o = tid - 64;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        tmem_ld16(tl + 160 + c * 16, v);
#pragma unroll
        for (int q = 0; q < 16; ++q) out[OW2 + o * kHid + c * 16 + q] = v[q];
      }
      tmem_ld16(tl + 224, v);
#pragma unroll
      for (int j = 0; j < kInP; ++j) out[OW1 + o * kInP + j] = j < kIn ? v[j] : 0.f;
    }
    __syncthreads();
    for (int q = tid; q < kHid; q += kRows) {
      out[OB1 + q] = ((red[q] + red[kRedW + q]) + red[2 * kRedW + q]) + red[3 * kRedW + q];
      out[OB2 + q] = ((red[64 + q] + red[kRedW + 64 + q]) + red[2 * kRedW + 64 + q]) + red[3 * kRedW + 64 + q];
    }
    if (tid < kOutP)
      out[OB3 + tid] = tid < kOut ? ((red[128 + tid] + red[kRedW + 128 + tid]) + red[2 * kRedW + 128 + tid]) +
                                        red[3 * kRedW + 128 + tid]
                                  : 0.f;
    if (tid == 0) out[kNParam] = ((red[132] + red[kRedW + 132]) + red[2 * kRedW + 132]) + red[3 * kRedW + 132];
  } else {
    if (tid == 0) atomicOr(a.err, pstep::kErrTimeout);
    tc05::mbar_wait(mbar, phase, kWaitLimit);  // MMAs possibly still in flight
  }
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  if (warp == 0) tmem_dealloc(tm, 256);
}

// partial gradients -> gradient (CTA order), then Adam; one block
__global__ void __launch_bounds__(1024) k_adam(float *__restrict__ P, float *__restrict__ m, float *__restrict__ v,
                                               const float *__restrict__ partials, int ncta, int64_t *step, float lr,
                                               float inv_count, float *__restrict__ loss_hist, int64_t t0,
                                               float *__restrict__ grad_out) {
  const int64_t t = *step + 1;
  const float bc1 = 1.f - powf(0.9f, (float)t), bc2 = 1.f - powf(0.999f, (float)t);
  for (int p = threadIdx.x; p < kNParam; p += blockDim.x) {
    float g = 0.f;
    for (int c = 0; c < ncta; ++c) g += partials[(size_t)c * kPartial + p];
    if (grad_out) {
      grad_out[p] = g;
      continue;
    }
    const float mn = 0.9f * m[p] + 0.1f * g;
    const float vn = 0.999f * v[p] + 0.001f * g * g;
    m[p] = mn;
    v[p] = vn;
    P[p] -= lr * (mn / bc1) / (sqrtf(vn / bc2) + 1e-8f);
  }
  if (threadIdx.x == 0) {
    float l = 0.f;
    for (int c = 0; c < ncta; ++c) l += partials[(size_t)c * kPartial + kNParam];
    l *= inv_count;
    if (grad_out) grad_out[kNParam] = l;
    else if (loss_hist) loss_hist[t - 1 - t0] = l;
  }
  __syncthreads();
  if (threadIdx.x == 0 && !grad_out) *step = t;
}

// forward pass for n rows, one tile of 128 rows per CTA
__global__ void __launch_bounds__(kRows) k_infer(const float *__restrict__ P, const float *__restrict__ xin, int64_t n,
                                                 float *__restrict__ yout, int32_t *err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  using namespace tc05;
  const int tid = threadIdx.x, warp = tid >> 5;
  uint8_t *XA = sm + I_XA, *H1A = sm + I_H1A, *H2A = sm + I_H2A, *W1 = sm + I_W1, *W2 = sm + I_W2, *W3 = sm + I_W3;
  float *b1 = reinterpret_cast<float *>(sm + I_BIAS), *b2 = b1 + kHid, *b3 = b2 + kHid;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + I_MISC);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + I_MISC + 8);
  for (int e = tid; e < kHid * kInP; e += kRows) st_bf16(W1, tile_off(e / kInP, e % kInP, kInP), P[OW1 + e]);
  for (int e = tid; e < kHid * kHid; e += kRows) st_bf16(W2, tile_off(e / kHid, e % kHid, kHid), P[OW2 + e]);
  for (int e = tid; e < kOutP * kHid; e += kRows) st_bf16(W3, tile_off(e / kHid, e % kHid, kHid), P[OW3 + e]);
  if (tid < kHid) { b1[tid] = P[OB1 + tid]; b2[tid] = P[OB2 + tid]; }
  if (tid < kOutP) b3[tid] = P[OB3 + tid];
  if (tid == 0) mbar_init(mbar, 1);
  if (warp == 0) tmem_alloc(tslot, 128);
  const int64_t row = (int64_t)blockIdx.x * kRows + tid;
  const bool live = row < n;
  float x[kInP];
#pragma unroll
  for (int j = 0; j < kInP; ++j) x[j] = (live && j < kIn) ? xin[row * kIn + j] : 0.f;
  st_row<kInP>(XA, tid, x);
  sync_for_mma();
  const uint32_t tm = *tslot;
  const uint32_t tl = tm + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  bool ok;
  if (tid == 0) {
    mma_bf16(tm, tile_desc(smem_u32(XA), kInP, 0, 0), tile_desc(smem_u32(W1), kInP, 0, 0), idesc_bf16(128, 64), 0);
    commit(mbar);
  }
  ok = wait_mma(mbar, phase);
  if (ok) {
    float h[kHid];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float v[16];
      tmem_ld16(tl + c * 16, v);
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const float z = v[q] + b1[c * 16 + q];
        h[c * 16 + q] = z * sigmoid_(z);
      }
    }
    st_row<kHid>(H1A, tid, h);
    sync_for_mma();
    if (tid == 0) {
#pragma unroll
      for (int ks = 0; ks < 4; ++ks)
        mma_bf16(tm + 64, tile_desc(smem_u32(H1A), kHid, 0, ks), tile_desc(smem_u32(W2), kHid, 0, ks), idesc_bf16(128, 64), ks);
      commit(mbar);
    }
    ok = wait_mma(mbar, phase);
  }
  if (ok) {
    float h[kHid];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float v[16];
      tmem_ld16(tl + 64 + c * 16, v);
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const float z = v[q] + b2[c * 16 + q];
        h[c * 16 + q] = z * sigmoid_(z);
      }
    }
    st_row<kHid>(H2A, tid, h);
    sync_for_mma();
    if (tid == 0) {  // D3 reuses columns [0,16): D1 has been read
#pragma unroll
      for (int ks = 0; ks < 4; ++ks)
        mma_bf16(tm, tile_desc(smem_u32(H2A), kHid, 0, ks), tile_desc(smem_u32(W3), kHid, 0, ks), idesc_bf16(128, 16), ks);
      commit(mbar);
    }
    ok = wait_mma(mbar, phase);
  }
  if (ok) {
    float v[16];
    tmem_ld16(tl, v);
    if (live) {
#pragma unroll
      for (int o = 0; o < kOut; ++o) yout[row * kOut + o] = v[o] + b3[o];
    }
  } else {
    if (tid == 0) atomicOr(err, pstep::kErrTimeout);
    tc05::mbar_wait(mbar, phase, kWaitLimit);
  }
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  if (warp == 0) tmem_dealloc(tm, 128);
}

}  // namespace pmlp

struct pmlp_ctx {
  int device;
  cudaStream_t stream;
  float *P, *m, *v, *partials, *x, *y, *grad, *loss_hist, *tmp_x, *tmp_y;
  int64_t *step;
  int32_t *err;
  int64_t n, loss_cap, steps_done, launches, partial_cap, tmp_cap;
  int num_sms;
  char msg[256];
};

namespace {

using namespace pmlp;

int fail(pmlp_ctx *h, int code, const char *what, cudaError_t e = cudaSuccess) {
  if (h) {
    if (e != cudaSuccess) snprintf(h->msg, sizeof h->msg, "%s: %s", what, cudaGetErrorString(e));
    else snprintf(h->msg, sizeof h->msg, "%s", what);
  }
  cudaGetLastError();
  return code;
}

#define MCUDA(h, x)                                          \
  do {                                                       \
    cudaError_t e_ = (x);                                    \
    if (e_ != cudaSuccess) return fail(h, PSTEP_ERR_CUDA, #x, e_); \
  } while (0)

template <typename T>
int dalloc(pmlp_ctx *h, T *&p, size_t count) {
  p = nullptr;
  cudaError_t e = cudaMalloc((void **)&p, sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess) {
    p = nullptr;
    return fail(h, PSTEP_ERR_NOMEM, "cudaMalloc", e);
  }
  return PSTEP_OK;
}
template <typename T>
void dfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

#define MTRY(x)                        \
  do {                                 \
    int rc_ = (x);                     \
    if (rc_ != PSTEP_OK) return rc_;   \
  } while (0)

uint64_t host_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// default linear-layer initialisation: U(-1/sqrt(fan_in), 1/sqrt(fan_in)), padding zero
void init_params(uint64_t seed, float *P) {
  memset(P, 0, sizeof(float) * kNParam);
  uint64_t s = seed;
  auto uni = [&](float bound) {
    s = host_mix(s);
    const double u = (double)(s >> 11) * (1.0 / 9007199254740992.0);
    return (float)((2.0 * u - 1.0) * bound);
  };
  const float a1 = 1.f / sqrtf((float)kIn), a2 = 1.f / sqrtf((float)kHid);
  for (int o = 0; o < kHid; ++o)
    for (int j = 0; j < kIn; ++j) P[OW1 + o * kInP + j] = uni(a1);
  for (int o = 0; o < kHid; ++o) P[OB1 + o] = uni(a1);
  for (int e = 0; e < kHid * kHid; ++e) P[OW2 + e] = uni(a2);
  for (int o = 0; o < kHid; ++o) P[OB2 + o] = uni(a2);
  for (int o = 0; o < kOut; ++o)
    for (int h = 0; h < kHid; ++h) P[OW3 + o * kHid + h] = uni(a2);
  for (int o = 0; o < kOut; ++o) P[OB3 + o] = uni(a2);
}

int check_err(pmlp_ctx *h) {
  int32_t e = 0;
  MCUDA(h, cudaMemcpyAsync(&e, h->err, sizeof e, cudaMemcpyDeviceToHost, h->stream));
  MCUDA(h, cudaStreamSynchronize(h->stream));
  if (e & pstep::kErrTimeout) return fail(h, PSTEP_ERR_TIMEOUT, "tensor-core completion wait ran out");
  return PSTEP_OK;
}

int ensure_partials(pmlp_ctx *h, int64_t ncta) {
  if (ncta <= h->partial_cap) return PSTEP_OK;
  dfree(h->partials);
  MTRY(dalloc(h, h->partials, (size_t)ncta * kPartial));
  h->partial_cap = ncta;
  return PSTEP_OK;
}

// one optimisation step (or, with grad_out, the gradient only): two launches
void launch_step(pmlp_ctx *h, const TrainArgs &a, int ncta, float lr, int64_t t0, float *grad_out) {
  k_train<<<ncta, kRows, kTrainSmem, h->stream>>>(a);
  k_adam<<<1, 1024, 0, h->stream>>>(h->P, h->m, h->v, h->partials, ncta, h->step, lr, a.inv_count, h->loss_hist, t0,
                                    grad_out);
  h->launches += 2;
}

int prepare_batch(pmlp_ctx *h, int batch, TrainArgs &a, int &ncta) {
  if (batch <= 0 || batch % kRows != 0) return fail(h, PSTEP_ERR_ARG, "batch must be a positive multiple of 128");
  if (!h->x || h->n <= 0) return fail(h, PSTEP_ERR_STATE, "no training data (pmlp_set_data)");
  const int ntiles = batch / kRows;
  const int max_cta = h->num_sms > 0 ? h->num_sms : 148;
  const int tpc = (ntiles + max_cta - 1) / max_cta;
  ncta = (ntiles + tpc - 1) / tpc;
  MTRY(ensure_partials(h, ncta));
  a.params = h->P;
  a.x = h->x;
  a.y = h->y;
  a.n = h->n;
  a.partials = h->partials;
  a.step = h->step;
  a.seed = 0;
  a.ntiles = ntiles;
  a.tiles_per_cta = tpc;
  a.random_rows = 1;
  a.inv_count = 1.f / ((float)batch * kOut);
  a.err = h->err;
  return PSTEP_OK;
}

}  // namespace

extern "C" {

int pmlp_create(uint64_t seed, pmlp_handle *out) {
  if (!out) return PSTEP_ERR_ARG;
  *out = nullptr;
  pmlp_ctx *h = new pmlp_ctx();
  memset((void *)h, 0, sizeof(pmlp_ctx));
  if (cudaGetDevice(&h->device) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return PSTEP_ERR_CUDA;
  }
  int major = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, h->device);
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  if (major < 10) {
    delete h;
    return PSTEP_ERR_CUDA;  // tcgen05 needs a Blackwell-class GPU
  }
  int rc = PSTEP_OK;
  if ((rc = dalloc(h, h->P, kNParam)) || (rc = dalloc(h, h->m, kNParam)) || (rc = dalloc(h, h->v, kNParam)) ||
      (rc = dalloc(h, h->grad, kNParam + 4)) || (rc = dalloc(h, h->step, 1)) || (rc = dalloc(h, h->err, 1))) {
    pmlp_destroy(h);
    return rc;
  }
  if (cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem) != cudaSuccess ||
      cudaFuncSetAttribute(k_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmemAlloc) !=
          cudaSuccess) {
    cudaGetLastError();
    pmlp_destroy(h);
    return PSTEP_ERR_CUDA;
  }
  float *host = (float *)malloc(sizeof(float) * kNParam);
  init_params(seed, host);
  rc = pmlp_set_params(h, host);
  free(host);
  if (rc != PSTEP_OK) {
    pmlp_destroy(h);
    return rc;
  }
  *out = h;
  return PSTEP_OK;
}

int pmlp_destroy(pmlp_handle h) {
  if (!h) return PSTEP_ERR_ARG;
  if (h->stream) cudaStreamSynchronize(h->stream);
  else cudaDeviceSynchronize();
  dfree(h->P); dfree(h->m); dfree(h->v); dfree(h->partials); dfree(h->x); dfree(h->y); dfree(h->grad);
  dfree(h->loss_hist); dfree(h->step); dfree(h->err); dfree(h->tmp_x); dfree(h->tmp_y);
  delete h;
  return PSTEP_OK;
}

int pmlp_set_stream(pmlp_handle h, void *stream) {
  if (!h) return PSTEP_ERR_ARG;
  h->stream = (cudaStream_t)stream;
  return PSTEP_OK;
}

int pmlp_get_params(pmlp_handle h, float *dst) {
  if (!h || !dst) return PSTEP_ERR_ARG;
  MCUDA(h, cudaMemcpyAsync(dst, h->P, sizeof(float) * kNParam, cudaMemcpyDeviceToHost, h->stream));
  MCUDA(h, cudaStreamSynchronize(h->stream));
  return PSTEP_OK;
}

int pmlp_set_params(pmlp_handle h, const float *src) {
  if (!h || !src) return PSTEP_ERR_ARG;
  MCUDA(h, cudaMemcpyAsync(h->P, src, sizeof(float) * kNParam, cudaMemcpyHostToDevice, h->stream));
  MCUDA(h, cudaMemsetAsync(h->m, 0, sizeof(float) * kNParam, h->stream));
  MCUDA(h, cudaMemsetAsync(h->v, 0, sizeof(float) * kNParam, h->stream));
  MCUDA(h, cudaMemsetAsync(h->step, 0, sizeof(int64_t), h->stream));
  MCUDA(h, cudaMemsetAsync(h->err, 0, sizeof(int32_t), h->stream));
  MCUDA(h, cudaStreamSynchronize(h->stream));
  h->steps_done = 0;
  return PSTEP_OK;
}

int pmlp_set_data(pmlp_handle h, const float *x, const float *y, int64_t n, int on_device) {
  if (!h || !x || !y || n <= 0) return PSTEP_ERR_ARG;
  dfree(h->x);
  dfree(h->y);
  h->n = 0;
  MTRY(dalloc(h, h->x, (size_t)n * kIn));
  MTRY(dalloc(h, h->y, (size_t)n * kOut));
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  MCUDA(h, cudaMemcpyAsync(h->x, x, sizeof(float) * n * kIn, kind, h->stream));
  MCUDA(h, cudaMemcpyAsync(h->y, y, sizeof(float) * n * kOut, kind, h->stream));
  MCUDA(h, cudaStreamSynchronize(h->stream));
  h->n = n;
  return PSTEP_OK;
}

int pmlp_train(pmlp_handle h, int64_t steps, int batch, float lr, uint64_t seed, float *loss) {
  if (!h || steps < 0) return PSTEP_ERR_ARG;
  if (!(lr > 0.f)) return fail(h, PSTEP_ERR_ARG, "learning rate must be positive");
  TrainArgs a;
  int ncta = 0;
  MTRY(prepare_batch(h, batch, a, ncta));
  a.seed = seed;
  if (steps == 0) return PSTEP_OK;
  if (steps > h->loss_cap) {
    dfree(h->loss_hist);
    MTRY(dalloc(h, h->loss_hist, (size_t)steps));
    h->loss_cap = steps;
  }
  const int64_t t0 = h->steps_done;
  // whole chunks of steps as one CUDA graph (the step counter is on the device)
  const int64_t chunk = 50;
  int64_t done = 0;
  if (steps >= chunk) {
    cudaStream_t cs = nullptr;
    MCUDA(h, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaStream_t keep = h->stream;
    MCUDA(h, cudaStreamSynchronize(keep));
    h->stream = cs;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      for (int64_t s = 0; s < chunk; ++s) launch_step(h, a, ncta, lr, t0, nullptr);
      e = cudaStreamEndCapture(cs, &g);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
    for (int64_t c = 0; e == cudaSuccess && c + chunk <= steps; c += chunk) {
      e = cudaGraphLaunch(ge, cs);
      done += chunk;
    }
    h->launches -= 2 * chunk;  // the captured launches were counted once; count replays
    h->launches += 2 * done;
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    cudaError_t e2 = cudaStreamSynchronize(cs);
    cudaStreamDestroy(cs);
    h->stream = keep;
    if (e != cudaSuccess) return fail(h, PSTEP_ERR_CUDA, "training graph", e);
    if (e2 != cudaSuccess) return fail(h, PSTEP_ERR_CUDA, "training graph", e2);
  }
  for (; done < steps; ++done) launch_step(h, a, ncta, lr, t0, nullptr);
  MCUDA(h, cudaGetLastError());
  MTRY(check_err(h));
  h->steps_done += steps;
  if (loss) {
    MCUDA(h, cudaMemcpyAsync(loss, h->loss_hist, sizeof(float) * steps, cudaMemcpyDeviceToHost, h->stream));
    MCUDA(h, cudaStreamSynchronize(h->stream));
  }
  return PSTEP_OK;
}

int pmlp_gradient(pmlp_handle h, int batch, float *grad, float *loss) {
  if (!h || !grad) return PSTEP_ERR_ARG;
  TrainArgs a;
  int ncta = 0;
  MTRY(prepare_batch(h, batch, a, ncta));
  if (batch > h->n) return fail(h, PSTEP_ERR_ARG, "batch larger than the training set");
  a.random_rows = 0;
  launch_step(h, a, ncta, 1.f, 0, h->grad);
  MCUDA(h, cudaGetLastError());
  MTRY(check_err(h));
  float tmp[kNParam + 1];
  MCUDA(h, cudaMemcpyAsync(tmp, h->grad, sizeof(float) * (kNParam + 1), cudaMemcpyDeviceToHost, h->stream));
  MCUDA(h, cudaStreamSynchronize(h->stream));
  memcpy(grad, tmp, sizeof(float) * kNParam);
  if (loss) *loss = tmp[kNParam];
  return PSTEP_OK;
}

int pmlp_forward(pmlp_handle h, const float *x, int64_t n, float *y, int on_device) {
  if (!h || !x || !y || n < 0) return PSTEP_ERR_ARG;
  if (n == 0) return PSTEP_OK;
  const float *dx = x;
  float *dy = y;
  if (!on_device) {
    if (n > h->tmp_cap) {
      dfree(h->tmp_x);
      dfree(h->tmp_y);
      h->tmp_cap = 0;
      MTRY(dalloc(h, h->tmp_x, (size_t)n * kIn));
      MTRY(dalloc(h, h->tmp_y, (size_t)n * kOut));
      h->tmp_cap = n;
    }
    MCUDA(h, cudaMemcpyAsync(h->tmp_x, x, sizeof(float) * n * kIn, cudaMemcpyHostToDevice, h->stream));
    dx = h->tmp_x;
    dy = h->tmp_y;
  }
  const int64_t blocks = (n + kRows - 1) / kRows;
  k_infer<<<(unsigned)blocks, kRows, kInferSmemAlloc, h->stream>>>(h->P, dx, n, dy, h->err);
  h->launches += 1;
  MCUDA(h, cudaGetLastError());
  if (!on_device)
    MCUDA(h, cudaMemcpyAsync(y, dy, sizeof(float) * n * kOut, cudaMemcpyDeviceToHost, h->stream));
  MTRY(check_err(h));
  return PSTEP_OK;
}

int64_t pmlp_steps(pmlp_handle h) { return h ? h->steps_done : -1; }
int64_t pmlp_launch_count(pmlp_handle h) { return h ? h->launches : -1; }
const char *pmlp_last_error(pmlp_handle h) { return h ? h->msg : "null handle"; }

}  // extern "C"

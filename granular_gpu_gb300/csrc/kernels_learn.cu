// kernels_learn.cu — the learned warm start: per-particle features, a
// 48 -> 64 -> 64 -> 3 MLP run on the 5th-generation tensor cores (tcgen05,
// BF16 operands in shared memory, FP32 accumulators in tensor memory), its
// training step (forward, backward and weight gradients on the tensor cores,
// Adam on the CUDA cores) and the application of its prediction to x*.
//
// The network predicts the Jacobi position correction of a substep, the
// displacement x*_final - x*_predict that the plain sweeps would reach, in
// units of |g| dt^2, from features of the particle's neighbourhood at x*.
// The plain sweeps always run afterwards, so the prediction only changes
// where they start.
//
// Tile shape: 128 particles per tile (the M = 128 MMA shape, one particle per
// TMEM lane); a CTA of 128 threads (one warpgroup) walks tiles persistently.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "tc_ptx.cuh"

namespace gg {

// ------------------------------------------------------------ layout

constexpr int kFeat = 48, kHid = 64, kOut = 3;
constexpr int kTile = 128;
// fp32 parameter vector: W1[48][64] b1[64] W2[64][64] b2[64] W3[64][3] b3[3]
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kFeat * kHid, kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid * kHid,
              kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid * kOut, kNParams = kOffB3 + kOut;
static_assert(kNParams == 7491, "parameter count");

// Packed BF16 operand tiles of the weights (canonical layout, tc_ptx.cuh),
// byte offsets in one buffer that a CTA copies to shared memory at once.
//   B1  forward layer 1: N = 64 (out) x K = 48 (in), (n, k) = W1[k][n]
//   B2  forward layer 2: N = 64 x K = 64,           (n, k) = W2[k][n]
//   B3  forward layer 3: N = 16 (3 used) x K = 64,  (n, k) = W3[k][n]
//   B2b backward dH1 = dH2 W2^T: N = 64 (h1) x K = 64 (h2), (n, k) = W2[n][k]
//   B3b backward dH2 = dY W3^T:  N = 64 (h2) x K = 16 (3 used), (n, k) = W3[n][k]
constexpr int kPB1 = 0, kPB2 = kPB1 + 64 * 48 * 2, kPB3 = kPB2 + 64 * 64 * 2, kPB2b = kPB3 + 16 * 64 * 2,
              kPB3b = kPB2b + 64 * 64 * 2, kPackBytes = kPB3b + 64 * 16 * 2;
static_assert(kPackBytes == 26624, "packed weight bytes");

__device__ __forceinline__ uint16_t bf16_bits(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float bf16_val(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// One thread per packed bf16 element.
__global__ void k_pack_weights(const float* __restrict__ P, uint8_t* __restrict__ pack) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  int e = t;
  auto put = [&](int base, int rows, int n, int k, float v) {
    *reinterpret_cast<uint16_t*>(pack + base + ((k >> 3) * rows * 16 + n * 16 + (k & 7) * 2)) = bf16_bits(v);
  };
  if (e < 64 * 48) { const int n = e / 48, k = e % 48; put(kPB1, 64, n, k, P[kOffW1 + k * kHid + n]); return; }
  e -= 64 * 48;
  if (e < 64 * 64) { const int n = e / 64, k = e % 64; put(kPB2, 64, n, k, P[kOffW2 + k * kHid + n]); return; }
  e -= 64 * 64;
  if (e < 16 * 64) {
    const int n = e / 64, k = e % 64;
    put(kPB3, 16, n, k, n < kOut ? P[kOffW3 + k * kOut + n] : 0.0f);
    return;
  }
  e -= 16 * 64;
  if (e < 64 * 64) { const int n = e / 64, k = e % 64; put(kPB2b, 64, n, k, P[kOffW2 + n * kHid + k]); return; }
  e -= 64 * 64;
  if (e < 64 * 16) {
    const int n = e / 16, k = e % 16;
    put(kPB3b, 64, n, k, k < kOut ? P[kOffW3 + n * kOut + k] : 0.0f);
  }
}
constexpr int kPackElems = kPackBytes / 2;

// ------------------------------------------------------------ features

struct FeatArgs {
  Grid g;
  int n;
  const float4* __restrict__ xs;   // x* after the predict (w = contact radius)
  const float4* __restrict__ pos;  // x at the start of the substep
  const float4* __restrict__ vel;
  const float* __restrict__ mass;
  const int32_t* __restrict__ cs;
  const int32_t* __restrict__ bcs;
  const float4* __restrict__ bpos;
  __nv_bfloat16* __restrict__ out;  // n x 48, row-major
  float inv_slen, inv_svel;         // 1 / (|g| dt^2), 1 / (|g| dt)
  float brad, minr;                 // wall particle radius, floor of r against walls
  float inv_height;                 // 1 / (ny L)
};

__device__ __forceinline__ float clampf(float x, float lim) { return fmaxf(-lim, fminf(x, lim)); }

// 48 features of particle i over the 27 cells around trunc(x*/L), the
// stencil the sweeps use; lengths in units of |g| dt^2, velocities in |g| dt.
__global__ void __launch_bounds__(256) k_features(FeatArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const Grid& g = a.g;
  const float4 x4 = a.xs[i];
  const float3 x = f3(x4);
  const float ri = x4.w;
  const float mi = a.mass[i];
  const float4 vi4 = a.vel[i];
  float f[kFeat];
#pragma unroll
  for (int k = 0; k < kFeat; ++k) f[k] = 0.0f;
  f[0] = 1.0f;
  const float4 p = a.pos[i];
  f[1] = (x.x - p.x) * a.inv_slen;
  f[2] = (x.y - p.y) * a.inv_slen;
  f[3] = (x.z - p.z) * a.inv_slen;
  f[4] = vi4.x * a.inv_svel;
  f[5] = vi4.y * a.inv_svel;
  f[6] = vi4.z * a.inv_svel;
  f[7] = mi;
  f[8] = ri / g.L;
  const float Bw = a.brad + fmaxf(ri, a.minr);
  const int3 q = trunc_cell(g, x);
  for_each_stencil_column(g, q, [&](int k0, int nc) {
    const int j1 = a.cs[k0 + nc];
    for (int j = a.cs[k0]; j < j1; ++j) {
      if (j == i) continue;
      const float4 xj = a.xs[j];
      const float dx = x.x - xj.x, dy = x.y - xj.y, dz = x.z - xj.z;
      const float R = ri + xj.w;
      const float d2 = dx * dx + dy * dy + dz * dz;
      const float Rn = 1.5f * R;
      if (!(d2 < Rn * Rn) || !(d2 > 0.0f)) continue;
      const float dis = sqrtf(d2);
      const float inv = 1.0f / dis;
      const float nx = dx * inv, ny = dy * inv, nz = dz * inv;
      const float ov = (R - dis) * a.inv_slen;
      const float ovp = fmaxf(ov, 0.0f);
      const float mj = a.mass[j];
      const float4 vj = a.vel[j];
      const float wm = mj / (mi + mj);
      f[10] += 1.0f;
      f[16] += nx; f[17] += ny; f[18] += nz;
      const float wl = 1.0f - dis / Rn;
      f[25] += wl * nx; f[26] += wl * ny; f[27] += wl * nz;
      f[32] += (vj.x - vi4.x) * a.inv_svel;
      f[33] += (vj.y - vi4.y) * a.inv_svel;
      f[34] += (vj.z - vi4.z) * a.inv_svel;
      if (ny > 0.5f) { f[28] += 1.0f; f[30] += ovp; }
      else if (ny < -0.5f) { f[29] += 1.0f; f[31] += ovp; }
      else { f[35] += ovp * nx; f[36] += ovp * ny; f[37] += ovp * nz; }
      if (ov >= 0.0f) {
        f[9] += 1.0f;
        f[11] += ovp;
        f[12] += ovp * nx; f[13] += ovp * ny; f[14] += ovp * nz;
        f[15] = fmaxf(f[15], ovp);
        f[19] += ovp * wm * nx; f[20] += ovp * wm * ny; f[21] += ovp * wm * nz;
        const float o2 = ovp * ovp * 0.125f;
        f[22] += o2 * nx; f[23] += o2 * ny; f[24] += o2 * nz;
      }
    }
    const int b1 = a.bcs[k0 + nc];
    for (int b = a.bcs[k0]; b < b1; ++b) {
      const float4 pb = a.bpos[b];
      const float dx = x.x - pb.x, dy = x.y - pb.y, dz = x.z - pb.z;
      const float d2 = dx * dx + dy * dy + dz * dz;
      const float Bn = 1.5f * Bw;
      if (!(d2 < Bn * Bn) || !(d2 > 0.0f)) continue;
      const float dis = sqrtf(d2);
      const float inv = 1.0f / dis;
      const float nx = dx * inv, ny = dy * inv, nz = dz * inv;
      f[43] += nx; f[44] += ny; f[45] += nz;
      const float ov = (Bw - dis) * a.inv_slen;
      if (ov >= 0.0f) {
        f[38] += 1.0f;
        f[39] += ov;
        f[40] += ov * nx; f[41] += ov * ny; f[42] += ov * nz;
      }
    }
  });
  f[46] = sqrtf(f[12] * f[12] + f[13] * f[13] + f[14] * f[14]);
  f[47] = x.y * a.inv_height;
  uint4* dst = reinterpret_cast<uint4*>(a.out + (size_t)i * kFeat);
#pragma unroll
  for (int c = 0; c < kFeat / 8; ++c) {
    uint32_t w[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const uint32_t lo = bf16_bits(clampf(f[8 * c + 2 * h], 256.0f));
      const uint32_t hi = bf16_bits(clampf(f[8 * c + 2 * h + 1], 256.0f));
      w[h] = lo | (hi << 16);
    }
    dst[c] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

}  // namespace gg

// ------------------------------------------------------------ MLP forward

namespace gg {

// Bounded mbarrier waits: the pipeline completes in microseconds; a wait
// that runs out records ERR_TIMEOUT and the kernel winds down.
constexpr uint32_t kWaitPolls = 1u << 20;

struct MlpArgs {
  int n;
  const uint8_t* __restrict__ pack;  // packed weights, kPackBytes
  const float* __restrict__ params;  // fp32 parameters (biases are read from here)
  float* __restrict__ y;             // n x 3 prediction (forward), or null
  float4* __restrict__ xs;           // apply: x* += scale_len * y
  const float4* __restrict__ pos;    // apply: x, for the displacement bound
  float scale_len;
  unsigned int* __restrict__ disp_bits;  // apply: max |x* - x| per axis (float bits)
  const float* __restrict__ target;  // training: n x 3
  float grad_scale;                  // training: 2 / (3 n), the mean squared error's factor
  float* __restrict__ grad;          // training: fp32 gradient (atomically accumulated)
  float* __restrict__ loss;          // training: sum of squared errors / (3 n)
  int* __restrict__ err;
};

// Forward shared-memory map (bytes, 1024-aligned blocks).
constexpr int kFwW = 0;                    // packed weights      26624
constexpr int kFwX = 27648;                // X tile 128 x 48     12288
constexpr int kFwH = kFwX + 12288;         // H tile 128 x 64     16384
constexpr int kFwB = kFwH + 16384;         // biases 131 floats     524
constexpr int kFwBar = kFwB + 528;         // 3 mbarriers            24
constexpr int kFwSlot = kFwBar + 24;       // TMEM base               4
constexpr int kFwSmem = kFwSlot + 8;

// Writes 16 consecutive activations (bias added, ReLU) of row r as bf16 into
// a canonical 128-row tile starting at column c0 (a multiple of 16).
__device__ __forceinline__ void store_act16(uint8_t* tile, int r, int c0, const float* v, const float* bias,
                                            bool relu) {
  uint32_t w[8];
#pragma unroll
  for (int h = 0; h < 8; ++h) {
    float a0 = v[2 * h] + bias[2 * h], a1 = v[2 * h + 1] + bias[2 * h + 1];
    if (relu) {
      a0 = fmaxf(a0, 0.0f);
      a1 = fmaxf(a1, 0.0f);
    }
    w[h] = (uint32_t)bf16_bits(a0) | ((uint32_t)bf16_bits(a1) << 16);
  }
  *reinterpret_cast<uint4*>(tile + tc::canon_off(r, c0, kTile)) = make_uint4(w[0], w[1], w[2], w[3]);
  *reinterpret_cast<uint4*>(tile + tc::canon_off(r, c0 + 8, kTile)) = make_uint4(w[4], w[5], w[6], w[7]);
}

// All threads: wait for a phase, then agree on success.  On success the
// phase flips; on failure the error word is set, the barrier and its phase
// are recorded for the wind-down, and the caller leaves its loop.
struct WaitState {
  uint64_t* bar = nullptr;
  uint32_t phase = 0;
};
__device__ __forceinline__ bool wait_all(uint64_t* bar, uint32_t& phase, int* err, WaitState& failed) {
  const bool mine = tc::mbar_wait(bar, phase, kWaitPolls);
  const bool ok = __syncthreads_and(mine) != 0;
  if (ok) {
    phase ^= 1u;
  } else {
    failed.bar = bar;
    failed.phase = phase;
    if (threadIdx.x == 0) atomicOr(err, ERR_TIMEOUT);
  }
  return ok;
}

// Wind-down after a failed wait: give the copy or MMA that did not complete
// one more bounded wait before the shared and tensor memory are released.
__device__ __forceinline__ void drain(const WaitState& failed) {
  if (failed.bar) tc::mbar_wait(failed.bar, failed.phase, kWaitPolls);
}

// Inference over the rows of X (n x 48 bf16 row-major, read through the
// tensor map `tmX`, box 8 columns x 128 rows).  kApply: add the prediction,
// scaled, to x*; else write it to y.
template <bool kApply>
__global__ void __launch_bounds__(kTile, 1) k_mlp_fwd(const __grid_constant__ CUtensorMap tmX, MlpArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sW = smem + kFwW;
  uint8_t* sX = smem + kFwX;
  uint8_t* sH = smem + kFwH;
  float* sB = reinterpret_cast<float*>(smem + kFwB);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kFwBar);
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + kFwSlot);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  if (t == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::mbar_init(&bars[2], 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(slot, 128);
  for (int k = t; k < 2 * kHid + kOut; k += kTile)
    sB[k] = k < kHid ? a.params[kOffB1 + k] : (k < 2 * kHid ? a.params[kOffB2 + k - kHid] : a.params[kOffB3 + k - 2 * kHid]);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  uint32_t ph_w = 0, ph_x = 0, ph_m = 0;
  WaitState failed;
  if (t == 0) {
    tc::mbar_arrive_expect_tx(&bars[0], kPackBytes);
    tc::bulk_g2s(sW, a.pack, kPackBytes, &bars[0]);
  }
  bool ok = wait_all(&bars[0], ph_w, a.err, failed);
  constexpr uint32_t kI64 = tc::idesc_bf16(128, 64, 0, 0);
  constexpr uint32_t kI16 = tc::idesc_bf16(128, 16, 0, 0);
  const uint32_t aX = tc::smem_u32(sX), aH = tc::smem_u32(sH), aW = tc::smem_u32(sW);
  const int ntiles = (a.n + kTile - 1) / kTile;
  unsigned int dmax = 0;
  // The X tile is loaded by TMA one tile ahead: as soon as layer 1 has read
  // it, the next tile's copy is issued and overlaps layers 2 and 3.
  auto load_x = [&](int tile) {
    tc::mbar_arrive_expect_tx(&bars[1], kTile * kFeat * 2);
#pragma unroll
    for (int c = 0; c < kFeat / 8; ++c) tc::tensor_g2s_2d(sX + c * kTile * 16, &tmX, 8 * c, tile * kTile, &bars[1]);
  };
  bool x_pending = ok && (int)blockIdx.x < ntiles;  // a tile copy is in flight (same in every thread)
  if (t == 0 && x_pending) load_x(blockIdx.x);
  for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
    if (!(ok = wait_all(&bars[1], ph_x, a.err, failed))) break;
    x_pending = false;
    // layer 1: D[0, 64) = X W1
    if (t == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kFeat / 16; ++kk)
        tc::mma_bf16(tmem, tc::smem_desc(aX + kk * 2 * kTile * 16, kTile * 16, 128),
                     tc::smem_desc(aW + kPB1 + kk * 2 * 64 * 16, 64 * 16, 128), kI64, kk > 0);
      tc::mma_commit(&bars[2]);
    }
    if (!(ok = wait_all(&bars[2], ph_m, a.err, failed))) break;
    if (tile + (int)gridDim.x < ntiles) {
      x_pending = true;
      if (t == 0) load_x(tile + gridDim.x);
    }
    tc::fence_after_sync();
    const int r = warp * 32 + lane;
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + c, v);
      store_act16(sH, r, c, v, sB + c, true);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    // layer 2: D[64, 128) = H1 W2
    if (t == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kHid / 16; ++kk)
        tc::mma_bf16(tmem + 64, tc::smem_desc(aH + kk * 2 * kTile * 16, kTile * 16, 128),
                     tc::smem_desc(aW + kPB2 + kk * 2 * 64 * 16, 64 * 16, 128), kI64, kk > 0);
      tc::mma_commit(&bars[2]);
    }
    if (!(ok = wait_all(&bars[2], ph_m, a.err, failed))) break;
    tc::fence_after_sync();
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + 64 + c, v);
      store_act16(sH, r, c, v, sB + kHid + c, true);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    // layer 3: D[0, 16) = H2 W3 (3 columns used)
    if (t == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kHid / 16; ++kk)
        tc::mma_bf16(tmem, tc::smem_desc(aH + kk * 2 * kTile * 16, kTile * 16, 128),
                     tc::smem_desc(aW + kPB3 + kk * 2 * 16 * 16, 16 * 16, 128), kI16, kk > 0);
      tc::mma_commit(&bars[2]);
    }
    if (!(ok = wait_all(&bars[2], ph_m, a.err, failed))) break;
    tc::fence_after_sync();
    float v[16];
    tc::tmem_ld16(tmem + lane_base, v);
    const int row = tile * kTile + r;
    if (row < a.n) {
      const float y0 = v[0] + sB[2 * kHid], y1 = v[1] + sB[2 * kHid + 1], y2 = v[2] + sB[2 * kHid + 2];
      if (kApply) {
        float4 x = a.xs[row];
        x.x = x.x + a.scale_len * y0;
        x.y = x.y + a.scale_len * y1;
        x.z = x.z + a.scale_len * y2;
        a.xs[row] = x;
        const float4 p = a.pos[row];
        const float d = fmaxf(fmaxf(fabsf(x.x - p.x), fabsf(x.y - p.y)), fabsf(x.z - p.z));
        dmax = max(dmax, __float_as_uint(d));
      } else {
        a.y[3 * (size_t)row] = y0;
        a.y[3 * (size_t)row + 1] = y1;
        a.y[3 * (size_t)row + 2] = y2;
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  drain(failed);
  if (x_pending && failed.bar != &bars[1]) tc::mbar_wait(&bars[1], ph_x, kWaitPolls);
  if (kApply) warp_max_bits(a.disp_bits, dmax);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 128);
  }
}

}  // namespace gg

// ------------------------------------------------------------ training

namespace gg {

// Training shared-memory map (bytes).  X, H1 and H2 are 128 x 128 tiles:
// their extra columns are zero except one constant 1 (column 48 of X,
// column 64 of H1 and H2), so that the weight-gradient MMAs, which read
// them transposed as 128-row operands, also produce the bias gradients.
constexpr int kTrW = 0;                     // packed weights   26624
constexpr int kTrX = 27648;                 // X   128 x 128    32768
constexpr int kTrH1 = kTrX + 32768;         // H1  128 x 128    32768
constexpr int kTrH2 = kTrH1 + 32768;        // H2  128 x 128    32768
constexpr int kTrDY = kTrH2 + 32768;        // dY  128 x 16      4096
constexpr int kTrD2 = kTrDY + 4096;         // dH2 128 x 64     16384
constexpr int kTrD1 = kTrD2 + 16384;        // dH1 128 x 64     16384
constexpr int kTrB = kTrD1 + 16384;         // biases 131 floats
constexpr int kTrBar = kTrB + 528;
constexpr int kTrSlot = kTrBar + 24;
constexpr int kTrSmem = kTrSlot + 8;
// TMEM columns (512 allocated)
constexpr uint32_t kTmD1 = 0, kTmD2 = 64, kTmD3 = 128, kTmGW1 = 256, kTmGW2 = 320, kTmGW3 = 384;

__device__ __forceinline__ float bf16_at(const uint8_t* tile, int r, int c) {
  return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(tile + tc::canon_off(r, c, kTile)));
}

// One pass over the samples: loss and gradient of the mean squared error
// between the MLP's prediction and the targets, accumulated into a.loss and
// a.grad (fp32, one atomic add per CTA and parameter).
__global__ void __launch_bounds__(kTile, 1) k_mlp_train(const __grid_constant__ CUtensorMap tmX, MlpArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sW = smem + kTrW;
  uint8_t* sX = smem + kTrX;
  uint8_t* sH1 = smem + kTrH1;
  uint8_t* sH2 = smem + kTrH2;
  uint8_t* sDY = smem + kTrDY;
  uint8_t* sD2 = smem + kTrD2;
  uint8_t* sD1 = smem + kTrD1;
  float* sB = reinterpret_cast<float*>(smem + kTrB);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kTrBar);
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + kTrSlot);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int r = warp * 32 + lane;
  if (t == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::mbar_init(&bars[2], 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(slot, 512);
  for (int k = t; k < 2 * kHid + kOut; k += kTile)
    sB[k] = k < kHid ? a.params[kOffB1 + k] : (k < 2 * kHid ? a.params[kOffB2 + k - kHid] : a.params[kOffB3 + k - 2 * kHid]);
  // padding columns: zeros and the constant-1 column
  {
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    const uint32_t one = (uint32_t)bf16_bits(1.0f);
    for (int c = kFeat / 8; c < 16; ++c)
      *reinterpret_cast<uint4*>(sX + tc::canon_off(r, 8 * c, kTile)) =
          c == kFeat / 8 ? make_uint4(one, 0u, 0u, 0u) : z;
    for (int c = kHid / 8; c < 16; ++c) {
      const uint4 v = c == kHid / 8 ? make_uint4(one, 0u, 0u, 0u) : z;
      *reinterpret_cast<uint4*>(sH1 + tc::canon_off(r, 8 * c, kTile)) = v;
      *reinterpret_cast<uint4*>(sH2 + tc::canon_off(r, 8 * c, kTile)) = v;
    }
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  uint32_t ph_w = 0, ph_x = 0, ph_m = 0;
  WaitState failed;
  if (t == 0) {
    tc::mbar_arrive_expect_tx(&bars[0], kPackBytes);
    tc::bulk_g2s(sW, a.pack, kPackBytes, &bars[0]);
  }
  bool ok = wait_all(&bars[0], ph_w, a.err, failed);
  constexpr uint32_t kI64 = tc::idesc_bf16(128, 64, 0, 0);
  constexpr uint32_t kI16 = tc::idesc_bf16(128, 16, 0, 0);
  constexpr uint32_t kG64 = tc::idesc_bf16(128, 64, 1, 1);  // transposed A and B
  constexpr uint32_t kG16 = tc::idesc_bf16(128, 16, 1, 1);
  const uint32_t aX = tc::smem_u32(sX), aH1 = tc::smem_u32(sH1), aH2 = tc::smem_u32(sH2), aDY = tc::smem_u32(sDY),
                 aD2 = tc::smem_u32(sD2), aD1 = tc::smem_u32(sD1), aW = tc::smem_u32(sW);
  constexpr uint32_t kColStep = kTile * 16;  // bytes between 16-byte column blocks of a 128-row tile
  // Transposed (MN-major) operands of the weight-gradient MMAs read the same
  // tiles with the 16-byte column blocks along M or N: without swizzling the
  // stride byte offset is then the M/N step (kColStep) and the leading byte
  // offset the K step (128 B per 8 samples).
  const int ntiles = (a.n + kTile - 1) / kTile;
  int done = 0;
  float lsum = 0.0f;
  for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x, ++done) {
    const int row = tile * kTile + r;
    float tg[kOut] = {0.f, 0.f, 0.f};
    if (row < a.n) {
#pragma unroll
      for (int o = 0; o < kOut; ++o) tg[o] = a.target[(size_t)kOut * row + o];
    }
    if (t == 0) {
      tc::mbar_arrive_expect_tx(&bars[1], kTile * kFeat * 2);
#pragma unroll
      for (int c = 0; c < kFeat / 8; ++c) tc::tensor_g2s_2d(sX + c * kColStep, &tmX, 8 * c, tile * kTile, &bars[1]);
    }
    if (!(ok = wait_all(&bars[1], ph_x, a.err, failed))) break;
    // ---- forward
    if (t == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kFeat / 16; ++kk)
        tc::mma_bf16(tmem + kTmD1, tc::smem_desc(aX + kk * 2 * kColStep, kColStep, 128),
                     tc::smem_desc(aW + kPB1 + kk * 2 * 64 * 16, 64 * 16, 128), kI64, kk > 0);
      tc::mma_commit(&bars[2]);
    }
    if (!(ok = wait_all(&bars[2], ph_m, a.err, failed))) break;
    tc::fence_after_sync();
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + kTmD1 + c, v);
      store_act16(sH1, r, c, v, sB + c, true);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (t == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kHid / 16; ++kk)
        tc::mma_bf16(tmem + kTmD2, tc::smem_desc(aH1 + kk * 2 * kColStep, kColStep, 128),
                     tc::smem_desc(aW + kPB2 + kk * 2 * 64 * 16, 64 * 16, 128), kI64, kk > 0);
      tc::mma_commit(&bars[2]);
    }
    if (!(ok = wait_all(&bars[2], ph_m, a.err, failed))) break;
    tc::fence_after_sync();
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + kTmD2 + c, v);
      store_act16(sH2, r, c, v, sB + kHid + c, true);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (t == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kHid / 16; ++kk)
        tc::mma_bf16(tmem + kTmD3, tc::smem_desc(aH2 + kk * 2 * kColStep, kColStep, 128),
                     tc::smem_desc(aW + kPB3 + kk * 2 * 16 * 16, 16 * 16, 128), kI16, kk > 0);
      tc::mma_commit(&bars[2]);
    }
    if (!(ok = wait_all(&bars[2], ph_m, a.err, failed))) break;
    tc::fence_after_sync();
    {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + kTmD3, v);
      float dy[kOut];
#pragma unroll
      for (int o = 0; o < kOut; ++o) {
        const float e = row < a.n ? (v[o] + sB[2 * kHid + o]) - tg[o] : 0.0f;
        lsum += e * e;
        dy[o] = a.grad_scale * e;
      }
      const uint32_t w0 = (uint32_t)bf16_bits(dy[0]) | ((uint32_t)bf16_bits(dy[1]) << 16);
      const uint32_t w1 = (uint32_t)bf16_bits(dy[2]);
      *reinterpret_cast<uint4*>(sDY + tc::canon_off(r, 0, kTile)) = make_uint4(w0, w1, 0u, 0u);
      *reinterpret_cast<uint4*>(sDY + tc::canon_off(r, 8, kTile)) = make_uint4(0u, 0u, 0u, 0u);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    // ---- backward: dW3 += H2^T dY (transposed operands, K = 128 samples),
    // dH2 = dY W3^T
    if (t == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kTile / 16; ++kk)
        tc::mma_bf16(tmem + kTmGW3, tc::smem_desc(aH2 + kk * 256, 128, kColStep),
                     tc::smem_desc(aDY + kk * 256, 128, kColStep), kG16, (done > 0 || kk > 0) ? 1u : 0u);
      tc::mma_bf16(tmem + kTmD1, tc::smem_desc(aDY, kColStep, 128), tc::smem_desc(aW + kPB3b, 64 * 16, 128), kI64,
                   0u);
      tc::mma_commit(&bars[2]);
    }
    if (!(ok = wait_all(&bars[2], ph_m, a.err, failed))) break;
    tc::fence_after_sync();
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + kTmD1 + c, v);
#pragma unroll
      for (int k = 0; k < 16; ++k)
        if (!(bf16_at(sH2, r, c + k) > 0.0f)) v[k] = 0.0f;
      const float zero[16] = {};
      store_act16(sD2, r, c, v, zero, false);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    // dW2 += H1^T dH2, dH1 = dH2 W2^T
    if (t == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kTile / 16; ++kk)
        tc::mma_bf16(tmem + kTmGW2, tc::smem_desc(aH1 + kk * 256, 128, kColStep),
                     tc::smem_desc(aD2 + kk * 256, 128, kColStep), kG64, (done > 0 || kk > 0) ? 1u : 0u);
#pragma unroll
      for (int kk = 0; kk < kHid / 16; ++kk)
        tc::mma_bf16(tmem + kTmD2, tc::smem_desc(aD2 + kk * 2 * kColStep, kColStep, 128),
                     tc::smem_desc(aW + kPB2b + kk * 2 * 64 * 16, 64 * 16, 128), kI64, kk > 0);
      tc::mma_commit(&bars[2]);
    }
    if (!(ok = wait_all(&bars[2], ph_m, a.err, failed))) break;
    tc::fence_after_sync();
#pragma unroll
    for (int c = 0; c < kHid; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + kTmD2 + c, v);
#pragma unroll
      for (int k = 0; k < 16; ++k)
        if (!(bf16_at(sH1, r, c + k) > 0.0f)) v[k] = 0.0f;
      const float zero[16] = {};
      store_act16(sD1, r, c, v, zero, false);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    // dW1 += X^T dH1
    if (t == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < kTile / 16; ++kk)
        tc::mma_bf16(tmem + kTmGW1, tc::smem_desc(aX + kk * 256, 128, kColStep),
                     tc::smem_desc(aD1 + kk * 256, 128, kColStep), kG64, (done > 0 || kk > 0) ? 1u : 0u);
      tc::mma_commit(&bars[2]);
    }
    if (!(ok = wait_all(&bars[2], ph_m, a.err, failed))) break;
    tc::fence_after_sync();
  }
  drain(failed);
  // loss
  {
    float l = lsum;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if (lane == 0 && l != 0.0f) atomicAdd(a.loss, l * a.grad_scale * 0.5f);
  }
  // gradients: TMEM lane r holds row r of each accumulator
  if (ok && done > 0) {
    tc::fence_after_sync();
    for (int c = 0; c < kHid; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + lane_base + kTmGW1 + c, v);
      if (r < kFeat) {
        for (int k = 0; k < 16; ++k) atomicAdd(&a.grad[kOffW1 + r * kHid + c + k], v[k]);
      } else if (r == kFeat) {
        for (int k = 0; k < 16; ++k) atomicAdd(&a.grad[kOffB1 + c + k], v[k]);
      }
      tc::tmem_ld16(tmem + lane_base + kTmGW2 + c, v);
      if (r < kHid) {
        for (int k = 0; k < 16; ++k) atomicAdd(&a.grad[kOffW2 + r * kHid + c + k], v[k]);
      } else if (r == kHid) {
        for (int k = 0; k < 16; ++k) atomicAdd(&a.grad[kOffB2 + c + k], v[k]);
      }
    }
    float v[16];
    tc::tmem_ld16(tmem + lane_base + kTmGW3, v);
    if (r < kHid) {
      for (int o = 0; o < kOut; ++o) atomicAdd(&a.grad[kOffW3 + r * kOut + o], v[o]);
    } else if (r == kHid) {
      for (int o = 0; o < kOut; ++o) atomicAdd(&a.grad[kOffB3 + o], v[o]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}

// Adam on the fp32 parameters (bias-corrected step sizes passed in).
__global__ void k_adam(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M,
                       float* __restrict__ V, int n, float lr_t, float b1, float b2, float eps, float wd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = G[i] + wd * P[i];
  const float m = b1 * M[i] + (1.0f - b1) * g;
  const float v = b2 * V[i] + (1.0f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  P[i] = P[i] - lr_t * m / (sqrtf(v) + eps);
}

}  // namespace gg

// ------------------------------------------------------------ host side

struct gg_mlp {
  int device = 0;
  int num_sms = 0;
  float* params = nullptr;  // fp32 master copy
  float* grad = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  float* loss = nullptr;
  int* err = nullptr;
  uint8_t* pack = nullptr;  // packed bf16 weights
  int64_t steps = 0;
};

namespace gg {

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// Tensor map of an n x 48 bf16 row-major feature matrix, box 8 columns x
// 128 rows (one 16-byte column block of a tile); rows past n read as zero.
gg_status feature_map(const void* X, int64_t n, CUtensorMap* map) {
  auto enc = encode_fn();
  if (!enc) {
    set_error("tensor map: cuTensorMapEncodeTiled is not available");
    return GG_ERR_CUDA;
  }
  if ((reinterpret_cast<uintptr_t>(X) & 15u) != 0) {
    set_error("features must be 16-byte aligned");
    return GG_ERR_INVALID_ARGUMENT;
  }
  cuuint64_t dims[2] = {(cuuint64_t)kFeat, (cuuint64_t)n};
  cuuint64_t strides[1] = {(cuuint64_t)kFeat * 2};
  cuuint32_t box[2] = {8, (cuuint32_t)kTile};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(X), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("tensor map: cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return GG_ERR_CUDA;
  }
  return GG_OK;
}

gg_status mlp_check_err(gg_mlp* M) {
  int e = 0;
  GG_CUDA(cudaMemcpy(&e, M->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    GG_CUDA(cudaMemset(M->err, 0, sizeof(int)));
    set_error("MLP kernel: a bounded wait on the tensor-core pipeline ran out");
    return GG_ERR_TIMEOUT;
  }
  return GG_OK;
}

gg_status mlp_pack(gg_mlp* M, cudaStream_t st) {
  k_pack_weights<<<(kPackElems + 255) / 256, 256, 0, st>>>(M->params, M->pack);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace

// Forward over n feature rows: into y (n x 3), or (apply) added to x*.
gg_status mlp_forward(gg_mlp* M, const void* X, int64_t n, float* y, float4* xs, const float4* pos,
                      float scale_len, unsigned int* disp_bits, cudaStream_t st, int64_t* launches) {
  if (n <= 0) return GG_OK;
  CUtensorMap map;
  gg_status rc = feature_map(X, n, &map);
  if (rc != GG_OK) return rc;
  MlpArgs a{};
  a.n = (int)n;
  a.pack = M->pack;
  a.params = M->params;
  a.y = y;
  a.xs = xs;
  a.pos = pos;
  a.scale_len = scale_len;
  a.disp_bits = disp_bits;
  a.err = M->err;
  const int ntiles = (int)((n + kTile - 1) / kTile);
  // four CTAs per SM (57 KB of shared memory and 128 TMEM columns each)
  const int grid = std::max(1, std::min(ntiles, 4 * M->num_sms));
  if (xs) {
    GG_CUDA(cudaFuncSetAttribute(k_mlp_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwSmem));
    k_mlp_fwd<true><<<grid, kTile, kFwSmem, st>>>(map, a);
  } else {
    GG_CUDA(cudaFuncSetAttribute(k_mlp_fwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwSmem));
    k_mlp_fwd<false><<<grid, kTile, kFwSmem, st>>>(map, a);
  }
  if (launches) ++*launches;
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

gg_status mlp_gradient(gg_mlp* M, const void* X, const float* T, int64_t n, cudaStream_t st) {
  CUtensorMap map;
  gg_status rc = feature_map(X, n, &map);
  if (rc != GG_OK) return rc;
  GG_CUDA(cudaMemsetAsync(M->grad, 0, sizeof(float) * kNParams, st));
  GG_CUDA(cudaMemsetAsync(M->loss, 0, sizeof(float), st));
  MlpArgs a{};
  a.n = (int)n;
  a.pack = M->pack;
  a.params = M->params;
  a.target = T;
  a.grad_scale = 2.0f / (3.0f * (float)n);
  a.grad = M->grad;
  a.loss = M->loss;
  a.err = M->err;
  const int ntiles = (int)((n + kTile - 1) / kTile);
  const int grid = std::max(1, std::min(ntiles, M->num_sms));
  GG_CUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrSmem));
  k_mlp_train<<<grid, kTile, kTrSmem, st>>>(map, a);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

gg_status gg_mlp_create(int32_t device, uint64_t seed, gg_mlp** out) {
  if (!out) {
    set_error("gg_mlp_create: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  GG_CUDA(cudaSetDevice(device));
  gg_mlp* M = new gg_mlp();
  M->device = device;
  cudaDeviceGetAttribute(&M->num_sms, cudaDevAttrMultiProcessorCount, device);
  cudaError_t e = cudaSuccess;
  for (float** p : {&M->params, &M->grad, &M->m, &M->v})
    if (e == cudaSuccess) e = cudaMalloc((void**)p, sizeof(float) * kNParams);
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->err, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->pack, kPackBytes);
  if (e != cudaSuccess) {
    gg_mlp_destroy(M);
    cudaGetLastError();
    set_error(std::string("gg_mlp_create: allocation failed: ") + cudaGetErrorString(e));
    return GG_ERR_OUT_OF_MEMORY;
  }
  // He-uniform weights, zero biases, from a 64-bit linear congruential
  // generator (reproducible on every host)
  std::vector<float> P(kNParams, 0.0f);
  uint64_t s = seed * 6364136223846793005ull + 1442695040888963407ull;
  auto uni = [&]() {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return (float)((double)(s >> 11) * (1.0 / 9007199254740992.0)) * 2.0f - 1.0f;
  };
  const float a1 = std::sqrt(6.0f / kFeat), a2 = std::sqrt(6.0f / kHid), a3 = std::sqrt(3.0f / kHid) * 0.1f;
  for (int k = 0; k < kFeat * kHid; ++k) P[kOffW1 + k] = a1 * uni();
  for (int k = 0; k < kHid * kHid; ++k) P[kOffW2 + k] = a2 * uni();
  for (int k = 0; k < kHid * kOut; ++k) P[kOffW3 + k] = a3 * uni();
  const gg_status rc = gg_mlp_set_params(M, P.data(), kNParams);
  if (rc != GG_OK) {
    gg_mlp_destroy(M);
    return rc;
  }
  *out = M;
  return GG_OK;
}

int64_t gg_mlp_num_params(void) { return kNParams; }

gg_status gg_mlp_set_params(gg_mlp* M, const float* host, int64_t n) {
  if (!M || !host || n != kNParams) {
    set_error("gg_mlp_set_params: null argument or wrong parameter count");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(M->device));
  GG_CUDA(cudaMemcpy(M->params, host, sizeof(float) * kNParams, cudaMemcpyHostToDevice));
  GG_CUDA(cudaMemset(M->m, 0, sizeof(float) * kNParams));
  GG_CUDA(cudaMemset(M->v, 0, sizeof(float) * kNParams));
  GG_CUDA(cudaMemset(M->err, 0, sizeof(int)));
  M->steps = 0;
  gg_status rc = mlp_pack(M, nullptr);
  if (rc != GG_OK) return rc;
  GG_CUDA(cudaDeviceSynchronize());
  return GG_OK;
}

gg_status gg_mlp_get_params(gg_mlp* M, float* host, int64_t n) {
  if (!M || !host || n != kNParams) {
    set_error("gg_mlp_get_params: null argument or wrong parameter count");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(M->device));
  GG_CUDA(cudaMemcpy(host, M->params, sizeof(float) * kNParams, cudaMemcpyDeviceToHost));
  return GG_OK;
}

gg_status gg_mlp_forward(gg_mlp* M, const void* d_features, int64_t n, float* d_out, void* stream) {
  if (!M || (n > 0 && (!d_features || !d_out)) || n < 0 || n > INT32_MAX - kTile) {
    set_error("gg_mlp_forward: bad argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(M->device));
  cudaStream_t st = (cudaStream_t)stream;
  gg_status rc = mlp_forward(M, d_features, n, d_out, nullptr, nullptr, 0.0f, nullptr, st, nullptr);
  if (rc != GG_OK) return rc;
  GG_CUDA(cudaStreamSynchronize(st));
  return mlp_check_err(M);
}

gg_status gg_mlp_gradient(gg_mlp* M, const void* d_features, const float* d_targets, int64_t n, float* host_grad,
                          float* host_loss, void* stream) {
  if (!M || !d_features || !d_targets || n <= 0 || n > INT32_MAX - kTile) {
    set_error("gg_mlp_gradient: bad argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(M->device));
  cudaStream_t st = (cudaStream_t)stream;
  gg_status rc = mlp_gradient(M, d_features, d_targets, n, st);
  if (rc != GG_OK) return rc;
  if (host_grad) GG_CUDA(cudaMemcpyAsync(host_grad, M->grad, sizeof(float) * kNParams, cudaMemcpyDeviceToHost, st));
  if (host_loss) GG_CUDA(cudaMemcpyAsync(host_loss, M->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  return mlp_check_err(M);
}

gg_status gg_mlp_train_step(gg_mlp* M, const void* d_features, const float* d_targets, int64_t n, float lr,
                            float weight_decay, float* host_loss, void* stream) {
  if (!M || !d_features || !d_targets || n <= 0 || n > INT32_MAX - kTile) {
    set_error("gg_mlp_train_step: bad argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(M->device));
  cudaStream_t st = (cudaStream_t)stream;
  gg_status rc = mlp_gradient(M, d_features, d_targets, n, st);
  if (rc != GG_OK) return rc;
  M->steps++;
  const float b1 = 0.9f, b2 = 0.999f;
  const double c1 = 1.0 - std::pow((double)b1, (double)M->steps);
  const double c2 = 1.0 - std::pow((double)b2, (double)M->steps);
  const float lr_t = (float)(lr * std::sqrt(c2) / c1);
  k_adam<<<(kNParams + 255) / 256, 256, 0, st>>>(M->params, M->grad, M->m, M->v, kNParams, lr_t, b1, b2, 1e-8f,
                                                 weight_decay);
  GG_CUDA(cudaGetLastError());
  rc = mlp_pack(M, st);
  if (rc != GG_OK) return rc;
  if (host_loss) GG_CUDA(cudaMemcpyAsync(host_loss, M->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  return mlp_check_err(M);
}

void gg_mlp_destroy(gg_mlp* M) {
  if (!M) return;
  cudaSetDevice(M->device);
  cudaFree(M->params);
  cudaFree(M->grad);
  cudaFree(M->m);
  cudaFree(M->v);
  cudaFree(M->loss);
  cudaFree(M->err);
  cudaFree(M->pack);
  delete M;
}

}  // extern "C"

// ------------------------------------------------------------ in the substep

namespace gg {

namespace {

// Length and velocity scales of the features and the prediction: |g| dt^2
// and |g| dt (a tenth of the cell length per substep without gravity).
void warm_scales(const gg_system* S, float& slen, float& svel) {
  const double g = std::sqrt((double)S->phys.g.x * S->phys.g.x + (double)S->phys.g.y * S->phys.g.y +
                             (double)S->phys.g.z * S->phys.g.z);
  const double dt = S->phys.dt;
  slen = (float)(g * dt * dt);
  svel = (float)(g * dt);
  if (!(slen > 0.0f) || !(svel > 0.0f)) {
    slen = 0.1f * S->grid.L;
    svel = slen / (float)(dt > 0 ? dt : 1.0);
  }
}

gg_status features(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  const int c = S->g.cur;
  float slen, svel;
  warm_scales(S, slen, svel);
  FeatArgs a;
  a.g = S->grid;
  a.n = (int)S->n;
  a.xs = S->g.xs;
  a.pos = S->g.pos[c];
  a.vel = S->g.vel[c];
  a.mass = S->g.mass[c];
  a.cs = S->g.cell_start;
  a.bcs = S->b.cell_start;
  a.bpos = S->b.pos;
  a.out = reinterpret_cast<__nv_bfloat16*>(S->feat);
  a.inv_slen = 1.0f / slen;
  a.inv_svel = 1.0f / svel;
  a.brad = (float)S->P.boundary_radius;
  a.minr = S->P.boundary_min_radius;
  a.inv_height = 1.0f / (S->grid.L * (float)S->grid.ny);
  prof_begin(S, PC_FEATURES, st);
  k_features<<<blocks_for(S->n, 256), 256, 0, st>>>(a);
  count_launches(S, 1);
  prof_end(S, PC_FEATURES, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

__global__ void k_warm_target(int n, const float4* __restrict__ xs, const float4* __restrict__ xs0,
                              float* __restrict__ target, float inv_slen) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = xs[i], b = xs0[i];
  target[3 * (size_t)i] = (a.x - b.x) * inv_slen;
  target[3 * (size_t)i + 1] = (a.y - b.y) * inv_slen;
  target[3 * (size_t)i + 2] = (a.z - b.z) * inv_slen;
}

// Penetration at x*, r_i + r_j - |x_i - x_j| over the particle pairs in the
// sweeps' stencil and (0.01 + max(r_i, 0.01)) - |x - b| over wall
// particles: the largest, and the sum and number of the positive ones (a
// pair counts once from each side; the mean is unchanged by that).
__global__ void __launch_bounds__(256) k_residual(Grid g, int n, const float4* __restrict__ xs,
                                                  const int32_t* __restrict__ cs, const int32_t* __restrict__ bcs,
                                                  const float4* __restrict__ bpos, float brad, float minr,
                                                  DevScalars* __restrict__ scal) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float best = 0.0f, sum = 0.0f;
  unsigned int cnt = 0;
  if (i < n) {
    const float4 x4 = xs[i];
    const float3 x = f3(x4);
    const float ri = x4.w;
    const float Bw = brad + fmaxf(ri, minr);
    const int3 q = trunc_cell(g, x);
    for_each_stencil_column(g, q, [&](int k0, int nc) {
      const int j1 = cs[k0 + nc];
      for (int j = cs[k0]; j < j1; ++j) {
        if (j == i) continue;
        const float4 xj = xs[j];
        const float dx = x.x - xj.x, dy = x.y - xj.y, dz = x.z - xj.z;
        const float R = ri + xj.w;
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 < R * R) {
          const float p = R - sqrtf(d2);
          best = fmaxf(best, p);
          sum += p;
          ++cnt;
        }
      }
      const int b1 = bcs[k0 + nc];
      for (int b = bcs[k0]; b < b1; ++b) {
        const float4 pb = bpos[b];
        const float dx = x.x - pb.x, dy = x.y - pb.y, dz = x.z - pb.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 < Bw * Bw) {
          const float p = Bw - sqrtf(d2);
          best = fmaxf(best, p);
          sum += p;
          ++cnt;
        }
      }
    });
  }
  __shared__ float s_sum[8];
  __shared__ unsigned int s_cnt[8];
  float ws = sum;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ws += __shfl_xor_sync(0xffffffffu, ws, o);
  const unsigned int wc = __reduce_add_sync(0xffffffffu, cnt);
  if ((threadIdx.x & 31) == 0) {
    s_sum[threadIdx.x >> 5] = ws;
    s_cnt[threadIdx.x >> 5] = wc;
  }
  block_max_bits<256>(&scal->pen_bits, __float_as_uint(best));  // synchronises the block
  if (threadIdx.x == 0) {
    double bs = 0.0;
    unsigned int bc = 0;
    for (int w = 0; w < 8; ++w) {
      bs += (double)s_sum[w];
      bc += s_cnt[w];
    }
    if (bc) {
      atomicAdd(&scal->pen_sum, bs);
      atomicAdd(&scal->pen_count, bc);
    }
  }
}

}  // namespace

gg_status warm_start_apply(gg_system* S, cudaStream_t st) {
  if (!S->mlp || !S->feat) {
    set_error("warm_start = 1 needs a network attached with gg_set_warm_start");
    return GG_ERR_INVALID_ARGUMENT;
  }
  if (S->n <= 0) return GG_OK;
  gg_status rc = features(S, st);
  if (rc != GG_OK) return rc;
  float slen, svel;
  warm_scales(S, slen, svel);
  prof_begin(S, PC_MLP, st);
  rc = mlp_forward(S->mlp, S->feat, S->n, nullptr, S->g.xs, S->g.pos[S->g.cur], slen * S->P.warm_start_scale,
                   &S->scal->disp0_bits, st, &S->launches);
  prof_end(S, PC_MLP, S->n, st);
  return rc;
}

gg_status warm_start_record(gg_system* S, cudaStream_t st) {
  if (!S->feat) {
    set_error("warm_start = 2 needs gg_set_warm_start (it allocates the buffers)");
    return GG_ERR_INVALID_ARGUMENT;
  }
  if (S->n <= 0) return GG_OK;
  gg_status rc = features(S, st);
  if (rc != GG_OK) return rc;
  GG_CUDA(cudaMemcpyAsync(S->xs0, S->g.xs, sizeof(float4) * (size_t)S->n, cudaMemcpyDeviceToDevice, st));
  return GG_OK;
}

gg_status warm_start_target(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  float slen, svel;
  warm_scales(S, slen, svel);
  k_warm_target<<<blocks_for(S->n, 256), 256, 0, st>>>((int)S->n, S->g.xs, S->xs0, S->warm_target, 1.0f / slen);
  count_launches(S, 1);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

gg_status residual(gg_system* S, cudaStream_t st, float* out) {
  *out = 0.0f;
  S->last_residual_max = 0.0f;
  if (S->n <= 0) return GG_OK;
  const size_t off = offsetof(DevScalars, pen_bits);
  const size_t len = offsetof(DevScalars, pen_sum) + sizeof(double) - off;
  GG_CUDA(cudaMemsetAsync(reinterpret_cast<char*>(S->scal) + off, 0, len, st));
  prof_begin(S, PC_RESIDUAL, st);
  k_residual<<<blocks_for(S->n, 256), 256, 0, st>>>(S->grid, (int)S->n, S->g.xs, S->g.cell_start, S->b.cell_start,
                                                    S->b.pos, (float)S->P.boundary_radius,
                                                    S->P.boundary_min_radius, S->scal);
  count_launches(S, 1);
  prof_end(S, PC_RESIDUAL, S->n, st);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(S->scal_host) + off, reinterpret_cast<char*>(S->scal) + off, len,
                          cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  std::memcpy(&S->last_residual_max, &S->scal_host->pen_bits, sizeof(float));
  const unsigned int c = S->scal_host->pen_count;
  *out = c ? (float)(S->scal_host->pen_sum / (double)c) : 0.0f;
  return GG_OK;
}

}  // namespace gg

extern "C" gg_status gg_set_warm_start(gg_system* S, gg_mlp* M) {
  if (!S) {
    set_error("gg_set_warm_start: null system");
    return GG_ERR_INVALID_ARGUMENT;
  }
  if (M && M->device != S->device) {
    set_error("gg_set_warm_start: the network lives on another device");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(S->device));
  const size_t cap = (size_t)std::max<int64_t>(S->cap, 1);
  cudaError_t e = cudaSuccess;
  if (!S->feat) e = cudaMalloc(&S->feat, cap * kFeat * 2);
  if (e == cudaSuccess && !S->xs0) e = cudaMalloc((void**)&S->xs0, cap * sizeof(float4));
  if (e == cudaSuccess && !S->warm_target) e = cudaMalloc((void**)&S->warm_target, cap * 3 * sizeof(float));
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(std::string("gg_set_warm_start: allocation failed: ") + cudaGetErrorString(e));
    return GG_ERR_OUT_OF_MEMORY;
  }
  S->mlp = M;
  return GG_OK;
}

// ------------------------------------------------------------ self-test of the bounded waits

namespace gg {

// One block waits, with the tensor-core kernels' bounded wait, for an
// mbarrier phase that nothing completes: the wait must give up after
// `polls` polls, agree across the block and record ERR_TIMEOUT.
__global__ void k_wait_selftest(uint32_t polls, int* __restrict__ err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  const bool mine = tc::mbar_wait(&bar, 0, polls);
  const bool ok = __syncthreads_and(mine) != 0;
  if (!ok && threadIdx.x == 0) atomicOr(err, ERR_TIMEOUT);
}

}  // namespace gg

extern "C" gg_status gg_selftest_bounded_wait(int32_t device, int32_t polls) {
  if (polls <= 0 || polls > (1 << 20)) {
    set_error("gg_selftest_bounded_wait: polls must be in 1..2^20");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(device));
  int* err = nullptr;
  GG_CUDA(cudaMalloc((void**)&err, sizeof(int)));
  cudaError_t e = cudaMemset(err, 0, sizeof(int));
  if (e == cudaSuccess) {
    k_wait_selftest<<<1, 128>>>((uint32_t)polls, err);
    e = cudaGetLastError();
  }
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(err);
  GG_CUDA(e);
  if (h & ERR_TIMEOUT) {
    set_error("gg_selftest_bounded_wait: the wait gave up after its poll limit, as designed");
    return GG_ERR_TIMEOUT;
  }
  set_error("gg_selftest_bounded_wait: a phase nothing completes was reported complete");
  return GG_ERR_CUDA;
}

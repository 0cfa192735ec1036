// common.cuh — device helpers shared by the kernels.
//
// Arithmetic here follows the reference's expressions operation by
// operation (helper_math.h semantics for float3), and the library is built
// with -fmad=false so no multiply-add is fused behind the source's back:
// the CPU oracle (built with -ffp-contract=off) performs the same roundings.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gg_internal.h"

namespace gg {

#define GG_PI_D 3.14159265358979323846
#define GG_PI_F 3.14159265358979323846f

__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 smul3(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 mul3s(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 div3s(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
// helper_math dot, left to right.
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len3(float3 a) { return sqrtf(dot3(a, a)); }
// helper_math normalize: v * rsqrtf(dot(v, v)).
__device__ __forceinline__ float3 normalize3(float3 a) { return mul3s(a, rsqrtf(dot3(a, a))); }

// particlePos2cellIdx, CUDAFunctions.cuh:71-79.
__device__ __forceinline__ int cell_key(const Grid& g, int x, int y, int z) {
  return (x >= 0 && x < g.nx && y >= 0 && y < g.ny && z >= 0 && z < g.nz)
             ? ((x * g.ny) + y) * g.nz + z
             : g.C;
}

// The 27-cell stencil of q in the reference's order m = 0..26 (dx, dy, dz
// from -1 to 1, dz fastest), grouped by column: for each (dx, dy) the cells
// z-1, z, z+1 that lie in the grid have consecutive keys, so f(k0, nc)
// receives the first key and the number of cells.  The cells skipped are
// exactly those cell_key maps to C.
template <class F>
__device__ __forceinline__ void for_each_stencil_column(const Grid& g, int3 q, F&& f) {
  const long long zl = max((long long)q.z - 1, 0LL);
  const long long zh = min((long long)q.z + 1, (long long)g.nz - 1);
  if (zl > zh) return;
  for (int ox = -1; ox <= 1; ++ox) {
    const long long x = (long long)q.x + ox;
    if (x < 0 || x >= g.nx) continue;
    for (int oy = -1; oy <= 1; ++oy) {
      const long long y = (long long)q.y + oy;
      if (y < 0 || y >= g.ny) continue;
      f((int)((x * g.ny + y) * g.nz + zl), (int)(zh - zl + 1));
    }
  }
}

// The same walk that stops as soon as f returns true.
template <class F>
__device__ __forceinline__ void for_each_stencil_column_until(const Grid& g, int3 q, F&& f) {
  const long long zl = max((long long)q.z - 1, 0LL);
  const long long zh = min((long long)q.z + 1, (long long)g.nz - 1);
  if (zl > zh) return;
  for (int ox = -1; ox <= 1; ++ox) {
    const long long x = (long long)q.x + ox;
    if (x < 0 || x >= g.nx) continue;
    for (int oy = -1; oy <= 1; ++oy) {
      const long long y = (long long)q.y + oy;
      if (y < 0 || y >= g.ny) continue;
      if (f((int)((x * g.ny + y) * g.nz + zl), (int)(zh - zl + 1))) return;
    }
  }
}

// n / d with the constants of make_udiv (d >= 1).
__device__ __forceinline__ uint32_t udiv(uint32_t n, const UDiv& u) {
  if (u.d <= 1) return n;
  const uint32_t t = __umulhi(u.m, n);
  return (t + ((n - t) >> 1)) >> u.s;
}

// sqrtf(dd) > X, with the clear cases decided from dd against X*X: beyond
// a relative margin of 2e-6 on the square the rounded root lies several
// ulps from X.  Near-ties, and X*X outside the normal range, take the root.
__device__ __forceinline__ bool sqrt_gt(float dd, float X) {
  const float X2 = X * X;
  if (X2 > 1e-30f && X2 < 1e30f) {
    if (dd > X2 * 1.000002f) return true;
    if (dd < X2 * 0.999998f) return false;
  }
  return sqrtf(dd) > X;
}

// make_int3(pos / cell_length): IEEE division then truncation (cvt.rzi).
__device__ __forceinline__ int3 trunc_cell(const Grid& g, float3 p) {
  return make_int3(__float2int_rz(p.x / g.L), __float2int_rz(p.y / g.L), __float2int_rz(p.z / g.L));
}
// make_int3(floorf(pos / cell_length)).
__device__ __forceinline__ int3 floor_cell(const Grid& g, float3 p) {
  return make_int3(__float2int_rz(floorf(p.x / g.L)), __float2int_rz(floorf(p.y / g.L)),
                   __float2int_rz(floorf(p.z / g.L)));
}

// Transcendentals by math mode: MM = 0 calls CUDA's float functions (the
// ones the reference calls); MM = 1 evaluates in double and rounds once,
// which the CPU restatement reproduces bit for bit.
template <int MM> __device__ __forceinline__ float m_cbrt(float x) { return MM ? (float)cbrt((double)x) : cbrtf(x); }
template <int MM> __device__ __forceinline__ float m_exp(float x) { return MM ? (float)exp((double)x) : expf(x); }
template <int MM> __device__ __forceinline__ float m_acos(float x) { return MM ? (float)acos((double)x) : acosf(x); }
template <int MM> __device__ __forceinline__ float m_rsqrt(float x) {
  return MM ? (float)(1.0 / sqrt((double)x)) : rsqrtf(x);
}
template <int MM> __device__ __forceinline__ float m_norm3(float a, float b, float c) {
  if (MM) {
    const double da = a, db = b, dc = c;
    return (float)sqrt(da * da + db * db + dc * dc);
  }
  return norm3df(a, b, c);
}
template <int MM> __device__ __forceinline__ float3 m_normalize3(float3 a) { return mul3s(a, m_rsqrt<MM>(dot3(a, a))); }

// Radius laws, each exactly as the reference writes it.
// compute_delta_pos passes `const int density` and uses double pi
// (Solver.cu:28,311,320-321): cbrtf((3*m) / (4*pi*density)).
template <int MM = 0>
__device__ __forceinline__ float radius_contact(float m, int rho_i) {
  return m_cbrt<MM>((float)((double)(3.0f * m) / (4.0 * GG_PI_D * (double)rho_i)));
}
// find_cover_vector / find_surface use float density, double PI_d
// (GranularSystem.cu:28,518).
template <int MM = 0>
__device__ __forceinline__ float radius_surface(float m, float rho_f) {
  return m_cbrt<MM>((float)((double)(3.0f * m) / (4.0 * GG_PI_D * (double)rho_f)));
}
// split_gpu: all float with the PI macro (Solver.cu:799).
template <int MM = 0>
__device__ __forceinline__ float radius_split(float m, float rho_f) {
  return m_cbrt<MM>((3.0f * m) / ((4.0f * GG_PI_F) * rho_f));
}

__device__ __forceinline__ unsigned int fbits_abs_max(float a, float b) {
  return __float_as_uint(fmaxf(fabsf(a), fabsf(b)));
}

// Warp-aggregated atomicMax of a non-negative float stored as bits.  NaN
// bits compare above every finite value, so a NaN disables pruning.  The
// value only grows, so a warp whose maximum does not exceed a value already
// read skips the atomic: every warp of a large launch would otherwise queue
// on the same address.
__device__ __forceinline__ void warp_max_bits(unsigned int* dst, unsigned int v) {
  v = __reduce_max_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && v > __ldcg(dst)) atomicMax(dst, v);
}

// The same for a whole block of kThreads threads (every thread calls it):
// one fire-and-forget atomic per block, so a large launch puts few
// requests on the one cache line that holds the maximum.
template <int kThreads>
__device__ __forceinline__ void block_max_bits(unsigned int* dst, unsigned int v) {
  __shared__ unsigned int s_max[kThreads / 32];
  v = __reduce_max_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned int m = threadIdx.x < kThreads / 32 ? s_max[threadIdx.x] : 0u;
    m = __reduce_max_sync(0xffffffffu, m);
    if (threadIdx.x == 0 && m) atomicMax(dst, m);
  }
  __syncthreads();  // s_max is reused by the next call
}

// The same for any block of at most 256 threads (a multiple of 32), the
// size read at run time, so that the launch shape can be tuned.
__device__ __forceinline__ void block_max_bits_any(unsigned int* dst, unsigned int v) {
  __shared__ unsigned int s_max[8];
  v = __reduce_max_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned int m = threadIdx.x < (blockDim.x >> 5) ? s_max[threadIdx.x] : 0u;
    m = __reduce_max_sync(0xffffffffu, m);
    if (threadIdx.x == 0 && m) atomicMax(dst, m);
  }
  __syncthreads();  // s_max is reused by the next call
}

__device__ __forceinline__ unsigned int lanemask_lt() {
  unsigned int m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

}  // namespace gg

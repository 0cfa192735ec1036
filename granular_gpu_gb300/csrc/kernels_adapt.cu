// kernels_adapt.cu — surface detection, distance to the surface, adaptive
// merge/split and the compaction that follows.
//
// Replaces GranularSystem::set_surface_particles / find_distance_to_surface
// (GranularSystem.cu:506-699) and Solver::adaptive_sampling with
// merge_mark_gpu, merge_count_gpu, split_gpu and the DArray compactions and
// appends (Solver.cu:526-1242, DArray.hpp:62-155).  No allocation and no
// host round trip except the new particle count.
#include <cmath>

#include <cooperative_groups.h>

#include "common.cuh"

namespace gg {

namespace cg = cooperative_groups;

// ------------------------------------------------------------ surface

// Prefilter of the neighbour test |d| <= 2 (r_i + r_j) with the surface-law
// radius r_j: no contact radius (pos.w, which divides by the density
// truncated to an integer) is below the surface-law radius, so with the
// substep's largest contact radius w_max, a candidate beyond
// R = 2.0002 (r_i + w_max), with a margin far above the roundings of a fused
// dot product, fails the exact test.  Marks, in bit b, the candidates
// c0 + b (b < cn <= 32) within R (R2 = R * R), leaving out i itself.
__device__ __forceinline__ unsigned surface_chunk_mask(const float4* __restrict__ pos, int c0, int cn, int i,
                                                       float3 xi, float R2) {
  unsigned mask = 0u;
#pragma unroll 4
  for (int b = 0; b < cn; ++b) {
    const float3 d = sub3(xi, f3(pos[c0 + b]));
    const float dd = __fmaf_rn(d.x, d.x, __fmaf_rn(d.y, d.y, __fmul_rn(d.z, d.z)));
    mask |= (dd > R2 ? 0u : 1u) << b;
  }
  const unsigned self = (unsigned)(i - c0);
  if (self < 32u) mask &= ~(1u << self);
  return mask;
}

// The nine stencil columns (x, y offsets in units of the signs of the cover
// vector's x and y), most aligned with it first.
__constant__ int kTowards[9][2] = {{1, 1}, {1, 0}, {0, 1}, {0, 0}, {1, -1}, {-1, 1}, {0, -1}, {-1, 0}, {-1, -1}};

template <int MM>
__global__ void __launch_bounds__(256, 6) k_surface(Grid g, int n, const float4* __restrict__ pos,
                                                 const float* __restrict__ rs, const int32_t* __restrict__ cs,
                                                 int32_t* __restrict__ surface, float cone, float cos_cone,
                                                 int min_nb, const unsigned int* __restrict__ rmax_bits,
                                                 const float* __restrict__ mass, float merge_cut,
                                                 float* __restrict__ ld_sum, int32_t* __restrict__ ld_cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float3 xi = f3(pos[i]);
  const int3 q = trunc_cell(g, xi);
  const float ri = rs[i];
  const float Rw = 2.0002f * (ri + __uint_as_float(*rmax_bits));
  const float R2 = Rw * Rw;
  float3 cv = make_float3(0.f, 0.f, 0.f);
  unsigned nn = 0;
  // The merge scan's local density (merge_mark_gpu, Solver.cu:526-653): the
  // mass within the merge radius, the particle itself included, summed in
  // candidate order.  Taken here when the prefilter reaches the merge
  // radius (its cut with the merge scan's own margin), so that the merge
  // scan only looks at candidates after i.
  const bool ldc = ld_cnt && merge_cut * 1.0001f <= R2;
  float ld = 0.0f;
  int lc = 0;
  // Each stencil column is scanned in chunks of 32: the prefilter marks
  // the candidates that may lie within 2 (r_i + r_j) in a mask, and the
  // exact test and the sums run over the marked ones in candidate order.
  for_each_stencil_column(g, q, [&](int k0, int nc) {
    const int j1 = cs[k0 + nc];
    for (int c0 = cs[k0]; c0 < j1; c0 += 32) {
      const int cn = min(32, j1 - c0);
      unsigned mask = surface_chunk_mask(pos, c0, cn, i, xi, R2);
      // the particle itself counts once, in the chunk that holds it
      const unsigned self = (unsigned)(i - c0);
      if (ldc && self < (unsigned)cn) mask |= 1u << self;
      while (mask) {
        const int j = c0 + __ffs(mask) - 1;
        mask &= mask - 1u;
        const float3 d = sub3(xi, f3(pos[j]));
        const float dd = dot3(d, d);
        if (ldc && dd < merge_cut) {
          ld += mass[j];
          ++lc;
        }
        if (j == i || sqrt_gt(dd, 2.0f * (ri + rs[j]))) continue;
        cv = add3(cv, m_normalize3<MM>(d));
        ++nn;
      }
    }
  });
  if (ld_cnt) {
    ld_sum[i] = ld;
    ld_cnt[i] = ldc ? lc : -1;
  }
  if (nn <= (unsigned)min_nb) {
    surface[i] = 1;
    return;
  }
  const float3 c = m_normalize3<MM>(cv);
  // The vote is an OR over the neighbours, so the order they are visited in
  // is free: the stencil columns towards c first, and within a column from
  // the end c.z points to, so that an interior particle meets a neighbour
  // inside the cone early.  acos(d) <= cone is decided from d alone away
  // from cos(cone) (the margin of 1e-5 on d is some 40 times the bound on
  // acosf's error there and over the rounding of cos_cone, computed on the
  // host); near it acos is evaluated.
  const float d_in = cos_cone + 1e-5f, d_out = cos_cone - 1e-5f;
  const int sx = c.x < 0.0f ? -1 : 1, sy = c.y < 0.0f ? -1 : 1;
  const bool up = c.z > 0.0f;
  // (64-bit cell coordinates: q saturates for positions far outside the grid)
  const long long zl = max((long long)q.z - 1, 0LL), zh = min((long long)q.z + 1, (long long)g.nz - 1);
  bool vote = false;
  if (zl <= zh) {
    for (int o = 0; o < 9 && !vote; ++o) {
      const long long x = (long long)q.x + sx * kTowards[o][0], y = (long long)q.y + sy * kTowards[o][1];
      if (x < 0 || x >= g.nx || y < 0 || y >= g.ny) continue;
      const int k0 = (int)((x * g.ny + y) * g.nz + zl);
      const int j0 = cs[k0], j1 = cs[k0 + (int)(zh - zl + 1)];
      const int nch = (j1 - j0 + 31) >> 5;
      for (int ch = 0; ch < nch && !vote; ++ch) {
        const int c0 = j0 + 32 * (up ? nch - 1 - ch : ch);
        unsigned mask = surface_chunk_mask(pos, c0, min(32, j1 - c0), i, xi, R2);
        while (mask) {
          const int bit = up ? 31 - __clz(mask) : __ffs(mask) - 1;
          mask &= ~(1u << bit);
          const int j = c0 + bit;
          float3 b = sub3(f3(pos[j]), xi);
          if (sqrt_gt(dot3(b, b), 2.0f * (ri + rs[j]))) continue;
          b = m_normalize3<MM>(b);
          const float d = dot3(b, c);
          const bool in = d > d_in ? true : (d < d_out ? false : m_acos<MM>(d) <= cone);
          if (in) {
            vote = true;
            break;
          }
        }
      }
    }
  }
  surface[i] = vote ? 0 : 1;
}

void merge_cuts(const gg_system* S, float& f_out, float& T_out);

gg_status surface(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  const int c = S->g.cur;
  prof_begin(S, PC_SURFACE, st);
  auto kern = S->P.math_mode ? k_surface<1> : k_surface<0>;
  float merge_f = 0.0f, merge_cut = 0.0f;
  merge_cuts(S, merge_f, merge_cut);
  kern<<<blocks_for(S->n, 256), 256, 0, st>>>(S->grid, (int)S->n, S->g.pos[c], S->g.rs[c], S->g.cell_start,
                                               S->g.surface, S->P.surface_cone, std::cos(S->P.surface_cone),
                                               S->P.surface_min_neighbors, &S->scal->rmax_bits, S->g.mass[c],
                                               merge_cut, S->g.ld_sum, S->g.ld_cnt);
  count_launches(S, 1);
  prof_end(S, PC_SURFACE, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// Marks the cells that hold a surface particle (by binning key).
__global__ void k_mark_surface_cells(int n, int C, const int32_t* __restrict__ surface,
                                     const uint32_t* __restrict__ keys, uint8_t* __restrict__ cell_surf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = keys[i];
  if (surface[i] != 0 && k < (uint32_t)C) cell_surf[k] = 1;
}

// compute_distance_to_surface, GranularSystem.cu:639-688.  The result is a
// minimum, so the visiting order does not matter, and cells without a
// surface particle (cell_surf 0) hold no candidate: they are skipped.
__global__ void __launch_bounds__(256) k_surfdist(Grid g, int n, const float4* __restrict__ pos,
                                                  const int32_t* __restrict__ surface,
                                                  const int32_t* __restrict__ cs,
                                                  const uint8_t* __restrict__ cell_surf, float* __restrict__ sdist,
                                                  float none) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (surface[i] == 1) {
    sdist[i] = 0.0f;
    return;
  }
  const float3 xi = f3(pos[i]);
  const int3 q = trunc_cell(g, xi);
  float best = none;
  for_each_stencil_column(g, q, [&](int k0, int nc) {
    for (int z = 0; z < nc; ++z) {
      if (!cell_surf[k0 + z]) continue;
      const int j1 = cs[k0 + z + 1];
      for (int j = cs[k0 + z]; j < j1; ++j) {
        if (j == i || surface[j] == 0) continue;
        const float3 d = sub3(xi, f3(pos[j]));
        const float d2 = dot3(d, d);
        if (d2 < best) best = d2;
      }
    }
  });
  sdist[i] = best;
}

gg_status surface_distance(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  prof_begin(S, PC_SURFDIST, st);
  GG_CUDA(cudaMemsetAsync(S->g.cell_surf, 0, (size_t)S->grid.C + 1, st));
  k_mark_surface_cells<<<blocks_for(S->n, 256), 256, 0, st>>>((int)S->n, S->grid.C, S->g.surface, S->g.keys,
                                                              S->g.cell_surf);
  k_surfdist<<<blocks_for(S->n, 256), 256, 0, st>>>(S->grid, (int)S->n, S->g.pos[S->g.cur], S->g.surface,
                                                    S->g.cell_start, S->g.cell_surf, S->g.sdist,
                                                    S->P.no_surface_distance);
  count_launches(S, 2);
  prof_end(S, PC_SURFDIST, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ------------------------------------------------------------ merge

struct MergeArgs {
  Grid g;
  int n;
  const float4* __restrict__ pos;
  const float4* __restrict__ vel;
  const float* __restrict__ mass;
  const int32_t* __restrict__ units;
  const int32_t* __restrict__ surface;
  const float* __restrict__ sdist;
  const int32_t* __restrict__ cs;
  int32_t* __restrict__ remove;
  float* __restrict__ merge;
  int32_t* __restrict__ merge_units;
  float4* __restrict__ merge_vel;
  int32_t* __restrict__ prop;
  float* __restrict__ ldens;
  int32_t* __restrict__ winner;
  float max_mass, min_mass, sdt, target_density;
  double merge_radius;
  float merge_radius_f;  // smallest float above merge_radius: dis < r (double) <=> dis < this
  float merge_r2_cut;    // smallest float whose sqrtf reaches merge_radius_f: dis < it <=> dd < this
  const float* __restrict__ ld_sum;    // density sums of the surface pass, or null
  const int32_t* __restrict__ ld_cnt;
  int lag;                             // merge_cas_lag, in warps
  int32_t* __restrict__ claim_tgt;
  uint8_t* claimed0;                   // claim statuses, iterations ping-pong
  uint8_t* claimed1;
  DevScalars* scal;
};

// merge_mark_gpu (Solver.cu:526-653), scan phase: every thread's neighbour
// scan sees remove[] as it was at kernel start.
// ALL: the merge radius reaches past every candidate of the stencil (the
// reference's 0.035 at r = 0.002), so the chunk masks would mark nearly all
// of them: every candidate is visited, in the same order, and the exact
// radius test alone decides, as in the masked form.
template <bool ALL>
__global__ void __launch_bounds__(256) k_merge_scan(MergeArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  a.winner[i] = 0x7fffffff;
  a.prop[i] = -1;
  const float mi = a.mass[i];
  if (a.surface[i] != 0 || a.remove[i] != 0 || mi < a.min_mass || mi >= a.max_mass || a.sdist[i] < a.sdt) return;
  const float3 xi = f3(a.pos[i]);
  const int3 q = trunc_cell(a.g, xi);
  float closest = 1000.0f;
  int ci = -1;
  float ld = 0.0f;
  int lc = 0;
  const bool sd_bug = a.sdist[i] < a.sdt;  // Solver.cu:578 tests [i]: always false here
  const float pre_cut = a.merge_r2_cut * 1.0001f;
  // With the density taken by the surface pass, only the partners j > i
  // are looked at: the particles are sorted by cell, so they are the
  // candidates from index i + 1 on, visited in the same order.
  const int pre_lc = a.ld_cnt ? a.ld_cnt[i] : -1;
  const bool dens_done = pre_lc >= 0;
  if (dens_done) {
    ld = a.ld_sum[i];
    lc = pre_lc;
  }
  for_each_stencil_column(a.g, q, [&](int k0, int nc) {
    const int j1 = min(a.cs[k0 + nc], a.n);
    for (int c0 = dens_done ? max(a.cs[k0], i + 1) : a.cs[k0]; c0 < j1; c0 += 32) {
      // candidates clearly beyond the merge radius (a fused dot product
      // against the cut with a margin far above its rounding) add nothing:
      // the chunk's mask marks the others, visited in candidate order
      const int cn = min(32, j1 - c0);
      unsigned mask = 0u;
      if (ALL) {
        mask = cn == 32 ? 0xffffffffu : (1u << cn) - 1u;
      } else {
#pragma unroll 4
        for (int b = 0; b < cn; ++b) {
          const float3 d = sub3(xi, f3(a.pos[c0 + b]));
          mask |= (__fmaf_rn(d.x, d.x, __fmaf_rn(d.y, d.y, __fmul_rn(d.z, d.z))) > pre_cut ? 0u : 1u) << b;
        }
      }
      while (mask) {
        const int j = c0 + __ffs(mask) - 1;
        mask &= mask - 1u;
        const float3 d = sub3(xi, f3(a.pos[j]));
        const float dd = dot3(d, d);
        // dis < merge radius (as a float) <=> dd below the smallest square
        // whose rounded root reaches it
        const bool inr = dd < a.merge_r2_cut;
        if (inr && !dens_done) {
          ld += a.mass[j];
          ++lc;
        }
        if (!inr || j <= i || sd_bug || a.remove[j] != 0 || a.surface[j] != 0) continue;
        if (mi + a.mass[j] > a.max_mass) continue;
        const float dis = sqrtf(dd);
        if (dis < closest) {
          closest = dis;
          ci = j;
        }
      }
    }
  });
  if (lc > 0 && ci != -1) {
    a.prop[i] = ci;
    a.ldens[i] = ld / (float)lc;
  }
}

__device__ __forceinline__ bool outer_ok(const MergeArgs& a, int i) {
  return a.surface[i] == 0 && a.sdist[i] > a.sdt;
}

// The compare-and-swaps of merge_mark_gpu (Solver.cu:608-651) race in the
// reference.  They run here under one fixed legal schedule: every scan ends
// before any compare-and-swap; then warps of 32 consecutive threads issue
// theirs in index order, the lanes of a warp together, warp w's first CAS
// (remove[i]) at time w and its second CAS (remove[closest]) at time
// w + lag + 1/2.  So:
//   - proposer i's claim on t can succeed only if t does not propose or
//     t's own first CAS is later: warp(i) + lag < warp(t);
//   - i acts at all (wins its own CAS) only if no proposer that acts has
//     claimed it first;
//   - of the proposers that act and can claim t, the lowest index wins.
// Whether a proposer acts depends on proposers below it only, along chains
// of claims.  The statuses are found by iterating "acts unless an acting
// claimer claims it" from "every proposer acts" until nothing changes: on
// a forest of claims each sweep settles one more level, and levels are few
// (6 to 8 on lattices of 13,824 and 64,000 particles).

__device__ __forceinline__ bool claim_can_win(const MergeArgs& a, int i, int t) {
  return a.prop[t] < 0 || (i >> 5) + a.lag < (t >> 5);
}

// Claims on proposing partners (the only ones that change who acts), and
// iteration 0's statuses: every proposer acts.
__global__ void k_merge_claims(MergeArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int t = a.prop[i];
  int e = -1;
  if (t >= 0 && outer_ok(a, i) && a.prop[t] >= 0 && claim_can_win(a, i, t)) e = t;
  a.claim_tgt[i] = e;
  a.claimed0[i] = 0;
}

// Iterates the claim statuses to their fixed point in one cooperative
// launch (grid-wide barriers between the passes of an iteration); at most
// kMergeMaxIter iterations, after which the error word records it.
__global__ void __launch_bounds__(256) k_merge_resolve(MergeArgs a) {
  cg::grid_group grid = cg::this_grid();
  const int stride = gridDim.x * blockDim.x;
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
  for (int m = 1; m <= kMergeMaxIter; ++m) {
    const uint8_t* prev = (m & 1) ? a.claimed0 : a.claimed1;
    uint8_t* cur = (m & 1) ? a.claimed1 : a.claimed0;
    for (int i = i0; i < a.n; i += stride) cur[i] = 0;
    grid.sync();
    for (int i = i0; i < a.n; i += stride) {
      const int t = a.claim_tgt[i];
      if (t >= 0 && !prev[i]) cur[t] = 1;
    }
    grid.sync();
    int changed = 0;
    for (int i = i0; i < a.n; i += stride) changed |= cur[i] != prev[i];
    changed = __syncthreads_or(changed);
    if (changed && threadIdx.x == 0) atomicOr(&a.scal->merge_changed[m], 1);
    grid.sync();
    if (*((volatile int*)&a.scal->merge_changed[m]) == 0) {
      if (i0 == 0) a.scal->merge_final = m;
      return;
    }
  }
  if (i0 == 0) {
    a.scal->merge_final = kMergeMaxIter;
    atomicOr(&a.scal->error_word, ERR_MERGE_SCHEDULE);
  }
}

__device__ __forceinline__ bool was_claimed(const MergeArgs& a, int i) {
  return ((a.scal->merge_final & 1) ? a.claimed1 : a.claimed0)[i] != 0;
}

__global__ void k_merge_winner(MergeArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int t = a.prop[i];
  if (t < 0 || was_claimed(a, i) || !outer_ok(a, i) || !claim_can_win(a, i, t)) return;
  atomicMin(&a.winner[t], i);
}

// The outcome of the schedule.  A claimed proposer does nothing (its
// claimer set its flag); an acting one sets its own flag, keeps it alone
// when its outer check fails (as the reference does), and merges with its
// partner when it won the partner and the partner passes the check.
__global__ void k_merge_apply(MergeArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int t = a.prop[i];
  if (t < 0 || was_claimed(a, i)) return;
  a.remove[i] = -1;
  if (!outer_ok(a, i)) return;
  if (a.winner[t] != i) {
    a.remove[i] = 0;
    return;
  }
  a.remove[t] = -1;
  if (!outer_ok(a, t)) {
    a.remove[i] = 0;
    return;
  }
  const float mi = a.mass[i], mt = a.mass[t];
  a.merge[t] = mi;
  a.merge[i] = -mi;
  a.merge_units[t] = a.units[i];
  a.merge_units[i] = -a.units[i];
  const float m_t = 1.0f / (mi + mt);
  const float3 vt = smul3(m_t, add3(smul3(mi, f3(a.vel[i])), smul3(mt, f3(a.vel[t]))));
  a.merge_vel[i] = make_float4(-vt.x, -vt.y, -vt.z, 0.f);
  const float df = fminf(1.0f, a.ldens[i] / a.target_density);
  const float3 mv = mul3s(vt, 1.0f + (1.0f - df) * 0.1f);
  a.merge_vel[t] = make_float4(mv.x, mv.y, mv.z, 0.f);
}

// The merge radius as float thresholds: f, the smallest float at or above
// merge_radius (dis < r in double <=> dis < f), and T, the smallest float
// whose rounded root reaches f (sqrtf(dd) < f <=> dd < T).
void merge_cuts(const gg_system* S, float& f_out, float& T_out) {
  float f = (float)S->P.merge_radius;
  if ((double)f < S->P.merge_radius) f = nextafterf(f, INFINITY);
  // dis < r_d  <=>  dis < f when f is the smallest float >= r_d and f != r_d;
  // when f == r_d exactly the comparison is already exact.
  // sqrtf is correctly rounded and monotone here and on the device, so
  // sqrtf(dd) < f  <=>  dd < T for the smallest float T with sqrtf(T) >= f.
  float T = (float)((double)f * (double)f);
  if (!(f > 0.0f)) T = 0.0f;  // no distance is below it (NaN included)
  else if (!std::isfinite(T)) T = INFINITY;
  else {
    while (T > 0.0f && std::sqrt(nextafterf(T, 0.0f)) >= f) T = nextafterf(T, 0.0f);
    while (std::sqrt(T) < f) T = nextafterf(T, INFINITY);
  }
  f_out = f;
  T_out = T;
}

gg_status merge_mark(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  const int c = S->g.cur;
  MergeArgs a;
  a.g = S->grid;
  a.n = (int)S->n;
  a.pos = S->g.pos[c];
  a.vel = S->g.vel[c];
  a.mass = S->g.mass[c];
  a.units = S->g.units[c];
  a.surface = S->g.surface;
  a.sdist = S->g.sdist;
  a.cs = S->g.cell_start;
  a.remove = S->g.remove[c];
  a.merge = S->g.merge[c];
  a.merge_units = S->g.merge_units[c];
  a.merge_vel = S->g.merge_vel;
  a.prop = S->g.prop;
  a.ldens = S->g.ldens;
  a.winner = S->g.winner;
  a.max_mass = S->P.max_mass;
  a.min_mass = S->P.min_merge_mass;
  a.sdt = S->P.surface_dist_threshold;
  a.target_density = S->P.target_density;
  a.merge_radius = S->P.merge_radius;
  merge_cuts(S, a.merge_radius_f, a.merge_r2_cut);
  // the density sums of the surface pass (count -1 where it did not take them)
  a.ld_sum = S->g.ld_sum;
  a.ld_cnt = S->g.ld_cnt;
  a.lag = S->P.merge_cas_lag;
  a.claim_tgt = S->g.claim_tgt;
  a.claimed0 = S->g.claimed;
  a.claimed1 = S->g.claimed + S->cap;
  a.scal = S->scal;
  if (S->merge_resolve_blocks <= 0) {
    int per_sm = 0;
    GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_merge_resolve, 256, 0));
    S->merge_resolve_blocks = std::max(1, per_sm) * S->num_sms;
  }
  const int nb = blocks_for(S->n, 256);
  prof_begin(S, PC_MERGE, st);
  // every candidate of a stencil lies within sqrt(12) cell lengths of the
  // particle, plus what it moved since the grid was built (the predicted
  // step and the sweeps; the ALL form stays exact either way)
  const float reach2 = 12.0f * S->grid.L * S->grid.L * 1.001f;
  if (reach2 < a.merge_r2_cut) k_merge_scan<true><<<nb, 256, 0, st>>>(a);
  else k_merge_scan<false><<<nb, 256, 0, st>>>(a);
  k_merge_claims<<<nb, 256, 0, st>>>(a);
  {
    void* args[] = {&a};
    const int rb = std::min(S->merge_resolve_blocks, nb);
    GG_CUDA(cudaLaunchCooperativeKernel((const void*)k_merge_resolve, dim3(rb), dim3(256), args, 0, st));
  }
  k_merge_winner<<<nb, 256, 0, st>>>(a);
  k_merge_apply<<<nb, 256, 0, st>>>(a);
  count_launches(S, 5);
  prof_end(S, PC_MERGE, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// merge_count_gpu (Solver.cu:658-699).  With the integer ledger the transfer
// of blend step k is floor(M(k+1)/B) - floor(Mk/B) units, so the B
// transfers sum to M exactly.  Radii follow the new mass.
template <int MM>
__global__ void k_merge_count(int n, float4* __restrict__ pos, float4* __restrict__ vel,
                              float* __restrict__ mass, float* __restrict__ rs, int32_t* __restrict__ units,
                              float* __restrict__ merge, int32_t* __restrict__ merge_units,
                              int32_t* __restrict__ merge_count, int32_t* __restrict__ remove,
                              int32_t* __restrict__ als, const float4* __restrict__ merge_vel, int B,
                              int ledger, int rho_i, float rho_f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (remove[i] != -1) return;
  const int old = merge_count[i];
  merge_count[i] = old + 1;
  const float4 mv = merge_vel[i];
  const float3 dvel = div3s(make_float3(mv.x, mv.y, mv.z), (float)B);
  float m;
  if (ledger) {
    const int mu = merge_units[i];
    const long long M = mu < 0 ? -(long long)mu : (long long)mu;
    long long amt = (M * (old + 1)) / B - (M * old) / B;
    if (mu < 0) amt = -amt;
    units[i] = units[i] + (int)amt;
    m = (float)((double)units[i] / (double)(1 << 20));
  } else {
    const float delta = merge[i] / (float)B;
    m = mass[i] + delta;
  }
  mass[i] = m;
  als[i] = 1;
  float4 v = vel[i];
  v.x = v.x + dvel.x;
  v.y = v.y + dvel.y;
  v.z = v.z + dvel.z;
  vel[i] = v;
  pos[i].w = radius_contact<MM>(m, rho_i);
  rs[i] = radius_surface<MM>(m, rho_f);
  if (old + 1 == B) {
    const bool giver = ledger ? (merge_units[i] < 0) : (merge[i] < 0.0f);
    if (giver) {
      remove[i] = 1;
      als[i] = 0;
    } else {
      remove[i] = 0;
    }
    merge_count[i] = 0;
    merge[i] = 0.0f;
    merge_units[i] = 0;
  }
}

gg_status merge_count(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  const int c = S->g.cur;
  prof_begin(S, PC_MERGE, st);
  auto kern = S->P.math_mode ? k_merge_count<1> : k_merge_count<0>;
  kern<<<blocks_for(S->n, 256), 256, 0, st>>>(
      (int)S->n, S->g.pos[c], S->g.vel[c], S->g.mass[c], S->g.rs[c], S->g.units[c], S->g.merge[c],
      S->g.merge_units[c], S->g.merge_count[c], S->g.remove[c], S->g.als[c], S->g.merge_vel, S->P.blend_factor,
      S->P.mass_ledger, S->phys.rho_i, S->phys.density);
  count_launches(S, 1);
  prof_end(S, PC_MERGE, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ------------------------------------------------------------ split

// split_gpu + check_neighborhood (Solver.cu:708-827): decides which surface
// particles split and where the child goes.  Also the keep flags of the
// compaction (remove == 1 is dropped, DArray.hpp:79-90).
template <int MM>
__global__ void __launch_bounds__(256) k_split_mark(Grid g, int n, const float4* __restrict__ pos,
                                                    const float* __restrict__ mass,
                                                    const int32_t* __restrict__ surface,
                                                    const int32_t* __restrict__ remove,
                                                    const int32_t* __restrict__ cs, const int32_t* __restrict__ bcs,
                                                    const float4* __restrict__ bpos, float split_min, float rho_f,
                                                    int32_t* __restrict__ split_flag, int32_t* __restrict__ keep,
                                                    float4* __restrict__ child_pos, uint32_t* __restrict__ cell_claim,
                                                    int32_t* __restrict__ child_cell) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keep[i] = remove[i] != 1;
  split_flag[i] = 0;
  if (cell_claim) child_cell[i] = -1;
  const float mi = mass[i];
  if (remove[i] != 0 || surface[i] != 1 || mi <= split_min) return;
  const float r_i = radius_split<MM>(mi, rho_f);
  const float max_dist = 2.0f * r_i;
  const float3 p = f3(pos[i]);
  const int3 q = trunc_cell(g, p);
  bool found = false;
  int found_cell = 0;
  float3 center = make_float3(0.f, 0.f, 0.f);
  for (int m = 0; m < 27; ++m) {
    const int cx = q.x + m / 9 - 1, cy = q.y + (m % 9) / 3 - 1, cz = q.z + m % 3 - 1;
    const int cell = cell_key(g, cx, cy, cz);
    if (cell == g.C) continue;
    if (!found && m != 13) {
      if (cs[cell] == cs[cell + 1] && bcs[cell] == bcs[cell + 1]) {
        center = make_float3(((float)cx + 0.5f) * g.L, ((float)cy + 0.5f) * g.L, ((float)cz + 0.5f) * g.L);
        found_cell = cell;
        found = true;
      }
    }
    const int j1 = bcs[cell + 1];
    for (int j = bcs[cell]; j < j1; ++j) {
      if (len3(sub3(p, f3(bpos[j]))) < max_dist) return;
    }
  }
  if (!found) return;
  split_flag[i] = 1;
  child_pos[i] = make_float4(center.x, center.y, center.z, 0.f);
  if (cell_claim) {
    // configured mode: the child claims its cell, the lowest parent wins
    child_cell[i] = found_cell;
    atomicMin(&cell_claim[found_cell], (uint32_t)i);
  }
}

// Configured mode (gg_params.split_claim): a parent that lost the claim on
// its child's cell does not split this substep.
__global__ void k_split_claim(int n, const int32_t* __restrict__ child_cell, const uint32_t* __restrict__ cell_claim,
                              int32_t* __restrict__ split_flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !split_flag[i]) return;
  if (cell_claim[child_cell[i]] != (uint32_t)i) split_flag[i] = 0;
}

// Clears the claims of this substep (all flagged parents' cells) once the
// winners are known, so the table is all-free (0xffffffff) at the next.
__global__ void k_split_claim_reset(int n, const int32_t* __restrict__ child_cell, uint32_t* __restrict__ cell_claim) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || child_cell[i] < 0) return;
  cell_claim[child_cell[i]] = 0xffffffffu;
}

struct CompactArgs {
  int n;
  int cap;
  int ledger;
  int rho_i;
  float rho_f;
  const int32_t* __restrict__ keep_slot;
  const int32_t* __restrict__ split_slot;
  const int32_t* __restrict__ split_flag;
  const float4* __restrict__ child_pos;
  const DevScalars* __restrict__ scal;
  int* __restrict__ error_word;
  // in
  const float4* __restrict__ pos;
  const float4* __restrict__ vel;
  const float* __restrict__ mass;
  const float* __restrict__ rs;
  const int32_t* __restrict__ units;
  const int32_t* __restrict__ als;
  const int32_t* __restrict__ mc;
  const float* __restrict__ merge;
  const int32_t* __restrict__ mu;
  const int32_t* __restrict__ remove;
  // out
  float4* __restrict__ pos_o;
  float4* __restrict__ vel_o;
  float* __restrict__ mass_o;
  float* __restrict__ rs_o;
  int32_t* __restrict__ units_o;
  int32_t* __restrict__ als_o;
  int32_t* __restrict__ mc_o;
  float* __restrict__ merge_o;
  int32_t* __restrict__ mu_o;
  int32_t* __restrict__ remove_o;
};

// Stream compaction of every compacted SoA field (order kept) followed by
// the children appended in ascending parent index (Solver.cu:1168-1221).
// A split parent keeps half of its mass (Solver.cu:816-826).
template <int MM>
__global__ void k_compact(CompactArgs a) {
  // nothing removed and nothing split: the compaction would copy every
  // particle to its own slot, so the state stays where it is (the host
  // keeps the current buffers, from the same two counts)
  if (a.scal->n_kept == a.n && a.scal->n_split == 0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  if (a.remove[i] == 1) return;
  const int d = a.keep_slot[i];
  float4 p = a.pos[i];
  float m = a.mass[i];
  float r_s = a.rs[i];
  int u = a.units[i];
  int al = a.als[i];
  if (a.split_flag[i]) {
    float mc_child;
    int uc = 0;
    if (a.ledger) {
      uc = u / 2;
      u = u - uc;
      m = (float)((double)u / (double)(1 << 20));
      mc_child = (float)((double)uc / (double)(1 << 20));
    } else {
      const float h = m / 2.0f;
      m = h;
      mc_child = h;
    }
    p.w = radius_contact<MM>(m, a.rho_i);
    r_s = radius_surface<MM>(m, a.rho_f);
    al = 1;
    const int cd = a.scal->n_kept + a.split_slot[i];
    if (cd < a.cap) {
      const float4 cp = a.child_pos[i];
      a.pos_o[cd] = make_float4(cp.x, cp.y, cp.z, radius_contact<MM>(mc_child, a.rho_i));
      a.vel_o[cd] = a.vel[i];
      a.mass_o[cd] = mc_child;
      a.rs_o[cd] = radius_surface<MM>(mc_child, a.rho_f);
      a.units_o[cd] = uc;
      a.als_o[cd] = 1;
      a.mc_o[cd] = 0;
      a.merge_o[cd] = 0.0f;
      a.mu_o[cd] = 0;
      a.remove_o[cd] = 0;
    } else {
      atomicOr(a.error_word, ERR_CAPACITY);
    }
  }
  a.pos_o[d] = p;
  a.vel_o[d] = a.vel[i];
  a.mass_o[d] = m;
  a.rs_o[d] = r_s;
  a.units_o[d] = u;
  a.als_o[d] = al;
  a.mc_o[d] = a.mc[i];
  a.merge_o[d] = a.merge[i];
  a.mu_o[d] = a.mu[i];
  a.remove_o[d] = a.remove[i];
}

__global__ void k_adapt_counts(DevScalars* s, int n, int cap) {
  const int kept = s->n_kept;
  const int split = s->n_split;
  const int room = cap - kept;
  const int app = split < room ? split : (room > 0 ? room : 0);
  s->n_removed = n - kept;
  s->n_split_appended = app;
  s->n_after = kept + app;
}

gg_status split_and_compact(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  Granular& G = S->g;
  const int c = G.cur, o = c ^ 1;
  const int nb = blocks_for(S->n, 256);
  prof_begin(S, PC_SPLIT, st);
  auto kmark = S->P.math_mode ? k_split_mark<1> : k_split_mark<0>;
  kmark<<<nb, 256, 0, st>>>(S->grid, (int)S->n, G.pos[c], G.mass[c], G.surface, G.remove[c], G.cell_start,
                                   S->b.cell_start, S->b.pos, S->P.split_min_mass, S->phys.density, G.split_flag,
                                   G.keep_flag, G.child_pos, S->P.split_claim ? G.cell_claim : nullptr,
                                   G.child_cell);
  count_launches(S, 1);
  if (S->P.split_claim) {
    k_split_claim<<<nb, 256, 0, st>>>((int)S->n, G.child_cell, G.cell_claim, G.split_flag);
    k_split_claim_reset<<<nb, 256, 0, st>>>((int)S->n, G.child_cell, G.cell_claim);
    count_launches(S, 2);
  }
  prof_end(S, PC_SPLIT, S->n, st);
  prof_begin(S, PC_COMPACT, st);
  gg_status rc = exclusive_scan(G.keep_flag, G.keep_slot, S->n, S->sort, st, &S->scal->n_kept);
  if (rc != GG_OK) return rc;
  rc = exclusive_scan(G.split_flag, G.split_slot, S->n, S->sort, st, &S->scal->n_split);
  if (rc != GG_OK) return rc;
  CompactArgs a;
  a.n = (int)S->n;
  a.cap = (int)S->cap;
  a.ledger = S->P.mass_ledger;
  a.rho_i = S->phys.rho_i;
  a.rho_f = S->phys.density;
  a.keep_slot = G.keep_slot;
  a.split_slot = G.split_slot;
  a.split_flag = G.split_flag;
  a.child_pos = G.child_pos;
  a.scal = S->scal;
  a.error_word = &S->scal->error_word;
  a.pos = G.pos[c]; a.vel = G.vel[c]; a.mass = G.mass[c]; a.rs = G.rs[c]; a.units = G.units[c];
  a.als = G.als[c]; a.mc = G.merge_count[c]; a.merge = G.merge[c]; a.mu = G.merge_units[c];
  a.remove = G.remove[c];
  a.pos_o = G.pos[o]; a.vel_o = G.vel[o]; a.mass_o = G.mass[o]; a.rs_o = G.rs[o]; a.units_o = G.units[o];
  a.als_o = G.als[o]; a.mc_o = G.merge_count[o]; a.merge_o = G.merge[o]; a.mu_o = G.merge_units[o];
  a.remove_o = G.remove[o];
  auto kcomp = S->P.math_mode ? k_compact<1> : k_compact<0>;
  kcomp<<<nb, 256, 0, st>>>(a);
  k_adapt_counts<<<1, 1, 0, st>>>(S->scal, (int)S->n, (int)S->cap);
  count_launches(S, 2);
  prof_end(S, PC_COMPACT, S->n, st);
  // the caller switches to the other buffers once it has read the counts
  // (unless the compaction was the identity)
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg

// kernels_sweep.cu — the Jacobi contact sweep (compute_delta_pos,
// Solver.cu:361-401, with boundary_constraint :272-307 and
// particles_constraint :309-359), race-free.
//
// Semantics.  The reference's scatters into delta_pos[j] are overwritten by
// each thread's final `delta_pos[i] = dp` when the whole grid is resident,
// while its constraint-count increments all land.  This kernel produces that
// outcome with gathers only:
//   delta_i = thread i's own corrections, accumulated in the reference's
//             loop order (27 cells; walls, then particles, by index);
//   n_i     = contacts i finds + particles that find i.
// "j finds i" is decided by i: i's binning cell lies in the stencil of
// trunc(x*_j / L) (the contact test itself is symmetric).  When it does not,
// i hands the count to j through s_extra (rare: only where predicted and
// binned cells disagree).
//
// Pruning.  Cells that cannot hold a partner (farther than r_i + r_max plus
// the largest displacement since binning) are skipped; they contribute
// nothing, so the sum and its order are unchanged.
//
// Kernels.  The default keeps per-particle contact lists across the sweeps
// of a substep (k_sweep_nlist_build / k_sweep_nlist_keep); without lists,
// k_sweep_list scans the 27 cells; k_sweep is the pruned one-thread-per-
// particle scan the autotuner may pick where lists do not pay.
#include <algorithm>
#include <climits>

#include "common.cuh"

namespace gg {

struct SweepArgs {
  Grid g;
  int n;
  int it;
  const float4* __restrict__ xs;
  const float* __restrict__ inv_m;
  const uint32_t* __restrict__ keys;
  const int32_t* __restrict__ cs;
  const int32_t* __restrict__ bcs;
  const float4* __restrict__ bpos;
  float4* __restrict__ delta;
  int32_t* __restrict__ s_extra;
  DevScalars* __restrict__ scal;
  double brad;   // boundary radius (double literal 0.01)
  double fcap;   // friction cap (double literal 0.8)
  float minr;    // floor of the particle radius against walls (0.01f)
  // contact candidate lists (the default sweep)
  int32_t* __restrict__ nl_idx;
  int4* __restrict__ nl_meta;
  float* __restrict__ nl_acc;
  int32_t* __restrict__ nl_queue;
  const uint32_t* __restrict__ cell_inc;
  int cap;
  float skin;
  float eabs;    // bound on the rounding of one position update
  UDiv div_yz, div_z;  // division by ny * nz and by nz (binning cell of a key)
  // batched scenes: scene of a particle = its x* slab, floor(x / width);
  // each scene has its own friction cap (null: a.fcap for every particle)
  const float* __restrict__ scene_fcap;
  float scene_inv_w;
  int n_scenes;
  // configured mode (gg_params.contact_law): substep-start positions for
  // the friction law and its output, the summed friction corrections and
  // their count (both null with the reference's law)
  const float4* __restrict__ pos0;
  float4* __restrict__ fdelta;
};

// The kernels' template argument MM: bit 0 the math mode (0 CUDA's
// functions, 1 rounded once from double), bit 1 the contact law (0 the
// reference's, 1 Coulomb friction).

// Which of the three cell columns [c-1, c, c+1] along one axis can hold a
// partner: bit k set for offset k-1.  Cells are [cL, (c+1)L) in binning
// coordinates; a partner binned there is within R of x.
__device__ __forceinline__ unsigned axis_mask(float x, int q, float L, float R) {
  unsigned m = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float lo = (float)(q + k - 1) * L;
    const float hi = (float)(q + k) * L;
    // NaN in x or R leaves the column in (never prunes)
    if (!(x < lo - R) && !(x > hi + R)) m |= 1u << k;
  }
  return m;
}

// Everything one target particle needs for its sweep.
struct Target {
  float3 x;
  float rc, rb;
  float Bf;       // 0.01 + r_b in double (Solver.cu:283), rounded to float
  float Bru;      // Bd rounded up to float: (double)d < Bd  <=>  d < Bru for every float d
  float capBru;   // (r_b + 0.01) * 0.8 in double, rounded up to float (same use)
  float Bcut;     // conservative float cut for the wall test
  float inv_m;
  int3 q;         // query cell trunc(x*/L)
  bool binned;
  int cx, cy, cz; // binning cell
  unsigned pm[3], bm[3];
  float fcapf;    // friction cap factor (0.8 in the reference; per scene in a batch), as float
  float3 x0;      // position at the substep's start (Coulomb law only)
  // Coulomb law: the friction corrections and their count, averaged on
  // their own by the apply kernel (mutable: the contact functions take the
  // target as const and add to these)
  mutable float3 df;
  mutable int fc;
};

// The friction cap in double, as the reference's comparisons and ratios use
// it (rare paths only, so targets carry the float copy).
__device__ __forceinline__ double target_fcap(const SweepArgs& a, const Target& t) {
  if (!a.scene_fcap) return a.fcap;
  const int s = min(max(__float2int_rz(t.x.x * a.scene_inv_w), 0), a.n_scenes - 1);
  return (double)a.scene_fcap[s];
}
// 0.01 + r_b in double (Solver.cu:283).
__device__ __forceinline__ double target_bd(const SweepArgs& a, const Target& t) { return a.brad + (double)t.rb; }

// The per-target values every sweep needs (no pruning masks).
__device__ __forceinline__ void make_target_lite(const SweepArgs& a, int i, float4 xi4, Target& t) {
  const Grid& g = a.g;
  t.x = f3(xi4);
  t.rc = xi4.w;
  t.rb = fmaxf(t.rc, a.minr);
  const double Bd = target_bd(a, t);
  t.Bru = __double2float_ru(Bd);
  const double fcap = target_fcap(a, t);
  t.fcapf = (float)fcap;
  t.capBru = __double2float_ru(((double)t.rb + a.brad) * fcap);
  t.Bf = (float)Bd;
  t.Bcut = t.Bf * t.Bf * 1.0001f;
  t.inv_m = a.inv_m[i];
  t.x0 = a.pos0 ? f3(a.pos0[i]) : t.x;
  t.df = make_float3(0.f, 0.f, 0.f);
  t.fc = 0;
  t.q = trunc_cell(g, t.x);
  const uint32_t key = a.keys[i];
  t.binned = (int)key < g.C;
  t.cx = t.cy = t.cz = 0;
  if (t.binned) {
    t.cx = (int)udiv(key, a.div_yz);
    const int r = (int)key - t.cx * g.ny * g.nz;
    t.cy = (int)udiv((uint32_t)r, a.div_z);
    t.cz = r - t.cy * g.nz;
  }
}

// Pruning masks: the stencil columns that can hold a partner within
// r_i + r_max plus the displacement since binning, or a wall within reach.
__device__ __forceinline__ void target_masks(const SweepArgs& a, Target& t) {
  const Grid& g = a.g;
  float disp = __uint_as_float(a.scal->disp0_bits);
  for (int k = 0; k < a.it; ++k) disp += __uint_as_float(a.scal->inc_bits[k]);
  const float rmax = __uint_as_float(a.scal->rmax_bits);
  const float ax = fmaxf(fmaxf(fabsf(t.x.x), fabsf(t.x.y)), fabsf(t.x.z));
  const float slack = 4e-6f * (ax + 1.0f) + 1e-5f * g.L;
  const float Rp = (t.rc + rmax + disp) * 1.0001f + slack;
  const float Rb = t.Bf * 1.0001f + slack;
  t.pm[0] = axis_mask(t.x.x, t.q.x, g.L, Rp);
  t.pm[1] = axis_mask(t.x.y, t.q.y, g.L, Rp);
  t.pm[2] = axis_mask(t.x.z, t.q.z, g.L, Rp);
  t.bm[0] = axis_mask(t.x.x, t.q.x, g.L, Rb);
  t.bm[1] = axis_mask(t.x.y, t.q.y, g.L, Rb);
  t.bm[2] = axis_mask(t.x.z, t.q.z, g.L, Rb);
}

__device__ __forceinline__ void make_target(const SweepArgs& a, int i, float4 xi4, Target& t) {
  make_target_lite(a, i, xi4, t);
  target_masks(a, t);
}

// boundary_constraint for one wall particle within the float cut
// (Solver.cu:272-307).  A float d compares below a double D exactly when it
// compares below D rounded up to float (no float lies strictly between the
// two roundings of D), so the double comparisons are decided in float.
template <int MM>
__device__ __forceinline__ void wall_contact(const SweepArgs& a, const Target& t, float4 pb, float3& dp, int& c) {
  const float bx = t.x.x - pb.x, by = t.x.y - pb.y, bz = t.x.z - pb.z;
  const float dis = m_norm3<(MM & 1)>(bx, by, bz);
  if (!(dis < t.Bru)) return;  // mag < 0
  const float mag = (float)((double)dis - target_bd(a, t));
  const float3 p12 = make_float3(bx, by, bz);
  const float3 dpi = smul3(mag / dis, p12);
  if (MM & 2) {
    // Coulomb law: the normal push, and the friction target: cancel the
    // tangential displacement since the substep began (the apply kernel
    // limits the averaged friction by the particle's normal corrections)
    const float3 drel = sub3(t.x, t.x0);
    const float dn = dot3(drel, p12) / (dis * dis);
    const float3 dtan = sub3(drel, smul3(dn, p12));
    dp = sub3(dp, dpi);
    t.df = sub3(t.df, dtan);
    ++t.fc;
    ++c;
    return;
  }
  const float3 perp = sub3(dpi, div3s(smul3(dot3(dpi, p12), p12), dis * dis));
  const float pn = m_norm3<(MM & 1)>(perp.x, perp.y, perp.z);
  if (pn < t.capBru) {
    dp = sub3(dp, dpi);
  } else {
    const float minf = (float)fmin((a.brad + (double)t.rb) * target_fcap(a, t) / (double)pn, 1.0);
    dp = sub3(dp, mul3s(dpi, minf));
  }
  ++c;
}

__device__ __forceinline__ bool wall_near(const Target& t, float4 pb) {
  const float bx = t.x.x - pb.x, by = t.x.y - pb.y, bz = t.x.z - pb.z;
  const float d2 = __fmaf_rn(bx, bx, __fmaf_rn(by, by, __fmul_rn(bz, bz)));
  return !(d2 > t.Bcut);
}

// boundary_constraint over one cell's wall particles.
template <int MM>
__device__ __forceinline__ void wall_cell(const SweepArgs& a, const Target& t, int cell, float3& dp, int& c) {
  const int b1 = a.bcs[cell + 1];
  for (int b = a.bcs[cell]; b < b1; ++b) {
    const float4 pb = a.bpos[b];
    if (wall_near(t, pb)) wall_contact<MM>(a, t, pb, dp, c);
  }
}

// particles_constraint for one candidate j (Solver.cu:314-357).
template <int MM, class InvF>
__device__ __forceinline__ void particle_pair_f(const SweepArgs& a, const Target& t, int j, float4 xj4, InvF&& inv_of,
                                                float3& dp, int& c, int& s_loc) {
  const float dx = t.x.x - xj4.x, dy = t.x.y - xj4.y, dz = t.x.z - xj4.z;
  const float rr = t.rc + xj4.w;
  const float d2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
  if (d2 > rr * rr * 1.0001f) return;
  const float dis = m_norm3<(MM & 1)>(dx, dy, dz);
  const float mag = rr - dis;
  if (!(mag >= 0.0f)) return;
  const float inv_mj = inv_of();
  // (float)(1.0 / (double)s) equals the IEEE float reciprocal of s (no
  // double-rounding case exists for 24-bit significands).
  const float inv_sum = __frcp_rn(t.inv_m + inv_mj);
  const float tt = mag / dis;
  const float3 p12 = make_float3(dx, dy, dz);
  if (MM & 2) {
    // Coulomb law: i's share of the normal push, and its share of cancelling
    // the relative tangential displacement since the substep began (limited
    // by the apply kernel)
    const float w = inv_sum * t.inv_m;
    const float4 xj0 = a.pos0[j];
    const float3 drel = sub3(sub3(t.x, t.x0), make_float3(xj4.x - xj0.x, xj4.y - xj0.y, xj4.z - xj0.z));
    const float dn = dot3(drel, p12) / (dis * dis);
    const float3 dtan = sub3(drel, smul3(dn, p12));
    dp = add3(dp, smul3(w * tt, p12));
    t.df = sub3(t.df, smul3(w, dtan));
    ++t.fc;
  } else {
  const float3 dpi = smul3((-inv_sum * t.inv_m) * tt, p12);
  const float3 dpj = smul3((inv_sum * inv_mj) * tt, p12);
  const float3 dpij = sub3(dpi, dpj);
  const float w = inv_sum * t.inv_m;
  const float capf = rr * t.fcapf;
  // The tangential part `perp` of dpij (which is parallel to p12) is
  // rounding noise: |perp| <= 2 (|a| + |b|) dis (1 + 8 eps) with a, b the
  // two scalar factors above.  When that bound is below the cap the
  // reference's branch is decided and perp need not be formed.
  const float bound = 2.0001f * (fabsf((-inv_sum * t.inv_m) * tt) + fabsf((inv_sum * inv_mj) * tt)) * dis;
  bool within;
  float pn = 0.0f;
  if (bound < capf * 0.999f) {
    within = true;
  } else {
    const float3 perp = sub3(dpij, div3s(smul3(dot3(dpij, p12), p12), dis * dis));
    pn = m_norm3<(MM & 1)>(perp.x, perp.y, perp.z);
    // (double)pn < (double)rr * 0.8, decided in float when clear-cut
    if (pn < capf * 0.999999f) within = true;
    else if (pn > capf * 1.000001f) within = false;
    else within = (double)pn < (double)rr * target_fcap(a, t);
  }
  if (within) {
    dp = sub3(dp, smul3(w, dpij));
  } else {
    const float minf = (float)fmin((double)rr * target_fcap(a, t) / (double)pn, 1.0);
    dp = sub3(dp, mul3s(smul3(w, dpij), minf));
  }
  }
  ++c;
  const int3 qj = trunc_cell(a.g, make_float3(xj4.x, xj4.y, xj4.z));
  // |c - qj| <= 1 per axis, as one unsigned window test: c is a binning
  // cell (0 <= c < n < 2^31), so c + 1 - qj stays below 2^32 for every int
  // qj and lies in [0, 2] exactly when qj is within one cell of c.
  const bool j_finds_i = t.binned && (unsigned)t.cx + 1u - (unsigned)qj.x <= 2u &&
                         (unsigned)t.cy + 1u - (unsigned)qj.y <= 2u && (unsigned)t.cz + 1u - (unsigned)qj.z <= 2u;
  if (j_finds_i) ++s_loc;
  else atomicAdd(&a.s_extra[j], 1);
}

template <int MM>
__device__ __forceinline__ void particle_pair(const SweepArgs& a, const Target& t, int j, float4 xj4,
                                              const float* inv_src, int inv_idx, float3& dp, int& c,
                                              int& s_loc) {
  particle_pair_f<MM>(a, t, j, xj4, [&]() { return inv_src[inv_idx]; }, dp, c, s_loc);
}

__device__ __forceinline__ bool use_cell(const unsigned* m, int ox, int oy, int oz) {
  return ((m[0] >> ox) & (m[1] >> oy) & (m[2] >> oz) & 1u) != 0;
}

// The reference loop for one target over global memory.
template <int MM>
__device__ void sweep_global(const SweepArgs& a, int i, const Target& t) {
  const Grid& g = a.g;
  float3 dp = make_float3(0.f, 0.f, 0.f);
  int c = 0, s_loc = 0;
  for (int ox = 0; ox < 3; ++ox) {
    for (int oy = 0; oy < 3; ++oy) {
      for (int oz = 0; oz < 3; ++oz) {
        const bool usep = use_cell(t.pm, ox, oy, oz);
        const bool useb = use_cell(t.bm, ox, oy, oz);
        if (!usep && !useb) continue;
        const int cell = cell_key(g, t.q.x + ox - 1, t.q.y + oy - 1, t.q.z + oz - 1);
        if (cell == g.C) continue;
        if (useb) wall_cell<MM>(a, t, cell, dp, c);
        if (usep) {
          const int j1 = a.cs[cell + 1];
          for (int j = a.cs[cell]; j < j1; ++j) {
            if (j == i) continue;
            particle_pair<MM>(a, t, j, a.xs[j], a.inv_m, j, dp, c, s_loc);
          }
        }
      }
    }
  }
  a.delta[i] = make_float4(dp.x, dp.y, dp.z, __int_as_float((c & 0xffff) | (s_loc << 16)));
  if (MM & 2) a.fdelta[i] = make_float4(t.df.x, t.df.y, t.df.z, __int_as_float(t.fc));
}

template <int MM>
__global__ void __launch_bounds__(256) k_sweep(SweepArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  Target t;
  make_target(a, i, a.xs[i], t);
  sweep_global<MM>(a, i, t);
}

// ------------------------------------------------------------ listed scan
//
// The reference sums a particle's corrections over its 27 cells in the
// order m = (dx+1)*9 + (dy+1)*3 + (dz+1) and, inside a cell, walls then
// particles by index.  Without contact lists (nlist_skin = 0) each lane
// walks its 27 cells in that order and keeps the candidates that pass a
// cheap distance test in a short list in shared memory (in order); the
// lanes then run the exact test on their k-th listed candidate together,
// which keeps the expensive contact body convergent across the warp.

constexpr int kWarpList = 32;      // listed candidates per lane before a flush
constexpr int kWarpThreads = 256;

template <int MM>
__device__ __forceinline__ void process_entry(const SweepArgs& a, const Target& t, int i, int e, float3& dp,
                                              int& c, int& s_loc) {
  if (e < 0) {
    // one wall particle (the exact test of boundary_constraint)
    wall_contact<MM>(a, t, a.bpos[-e - 1], dp, c);
  } else {
    particle_pair<MM>(a, t, e, a.xs[e], a.inv_m, e, dp, c, s_loc);
  }
}

// One thread per particle over all 27 cells (no per-lane pruning, so the
// lanes of a warp walk the same cell sequence), with the candidates that
// pass the cheap distance test listed in order and processed by all lanes
// together afterwards.
template <int MM>
__global__ void __launch_bounds__(kWarpThreads) k_sweep_list(SweepArgs a) {
  __shared__ int s_list[kWarpThreads / 32][kWarpList][32];
  const Grid& g = a.g;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * kWarpThreads + threadIdx.x;
  if (i >= a.n) return;
  Target t;
  make_target(a, i, a.xs[i], t);
  float3 dp = make_float3(0.f, 0.f, 0.f);
  int c = 0, s_loc = 0, cnt = 0;
  auto flush = [&]() {
    for (int k = 0; k < cnt; ++k) process_entry<MM>(a, t, i, s_list[w][k][lane], dp, c, s_loc);
    cnt = 0;
  };
  auto push = [&](int e) {
    if (cnt == kWarpList) flush();
    s_list[w][cnt++][lane] = e;
  };
  for (int m = 0; m < 27; ++m) {
    const int ox = m / 9, oy = (m % 9) / 3, oz = m % 3;
    const int cell = cell_key(g, t.q.x + ox - 1, t.q.y + oy - 1, t.q.z + oz - 1);
    if (cell == g.C) continue;
    if (use_cell(t.bm, ox, oy, oz)) {
      const int b1 = a.bcs[cell + 1];
      for (int b = a.bcs[cell]; b < b1; ++b) {
        const float4 pb = a.bpos[b];
        const float bx = t.x.x - pb.x, by = t.x.y - pb.y, bz = t.x.z - pb.z;
        const float d2 = __fmaf_rn(bx, bx, __fmaf_rn(by, by, __fmul_rn(bz, bz)));
        if (!(d2 > t.Bcut)) push(-b - 1);
      }
    }
    const int j1 = a.cs[cell + 1];
    for (int j = a.cs[cell]; j < j1; ++j) {
      const float4 xj = a.xs[j];
      const float dx = t.x.x - xj.x, dy = t.x.y - xj.y, dz = t.x.z - xj.z;
      const float rr = t.rc + xj.w;
      const float d2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
      if (!(d2 > rr * rr * 1.0001f) && j != i) push(j);
    }
  }
  flush();
  a.delta[i] = make_float4(dp.x, dp.y, dp.z, __int_as_float((c & 0xffff) | (s_loc << 16)));
  if (MM & 2) a.fdelta[i] = make_float4(t.df.x, t.df.y, t.df.z, __int_as_float(t.fc));
}

// ------------------------------------------------------------ listed sweep
//
// The grid is fixed for all sweeps of a substep and particles move little
// between sweeps, so each particle keeps the candidates of its stencil that
// lie within r_i + r_j + skin (walls within 0.01 + r_b + skin), in the
// reference's order, and runs the contact test on that list only.
//
// A list built at sweep t stays exact at sweep s while the particle's query
// cell (hence its stencil) is unchanged and
//   A * 1.0001 + 4 e < skin,   A = sum over sweeps u in [t, s) of 2 (N_u + sqrt(3) e),
// where N_u bounds the length of the x* increment of sweep u of the particle
// and of every particle binned in its stencil, and e bounds the rounding of
// one coordinate's position update.  A candidate left out was farther than
// r_i + r_j + skin and has since closed in by less than the skin, so it is
// still no contact: the corrections, their order and the counts are those
// of the full scan.  N_u is the sweep's global maximum increment length when
// that is small enough, else the largest per-cell maximum (recorded by the
// apply kernel) over the 27 stencil cells and the particle's own cell.
// Lists whose bound runs out are rebuilt by their own thread; the others are
// kept.

// The listed candidates in order, with the next entry's gathers issued
// before the current one is processed.  entry(k) gives the k-th entry: a
// particle index, or -(wall index) - 1.
__device__ __forceinline__ void fetch_entry(const SweepArgs& a, int e, float4& p, float& im) {
  if (e >= 0) {
    p = a.xs[e];
    im = a.inv_m[e];
  } else if (e != INT_MIN) {
    p = a.bpos[-e - 1];
  }
}

template <int MM, class EntryF>
__device__ __forceinline__ void apply_entries(const SweepArgs& a, const Target& t, int cnt, EntryF&& entry,
                                              float3& dp, int& c, int& s_loc) {
  if (cnt <= 0) return;
  int e_next = entry(0);
  int e_after = cnt > 1 ? entry(1) : INT_MIN;
  float4 p_next = make_float4(0.f, 0.f, 0.f, 0.f);
  float im_next = 0.0f;
  fetch_entry(a, e_next, p_next, im_next);
  for (int k = 0; k < cnt; ++k) {
    const int e = e_next;
    const float4 p = p_next;
    const float im = im_next;
    e_next = e_after;
    fetch_entry(a, e_next, p_next, im_next);
    e_after = (k + 2 < cnt) ? entry(k + 2) : INT_MIN;
    if (e >= 0) {
      particle_pair_f<MM>(a, t, e, p, [&]() { return im; }, dp, c, s_loc);
    } else if (wall_near(t, p)) {
      wall_contact<MM>(a, t, p, dp, c);
    }
  }
}

__device__ __forceinline__ bool nlist_bound_ok(const SweepArgs& a, float A) {
  return A * 1.0001f + 4.0f * a.eabs < a.skin;
}

// One sweep's share of the bound A for an increment-length bound N.
__device__ __forceinline__ float nlist_step(const SweepArgs& a, float N) { return 2.0f * (N + 1.7320509f * a.eabs); }

// Largest per-cell increment of the last sweep over the stencil of q and the
// particle's own binning cell.  Every cell_inc entry holds the largest
// increment over its cell and the cell's two z neighbours (k_apply), so the
// stencil's 27 cells are covered by the nine entries of its columns at q.z;
// the own cell adds its entry when it is not one of the 27 (the entry bounds
// its increment from above).  A query cell outside the grid in z reads the
// stencil's cells one by one (entries that may bound from above as well).
__device__ __forceinline__ float nlist_cell_bound(const SweepArgs& a, int3 q, uint32_t own_key) {
  const Grid& g = a.g;
  uint32_t m = 0u;
  if (q.z >= 0 && q.z < g.nz) {
    bool own_in = false;
    for (int ox = -1; ox <= 1; ++ox)
      for (int oy = -1; oy <= 1; ++oy) {
        const int c = cell_key(g, q.x + ox, q.y + oy, q.z);
        if (c == g.C) continue;
        m = max(m, a.cell_inc[c]);
        own_in |= own_key == (uint32_t)c || (own_key == (uint32_t)(c - 1) && q.z > 0) ||
                  (own_key == (uint32_t)(c + 1) && q.z < g.nz - 1);
      }
    if (!own_in) m = max(m, a.cell_inc[own_key]);
    return __uint_as_float(m);
  }
  m = a.cell_inc[own_key];
  for (int ox = -1; ox <= 1; ++ox)
    for (int oy = -1; oy <= 1; ++oy) {
      const int c0 = cell_key(g, q.x + ox, q.y + oy, q.z - 1);
      const int c1 = cell_key(g, q.x + ox, q.y + oy, q.z);
      const int c2 = cell_key(g, q.x + ox, q.y + oy, q.z + 1);
      if (c0 != g.C) m = max(m, a.cell_inc[c0]);
      if (c1 != g.C) m = max(m, a.cell_inc[c1]);
      if (c2 != g.C) m = max(m, a.cell_inc[c2]);
    }
  return __uint_as_float(m);
}

// Sweeps after the first: particles whose list is still exact run it; the
// others are queued for k_sweep_nlist_build.
// 5 resident blocks of 256 (48 registers; the per-target state carries no
// double, and a few bytes spill): about 2 % faster than 4 blocks at 64.
template <int MM>
__global__ void __launch_bounds__(256, 5) k_sweep_nlist_keep(SweepArgs a) {
  const Grid& g = a.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool rebuild = false;
  if (i < a.n) {
    const float4 xi4 = a.xs[i];
    const int3 q = trunc_cell(g, f3(xi4));
    const int4 m = a.nl_meta[i];
    bool keep = false;
    if (m.w >= 0 && m.x == q.x && m.y == q.y && m.z == q.z) {
      const float A0 = a.nl_acc[i];
      float A = A0 + nlist_step(a, __uint_as_float(a.scal->inc_norm_bits[a.it - 1]));
      if (!nlist_bound_ok(a, A)) A = A0 + nlist_step(a, nlist_cell_bound(a, q, a.keys[i]));
      if (nlist_bound_ok(a, A)) {
        keep = true;
        a.nl_acc[i] = A;
      }
    }
    if (keep) {
      Target t;
      make_target_lite(a, i, xi4, t);
      float3 dp = make_float3(0.f, 0.f, 0.f);
      int c = 0, s_loc = 0;
      const int32_t* __restrict__ li = a.nl_idx + i;
      apply_entries<MM>(a, t, m.w, [&](int k) { return __ldcs(li + (size_t)k * a.cap); }, dp, c, s_loc);
      a.delta[i] = make_float4(dp.x, dp.y, dp.z, __int_as_float((c & 0xffff) | (s_loc << 16)));
      if (MM & 2) a.fdelta[i] = make_float4(t.df.x, t.df.y, t.df.z, __int_as_float(t.fc));
    } else {
      rebuild = true;
    }
  }
  // The block's rebuilds go to the queue together, in index order: the
  // rebuild kernel then takes neighbouring particles into one warp (warps
  // appending on their own interleave the regions all SMs work on).
  __shared__ int s_cnt[8], s_base;
  const unsigned bal = __ballot_sync(0xffffffffu, rebuild);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) s_cnt[w] = __popc(bal);
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      const int c = s_cnt[k];
      s_cnt[k] = tot;
      tot += c;
    }
    s_base = tot ? atomicAdd(&a.scal->nl_queued[a.it], tot) : 0;
  }
  __syncthreads();
  if (rebuild) a.nl_queue[s_base + s_cnt[w] + __popc(bal & lanemask_lt())] = i;
}

// List build: scan the 27 cells in the reference order, write the
// candidates within reach of the skin to the particle's list as they are
// found, then run the list.  Every particle at the first sweep of a substep;
// the queued ones later.
constexpr int kBuildThreads = 128;

// 8 resident blocks of 128 (64 registers, a few bytes spilled): the queued
// rebuilds are latency-bound, and the extra warps hide more than the spills
// cost (72 registers and 7 blocks measured 3 % slower over the sweeps).
template <int MM>
__global__ void __launch_bounds__(kBuildThreads, 8) k_sweep_nlist_build(SweepArgs a, int queued) {
  const Grid& g = a.g;
  const int lane = threadIdx.x & 31;
  const int total = queued ? a.scal->nl_queued[a.it] : a.n;
  for (int base = blockIdx.x * kBuildThreads; base < total; base += gridDim.x * kBuildThreads) {
    const int slot = base + threadIdx.x;
    const bool act = slot < total;
    {
      const unsigned bal = __ballot_sync(0xffffffffu, act);
      if (lane == 0 && bal) atomicAdd(&a.scal->nlist_rebuilds, (unsigned long long)__popc(bal));
    }
    if (!act) continue;
    const int i = queued ? a.nl_queue[slot] : slot;
    Target t;
    make_target_lite(a, i, a.xs[i], t);
    const float Bs = t.Bf + a.skin;
    const float Bs2 = Bs * Bs * 1.0001f;
    const float rcs = t.rc + a.skin;
    int cnt = 0;
    int32_t* __restrict__ li = a.nl_idx + i;
    auto push = [&](int e) {
      if (cnt < kNlistMax) li[(size_t)cnt * a.cap] = e;
      ++cnt;
    };
    // candidates in chunks of 32: a mask of those within the reach of the
    // largest contact radius of the substep, then, in index order, the
    // exact reach test for each and the pushes
    const float rmax = __uint_as_float(a.scal->rmax_bits);
    const float wide = (rcs + rmax) * (rcs + rmax) * 1.0001f;
    auto scan_particles = [&](int j0, int j1) {
      for (int c0 = j0; c0 < j1; c0 += 32) {
        const int cn = min(32, j1 - c0);
        unsigned mask = 0u;
#pragma unroll 4
        for (int b = 0; b < cn; ++b) {
          const float4 xj = a.xs[c0 + b];
          const float dx = t.x.x - xj.x, dy = t.x.y - xj.y, dz = t.x.z - xj.z;
          const float d2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
          mask |= (d2 > wide ? 0u : 1u) << b;
        }
        const unsigned self = (unsigned)(i - c0);
        if (self < 32u) mask &= ~(1u << self);
        while (mask) {
          const int j = c0 + __ffs(mask) - 1;
          mask &= mask - 1u;
          const float4 xj = a.xs[j];
          const float dx = t.x.x - xj.x, dy = t.x.y - xj.y, dz = t.x.z - xj.z;
          const float rs = rcs + xj.w;
          const float d2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
          if (!(d2 > rs * rs * 1.0001f)) push(j);
        }
      }
    };
    for_each_stencil_column(g, t.q, [&](int k0, int nc) {
      if (a.bcs[k0] == a.bcs[k0 + nc]) {
        // no walls in this column: its particles in index order
        scan_particles(a.cs[k0], a.cs[k0 + nc]);
        return;
      }
      for (int z = 0; z < nc; ++z) {
        const int b1 = a.bcs[k0 + z + 1];
        for (int b = a.bcs[k0 + z]; b < b1; ++b) {
          const float4 pb = a.bpos[b];
          const float bx = t.x.x - pb.x, by = t.x.y - pb.y, bz = t.x.z - pb.z;
          const float d2 = __fmaf_rn(bx, bx, __fmaf_rn(by, by, __fmul_rn(bz, bz)));
          if (!(d2 > Bs2)) push(-b - 1);
        }
        scan_particles(a.cs[k0 + z], a.cs[k0 + z + 1]);
      }
    });
    if (cnt > kNlistMax) {
      // too many candidates to list: full scan, and again at the next sweep
      a.nl_meta[i] = make_int4(t.q.x, t.q.y, t.q.z, -1);
      target_masks(a, t);
      sweep_global<MM>(a, i, t);
      continue;
    }
    a.nl_meta[i] = make_int4(t.q.x, t.q.y, t.q.z, cnt);
    a.nl_acc[i] = 0.0f;
    float3 dp = make_float3(0.f, 0.f, 0.f);
    int c = 0, s_loc = 0;
    // the list this thread just wrote (its own stores: read back in order)
    apply_entries<MM>(a, t, cnt, [&](int k) { return li[(size_t)k * a.cap]; }, dp, c, s_loc);
    a.delta[i] = make_float4(dp.x, dp.y, dp.z, __int_as_float((c & 0xffff) | (s_loc << 16)));
    if (MM & 2) a.fdelta[i] = make_float4(t.df.x, t.df.y, t.df.z, __int_as_float(t.fc));
  }
}

gg_status sweep(gg_system* S, int it, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  SweepArgs a;
  a.g = S->grid;
  a.n = (int)S->n;
  a.it = it;
  a.xs = S->g.xs;
  a.inv_m = S->g.inv_m;
  a.keys = S->g.keys;
  a.cs = S->g.cell_start;
  a.bcs = S->b.cell_start;
  a.bpos = S->b.pos;
  a.delta = S->g.delta;
  a.s_extra = S->g.s_extra;
  a.scal = S->scal;
  a.brad = S->P.boundary_radius;
  a.fcap = S->P.friction_cap;
  a.scene_fcap = S->scene_fcap;
  a.scene_inv_w = S->scene_width > 0.0f ? 1.0f / S->scene_width : 0.0f;
  a.n_scenes = S->n_scenes;
  a.minr = S->P.boundary_min_radius;
  const bool coulomb = S->P.contact_law == 1;
  a.pos0 = coulomb ? S->g.pos[S->g.cur] : nullptr;
  a.fdelta = coulomb ? S->g.fdelta : nullptr;
  const int mm = (S->P.math_mode ? 1 : 0) | (coulomb ? 2 : 0);  // the kernels' template argument
  a.nl_idx = S->g.nl_idx;
  a.nl_meta = S->g.nl_meta;
  a.nl_acc = S->g.nl_acc;
  a.nl_queue = S->g.nl_queue;
  a.cell_inc = S->g.cell_inc;
  a.cap = (int)S->cap;
  a.skin = S->nl_skin;
  a.div_yz = make_udiv((uint32_t)(S->grid.ny * S->grid.nz));
  a.div_z = make_udiv((uint32_t)S->grid.nz);
  {
    // half an ulp of the largest in-grid coordinate, with a margin
    const float ext = S->grid.L * (float)std::max(S->grid.nx, std::max(S->grid.ny, S->grid.nz));
    a.eabs = 2.5e-7f * (1.0f + ext);
  }
  prof_begin(S, PC_SWEEP, st);
  // the sweep kernel: contact lists when they are allocated (the default),
  // else one thread per particle over all 27 cells with its candidates
  // listed in order; gg_tuning.sweep_variant = 1 picks the pruned
  // one-thread-per-particle stencil sweep instead (same results)
  if (S->tune.sweep_variant == 1) {
    auto kern = (mm == 0 ? k_sweep<0> : mm == 1 ? k_sweep<1> : mm == 2 ? k_sweep<2> : k_sweep<3>);
    kern<<<blocks_for(S->n, 256), 256, 0, st>>>(a);
  } else if (S->g.nl_idx) {
    auto build = (mm == 0 ? k_sweep_nlist_build<0> : mm == 1 ? k_sweep_nlist_build<1> : mm == 2 ? k_sweep_nlist_build<2> : k_sweep_nlist_build<3>);
    if (it == 0) {
      build<<<blocks_for(S->n, kBuildThreads), kBuildThreads, 0, st>>>(a, 0);
    } else {
      auto keep = (mm == 0 ? k_sweep_nlist_keep<0> : mm == 1 ? k_sweep_nlist_keep<1> : mm == 2 ? k_sweep_nlist_keep<2> : k_sweep_nlist_keep<3>);
      const int tk = S->tune.keep_threads;
      keep<<<blocks_for(S->n, tk), tk, 0, st>>>(a);
      const int nb = std::min(blocks_for(S->n, kBuildThreads), S->num_sms * S->tune.build_blocks_per_sm);
      build<<<nb, kBuildThreads, 0, st>>>(a, 1);
      count_launches(S, 1);
    }
  } else {
    auto kern = (mm == 0 ? k_sweep_list<0> : mm == 1 ? k_sweep_list<1> : mm == 2 ? k_sweep_list<2> : k_sweep_list<3>);
    kern<<<blocks_for(S->n, kWarpThreads), kWarpThreads, 0, st>>>(a);
  }
  count_launches(S, 1);
  prof_end(S, PC_SWEEP, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg

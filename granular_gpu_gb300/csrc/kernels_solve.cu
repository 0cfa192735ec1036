// kernels_solve.cu — one PBD substep: predict, Jacobi sweeps, finalize, and
// the upsampled-point advection.
//
// Replaces Solver::step (Solver.cu:82-109): add_external_force,
// update_particle_positions and apply_mass_scaling (:125-191) become one
// predict kernel; each project() iteration (:416-513) becomes one sweep and
// one apply kernel with no fill kernels; final_update (:193-270) and the
// adaptive_last_step fill (:103-108) become one finalize kernel.
#include "common.cuh"

namespace gg {

// ------------------------------------------------------------ radii

// Contact radius into pos.w and surface-law radius, for every particle.
template <int MM>
__global__ void k_radii(int n, float4* __restrict__ pos, const float* __restrict__ mass,
                        float* __restrict__ rs, int rho_i, float rho_f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float m = mass[i];
  pos[i].w = radius_contact<MM>(m, rho_i);
  rs[i] = radius_surface<MM>(m, rho_f);
}

gg_status radii_all(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  const int c = S->g.cur;
  auto kern = S->P.math_mode ? k_radii<1> : k_radii<0>;
  kern<<<blocks_for(S->n, 256), 256, 0, st>>>((int)S->n, S->g.pos[c], S->g.mass[c], S->g.rs[c],
                                              S->phys.rho_i, S->phys.density);
  count_launches(S, 1);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ------------------------------------------------------------ predict

// v += dt*G (Solver.cu:125-131); x* = x + dt*v (:133-160);
// scaled mass m*exp(-y) (:162-191) kept as its reciprocal (:317).
// Also the pruning bounds: max contact radius and max |x* - x|.
template <int MM>
__global__ void k_predict(int n, const float4* __restrict__ pos, const float4* __restrict__ vel,
                          const float* __restrict__ mass, float4* __restrict__ xs,
                          float* __restrict__ inv_m, float dt, float3 dv, DevScalars* scal) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int rbits = 0, dbits = 0;
  if (i < n) {
    const float4 p = pos[i];
    const float4 v4 = vel[i];
    const float3 v = add3(f3(v4), dv);
    const float4 x = make_float4(p.x + dt * v.x, p.y + dt * v.y, p.z + dt * v.z, p.w);
    xs[i] = x;
    const float sm = mass[i] * m_exp<MM>(-p.y);
    inv_m[i] = 1.0f / sm;
    rbits = __float_as_uint(fabsf(p.w));
    dbits = __float_as_uint(fmaxf(fmaxf(fabsf(x.x - p.x), fabsf(x.y - p.y)), fabsf(x.z - p.z)));
  }
  warp_max_bits(&scal->rmax_bits, rbits);
  warp_max_bits(&scal->disp0_bits, dbits);
}

gg_status predict(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  const int c = S->g.cur;
  const float dt = S->phys.dt;
  const float3 dv = make_float3(dt * S->phys.g.x, dt * S->phys.g.y, dt * S->phys.g.z);
  prof_begin(S, PC_PREDICT, st);
  auto kern = S->P.math_mode ? k_predict<1> : k_predict<0>;
  kern<<<blocks_for(S->n, 256), 256, 0, st>>>((int)S->n, S->g.pos[c], S->g.vel[c], S->g.mass[c], S->g.xs,
                                                   S->g.inv_m, dt, dv, S->scal);
  count_launches(S, 1);
  prof_end(S, PC_PREDICT, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ------------------------------------------------------------ Jacobi sweep

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
  const DevScalars* __restrict__ scal;
  double brad;   // boundary radius (double literal 0.01)
  double fcap;   // friction cap (double literal 0.8)
  float minr;    // floor of the particle radius against walls (0.01f)
};

// Which of the three cell columns [c-1, c, c+1] along one axis can hold a
// contact partner: bit k set for offset k-1.  Cells are [cL, (c+1)L) in
// binning coordinates; a partner binned there is within R of x.
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

// compute_delta_pos (Solver.cu:361-401) with boundary_constraint
// (:272-307) and particles_constraint (:309-359), race-free.
//
// The reference's scatters into delta_pos[j] are overwritten by each
// thread's final `delta_pos[i] = dp` when the grid is resident, while its
// constraint-count increments all land.  This kernel produces exactly that
// outcome with gathers only:
//   delta_i = thread i's own corrections, accumulated in the reference's
//             loop order (27 cells; walls, then particles, by index);
//   n_i     = contacts i finds + particles that find i.
// "j finds i" is decided here by i: i's binning cell lies in the stencil of
// trunc(x*_j / L) (the contact test is symmetric).  When it does not, i
// hands the count to j through s_extra (rare: only where predicted and
// binned cells disagree).
//
// Cells that cannot hold a partner (farther than r_i + r_max plus the
// largest displacement since binning) are skipped; they contribute nothing,
// so the sum and its order are unchanged.
template <int MM>
__global__ void __launch_bounds__(256) k_sweep(SweepArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const Grid g = a.g;
  const float4 xi4 = a.xs[i];
  const float3 xi = f3(xi4);
  const float rc_i = xi4.w;
  const float rb_i = fmaxf(rc_i, a.minr);
  const double Bd = a.brad + (double)rb_i;
  const float Bf = (float)Bd;
  const float inv_mi = a.inv_m[i];
  const int3 q = trunc_cell(g, xi);

  const uint32_t key_i = a.keys[i];
  const bool binned = (int)key_i < g.C;
  int cix = 0, ciy = 0, ciz = 0;
  if (binned) {
    const int nyz = g.ny * g.nz;
    cix = (int)key_i / nyz;
    const int r = (int)key_i - cix * nyz;
    ciy = r / g.nz;
    ciz = r - ciy * g.nz;
  }

  float disp = __uint_as_float(a.scal->disp0_bits);
  for (int k = 0; k < a.it; ++k) disp += __uint_as_float(a.scal->inc_bits[k]);
  const float rmax = __uint_as_float(a.scal->rmax_bits);
  const float ax = fmaxf(fmaxf(fabsf(xi.x), fabsf(xi.y)), fabsf(xi.z));
  const float slack = 4e-6f * (ax + 1.0f) + 1e-5f * g.L;
  const float Rp = (rc_i + rmax + disp) * 1.0001f + slack;
  const float Rb = Bf * 1.0001f + slack;
  const unsigned pmx = axis_mask(xi.x, q.x, g.L, Rp), pmy = axis_mask(xi.y, q.y, g.L, Rp),
                 pmz = axis_mask(xi.z, q.z, g.L, Rp);
  const unsigned bmx = axis_mask(xi.x, q.x, g.L, Rb), bmy = axis_mask(xi.y, q.y, g.L, Rb),
                 bmz = axis_mask(xi.z, q.z, g.L, Rb);
  const float Bcut = Bf * Bf * 1.0001f;

  float3 dp = make_float3(0.f, 0.f, 0.f);
  int c = 0, s_loc = 0;
  for (int ox = 0; ox < 3; ++ox) {
    if (!(((pmx | bmx) >> ox) & 1u)) continue;
    for (int oy = 0; oy < 3; ++oy) {
      if (!(((pmy | bmy) >> oy) & 1u)) continue;
      for (int oz = 0; oz < 3; ++oz) {
        const bool usep = ((pmx >> ox) & (pmy >> oy) & (pmz >> oz) & 1u) != 0;
        const bool useb = ((bmx >> ox) & (bmy >> oy) & (bmz >> oz) & 1u) != 0;
        if (!usep && !useb) continue;
        const int cell = cell_key(g, q.x + ox - 1, q.y + oy - 1, q.z + oz - 1);
        if (cell == g.C) continue;
        if (useb) {
          const int b1 = a.bcs[cell + 1];
          for (int b = a.bcs[cell]; b < b1; ++b) {
            const float4 pb = a.bpos[b];
            const float bx = xi.x - pb.x, by = xi.y - pb.y, bz = xi.z - pb.z;
            const float d2 = __fmaf_rn(bx, bx, __fmaf_rn(by, by, __fmul_rn(bz, bz)));
            if (d2 > Bcut) continue;
            const float dis = m_norm3<MM>(bx, by, bz);
            if (!((double)dis < Bd)) continue;  // mag < 0
            const float mag = (float)((double)dis - Bd);
            const float3 p12 = make_float3(bx, by, bz);
            const float3 dpi = smul3(mag / dis, p12);
            const float3 perp = sub3(dpi, div3s(smul3(dot3(dpi, p12), p12), dis * dis));
            const float pn = m_norm3<MM>(perp.x, perp.y, perp.z);
            if ((double)pn < ((double)rb_i + a.brad) * a.fcap) {
              dp = sub3(dp, dpi);
            } else {
              const float minf = (float)fmin((a.brad + (double)rb_i) * a.fcap / (double)pn, 1.0);
              dp = sub3(dp, mul3s(dpi, minf));
            }
            ++c;
          }
        }
        if (usep) {
          const int j1 = a.cs[cell + 1];
          for (int j = a.cs[cell]; j < j1; ++j) {
            if (j == i) continue;
            const float4 xj4 = a.xs[j];
            const float dx = xi.x - xj4.x, dy = xi.y - xj4.y, dz = xi.z - xj4.z;
            const float rr = rc_i + xj4.w;
            const float d2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
            if (d2 > rr * rr * 1.0001f) continue;
            const float dis = m_norm3<MM>(dx, dy, dz);
            const float mag = rr - dis;
            if (!(mag >= 0.0f)) continue;
            const float inv_mj = a.inv_m[j];
            // (float)(1.0 / (double)s) equals the IEEE float reciprocal of s
            // (no double-rounding case exists for 24-bit significands).
            const float inv_sum = __frcp_rn(inv_mi + inv_mj);
            const float t = mag / dis;
            const float3 p12 = make_float3(dx, dy, dz);
            const float3 dpi = smul3((-inv_sum * inv_mi) * t, p12);
            const float3 dpj = smul3((inv_sum * inv_mj) * t, p12);
            const float3 dpij = sub3(dpi, dpj);
            const float3 perp = sub3(dpij, div3s(smul3(dot3(dpij, p12), p12), dis * dis));
            const float pn = m_norm3<MM>(perp.x, perp.y, perp.z);
            const float w = inv_sum * inv_mi;
            // (double)pn < (double)rr * 0.8, decided in float when clear-cut
            const float capf = rr * (float)a.fcap;
            bool within;
            if (pn < capf * 0.999999f) within = true;
            else if (pn > capf * 1.000001f) within = false;
            else within = (double)pn < (double)rr * a.fcap;
            if (within) {
              dp = sub3(dp, smul3(w, dpij));
            } else {
              const float minf = (float)fmin((double)rr * a.fcap / (double)pn, 1.0);
              dp = sub3(dp, mul3s(smul3(w, dpij), minf));
            }
            ++c;
            const int3 qj = trunc_cell(g, make_float3(xj4.x, xj4.y, xj4.z));
            const bool j_finds_i = binned && abs(cix - qj.x) <= 1 && abs(ciy - qj.y) <= 1 &&
                                   abs(ciz - qj.z) <= 1;
            if (j_finds_i) ++s_loc;
            else atomicAdd(&a.s_extra[j], 1);
          }
        }
      }
    }
  }
  a.delta[i] = make_float4(dp.x, dp.y, dp.z, __int_as_float((c & 0xffff) | (s_loc << 16)));
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
  a.minr = S->P.boundary_min_radius;
  prof_begin(S, PC_SWEEP, st);
  auto kern = S->P.math_mode ? k_sweep<1> : k_sweep<0>;
  kern<<<blocks_for(S->n, 256), 256, 0, st>>>(a);
  count_launches(S, 1);
  prof_end(S, PC_SWEEP, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// change_position_functor (Solver.cu:403-414): x* += delta / max(1, n); in
// the stabilisation sweeps x as well (:457-460).
__global__ void k_apply(int n, float4* __restrict__ xs, float4* __restrict__ pos,
                        const float4* __restrict__ delta, int32_t* __restrict__ s_extra,
                        int32_t* __restrict__ ncon, int32_t* __restrict__ contacts, int stab, int last,
                        unsigned int* __restrict__ inc_bits) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int bits = 0;
  if (i < n) {
    const float4 d = delta[i];
    const int packed = __float_as_int(d.w);
    const int c = packed & 0xffff;
    const int sl = (int)((unsigned)packed >> 16);
    const int se = s_extra[i];
    s_extra[i] = 0;
    const int nn = c + sl + se;
    const float3 inc = div3s(make_float3(d.x, d.y, d.z), (float)(nn > 1 ? nn : 1));
    float4 x = xs[i];
    x.x = x.x + inc.x;
    x.y = x.y + inc.y;
    x.z = x.z + inc.z;
    xs[i] = x;
    if (stab) {
      float4 p = pos[i];
      p.x = p.x + inc.x;
      p.y = p.y + inc.y;
      p.z = p.z + inc.z;
      pos[i] = p;
    }
    if (last) {
      ncon[i] = nn;
      contacts[i] = c;
    }
    bits = __float_as_uint(fmaxf(fmaxf(fabsf(inc.x), fabsf(inc.y)), fabsf(inc.z)));
  }
  warp_max_bits(inc_bits, bits);
}

gg_status apply(gg_system* S, int it, bool stab, bool last, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  prof_begin(S, PC_APPLY, st);
  k_apply<<<blocks_for(S->n, 256), 256, 0, st>>>((int)S->n, S->g.xs, S->g.pos[S->g.cur], S->g.delta,
                                                 S->g.s_extra, S->g.ncon, S->g.contacts, stab ? 1 : 0,
                                                 last ? 1 : 0, &S->scal->inc_bits[it]);
  count_launches(S, 1);
  prof_end(S, PC_APPLY, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ------------------------------------------------------------ finalize

struct FinalArgs {
  float dt_inv, rest, dmin_speed, span, dmin, dmax, rate, adamp;
};

// final_velocity_functor (Solver.cu:193-248), final_update (:249-270) and
// the adaptive_last_step reset (:103-108).
template <int MM>
__global__ void k_finalize(int n, float4* __restrict__ pos, const float4* __restrict__ xs,
                           float4* __restrict__ vel, int32_t* __restrict__ als, FinalArgs f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos[i];
  const float4 x = xs[i];
  float3 v = make_float3(f.dt_inv * (x.x - p.x), f.dt_inv * (x.y - p.y), f.dt_inv * (x.z - p.z));
  const float speed = len3(v);
  if (speed < f.rest) {
    v = make_float3(0.f, 0.f, 0.f);
  } else if (speed > f.dmin_speed) {
    float t = (speed - f.dmin_speed) / f.span;
    t = fmaxf(0.0f, fminf(t, 1.0f));
    const float damping = f.dmin + (f.dmax - f.dmin) * t;
    const float fac = damping + (1.0f - damping) * m_exp<MM>(-speed * f.rate);
    v = mul3s(v, fac);
    if (als[i] == 1) v = mul3s(v, f.adamp);
  }
  vel[i] = make_float4(v.x, v.y, v.z, 0.f);
  pos[i] = x;
  als[i] = 0;
}

gg_status finalize(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  FinalArgs f;
  f.dt_inv = 1.0f / S->phys.dt;
  f.rest = S->P.rest_speed;
  f.dmin_speed = S->P.damp_min_speed;
  f.span = S->P.damp_max_speed - S->P.damp_min_speed;
  f.dmin = S->P.damp_min;
  f.dmax = S->P.damp_max;
  f.rate = S->P.damp_exp_rate;
  f.adamp = S->P.adaptive_damp;
  const int c = S->g.cur;
  prof_begin(S, PC_FINALIZE, st);
  auto kern = S->P.math_mode ? k_finalize<1> : k_finalize<0>;
  kern<<<blocks_for(S->n, 256), 256, 0, st>>>((int)S->n, S->g.pos[c], S->g.xs, S->g.vel[c], S->g.als[c], f);
  count_launches(S, 1);
  prof_end(S, PC_FINALIZE, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ------------------------------------------------------------ upsampling

struct UpArgs {
  Grid g;
  int n;
  float4* __restrict__ upos;
  float4* __restrict__ uvel;
  const float4* __restrict__ gpos;
  const float4* __restrict__ gvel;
  const float4* __restrict__ bpos;
  const int32_t* __restrict__ cs;
  const int32_t* __restrict__ bcs;
  float r9, cut2, gdt_y, dtu, brad, brad_cut2, repulsion, vmax, floor_y, floor_fric, bdamp, band, gdamp;
};

// update_upsampled_cuda, Solver.cu:1244-1369.  Candidates beyond the kernel
// support (w = 0 exactly) are skipped; adding +0 would not change a sum.
__global__ void __launch_bounds__(256) k_upsample(UpArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const Grid g = a.g;
  const float4 p4 = a.upos[i];
  const float3 p = f3(p4);
  float3 wv = make_float3(0.f, 0.f, 0.f), rep = make_float3(0.f, 0.f, 0.f);
  float gw = 0.f, maxw = 0.f;
  bool near_b = false;
  const int3 q = floor_cell(g, p);
  for (int m = 0; m < 27; ++m) {
    const int cell = cell_key(g, q.x + m / 9 - 1, q.y + (m % 9) / 3 - 1, q.z + m % 3 - 1);
    if (cell == g.C) continue;
    const int j1 = a.cs[cell + 1];
    for (int j = a.cs[cell]; j < j1; ++j) {
      const float4 xj = a.gpos[j];
      const float3 d = make_float3(p.x - xj.x, p.y - xj.y, p.z - xj.z);
      const float dd = dot3(d, d);
      if (dd > a.cut2) continue;
      const float dis = sqrtf(dd);
      const float t1 = 1.0f - (dis * dis * a.r9);
      const float w = fmaxf(0.0f, t1 * t1 * t1);
      gw += w;
      const float4 vj = a.gvel[j];
      wv = add3(wv, smul3(w, make_float3(vj.x, vj.y, vj.z)));
      maxw = fmaxf(maxw, w);
    }
    const int k1 = a.bcs[cell + 1];
    for (int k = a.bcs[cell]; k < k1; ++k) {
      const float4 b = a.bpos[k];
      const float3 tb = make_float3(p.x - b.x, p.y - b.y, p.z - b.z);
      const float dd = dot3(tb, tb);
      if (dd > a.brad_cut2) continue;
      const float dis = sqrtf(dd);
      if (dis < a.brad) {
        near_b = true;
        const float3 nrm = div3s(tb, dis + 1e-6f);
        const float force = a.repulsion * (a.brad - dis) / a.brad;
        rep = add3(rep, mul3s(nrm, force));
      }
    }
  }
  const float4 uv4 = a.uvel[i];
  const float3 uv = f3(uv4);
  const float3 gdt = make_float3(0.0f * a.dtu, a.gdt_y, 0.0f * a.dtu);
  float3 nv;
  if (gw > 1e-6f) {
    wv = div3s(wv, gw);
    const float alpha = fmaxf(0.0f, 1.0f - maxw);
    nv = add3(smul3(alpha, add3(uv, gdt)), smul3(1.0f - alpha, wv));
  } else {
    nv = add3(uv, gdt);
    if (near_b) {
      nv = mul3s(nv, a.bdamp);
      if (p.y < a.band) nv.y = nv.y * a.gdamp;
    }
  }
  nv = add3(nv, rep);
  nv.x = fmaxf(-a.vmax, fminf(nv.x, a.vmax));
  nv.y = fmaxf(-a.vmax, fminf(nv.y, a.vmax));
  nv.z = fmaxf(-a.vmax, fminf(nv.z, a.vmax));
  if (isnan(nv.x) || isnan(nv.y) || isnan(nv.z)) nv = make_float3(0.f, 0.f, 0.f);
  float3 up = add3(p, mul3s(nv, a.dtu));
  if (up.y < a.floor_y) {
    up.y = a.floor_y;
    nv.y = 0.0f;
    nv.x = nv.x * a.floor_fric;
    nv.z = nv.z * a.floor_fric;
  }
  if (up.x < 0.0f) {
    up.x = 0.0f;
    nv.x = 0.0f;
  }
  if (up.z < 0.0f) {
    up.z = 0.0f;
    nv.z = 0.0f;
  }
  a.uvel[i] = make_float4(nv.x, nv.y, nv.z, 0.f);
  a.upos[i] = make_float4(up.x, up.y, up.z, p4.w);
}

gg_status upsample(gg_system* S, cudaStream_t st) {
  if (S->nu <= 0) return GG_OK;
  UpArgs a;
  a.g = S->grid;
  a.n = (int)S->nu;
  a.upos = S->u.pos[S->u.cur];
  a.uvel = S->u.vel[S->u.cur];
  a.gpos = S->g.pos[S->g.cur];
  a.gvel = S->g.vel[S->g.cur];
  a.bpos = S->b.pos;
  a.cs = S->g.cell_start;
  a.bcs = S->b.cell_start;
  a.r9 = S->P.up_inv_h2;
  // w > 0 needs dis^2 r9 < 1; the margin keeps every such candidate
  a.cut2 = (1.0f / S->P.up_inv_h2) * 1.001f;
  a.dtu = S->P.up_dt;
  a.gdt_y = S->P.up_gravity_y * S->P.up_dt;
  a.brad = S->P.up_boundary_radius;
  a.brad_cut2 = S->P.up_boundary_radius * S->P.up_boundary_radius * 1.001f;
  a.repulsion = S->P.up_repulsion;
  a.vmax = S->P.up_max_velocity;
  a.floor_y = S->P.up_floor_y;
  a.floor_fric = S->P.up_floor_friction;
  a.bdamp = S->P.up_boundary_damping;
  a.band = S->P.up_ground_band;
  a.gdamp = S->P.up_ground_damping;
  prof_begin(S, PC_UPSAMPLE, st);
  k_upsample<<<blocks_for(S->nu, 256), 256, 0, st>>>(a);
  count_launches(S, 1);
  prof_end(S, PC_UPSAMPLE, S->nu, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ------------------------------------------------------------ explosion

// apply_explosion_force, Solver.cu:1389-1409.
__global__ void k_explosion(int n, const float4* __restrict__ pos, float4* __restrict__ vel,
                            const float* __restrict__ mass, float3 com, float force) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float3 dir = sub3(f3(pos[i]), com);
  const float dist = len3(dir);
  if (dist < 1e-4f) return;
  dir = div3s(dir, dist);
  const float fm = force / (1.0f + dist * dist);
  const float3 dv = div3s(mul3s(dir, fm), mass[i]);
  float4 v = vel[i];
  v.x = v.x + dv.x;
  v.y = v.y + dv.y;
  v.z = v.z + dv.z;
  vel[i] = v;
}

gg_status explosion(gg_system* S, float force, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  gg_stats_t stt;
  gg_status rc = stats_compute(S, &stt);
  if (rc != GG_OK) return rc;
  float3 com = make_float3(0.f, 0.f, 0.f);
  if (stt.total_mass > 0)
    com = make_float3((float)stt.center_of_mass[0], (float)stt.center_of_mass[1], (float)stt.center_of_mass[2]);
  const int c = S->g.cur;
  k_explosion<<<blocks_for(S->n, 256), 256, 0, st>>>((int)S->n, S->g.pos[c], S->g.vel[c], S->g.mass[c], com, force);
  count_launches(S, 1);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg

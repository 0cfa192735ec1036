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
  block_max_bits_any(&scal->rmax_bits, rbits);
  block_max_bits_any(&scal->disp0_bits, dbits);
}

gg_status predict(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  const int c = S->g.cur;
  const float dt = S->phys.dt;
  const float3 dv = make_float3(dt * S->phys.g.x, dt * S->phys.g.y, dt * S->phys.g.z);
  prof_begin(S, PC_PREDICT, st);
  auto kern = S->P.math_mode ? k_predict<1> : k_predict<0>;
  const int tp = S->tune.predict_threads;
  kern<<<blocks_for(S->n, tp), tp, 0, st>>>((int)S->n, S->g.pos[c], S->g.vel[c], S->g.mass[c], S->g.xs,
                                                   S->g.inv_m, dt, dv, S->scal);
  count_launches(S, 1);
  prof_end(S, PC_PREDICT, S->n, st);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// Analytic walls of the configured mode (gg_params.planes) and its Coulomb
// friction.
struct PlaneArgs {
  int n;          // planes in use (0: none)
  int coulomb;    // contact_law 1
  float mus, muk;
  float4 pl[8];   // unit normal, offset: a particle keeps n . x >= d + r
  // batched scenes: walls in scene coordinates (x - s W for scene s, the
  // slab floor(x / W)) and, when given, Coulomb coefficients per scene
  int n_scenes;
  float scene_w, scene_inv_w;
  const float2* __restrict__ scene_mu;
};

// change_position_functor (Solver.cu:403-414): x* += delta / max(1, n); in
// the stabilisation sweeps x as well (:457-460).
//
// Configured mode.  Analytic walls are hard constraints: x* is projected
// onto each wall it is within its radius of (in a stabilisation sweep x
// moves with it).  With the Coulomb law, outside the stabilisation sweeps,
// friction targets cancel the tangential slip since the substep began:
// the particle contacts' targets from the sweep (fdelta) are averaged like
// the normal corrections, each wall in contact (within 1 % of the radius)
// gets its own, applied in full like its projection.  A target is applied
// whole while its length is below mu_static times the normal correction the
// particle received in this substep so far (pn: the averaged contact
// corrections and the wall projections), else cut to mu_kinetic times it.
// In a batch of scenes the walls are in each scene's own coordinates and
// the coefficients those of the particle's scene.
__global__ void __launch_bounds__(256) k_apply(int n, float4* __restrict__ xs, float4* __restrict__ pos,
                        const float4* __restrict__ delta, int32_t* __restrict__ s_extra,
                        int32_t* __restrict__ ncon, int32_t* __restrict__ contacts, int stab, int last,
                        unsigned int* __restrict__ inc_bits, unsigned int* __restrict__ inc_norm_bits,
                        const uint32_t* __restrict__ keys,
                        uint32_t* __restrict__ cell_inc, int C, int nz, UDiv div_z, PlaneArgs pa,
                        const float4* __restrict__ fdelta, float* __restrict__ pn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int bits = 0, nbits = 0;
  uint32_t key = 0xffffffffu;
  if (i < n) {
    // every load first, so that they are in flight together
    const float4 d = __ldcs(&delta[i]);
    const int se = s_extra[i];
    float4 x = xs[i];
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    if (stab || fdelta) p = pos[i];
    if (cell_inc) key = keys[i];
    const int packed = __float_as_int(d.w);
    const int c = packed & 0xffff;
    const int sl = (int)((unsigned)packed >> 16);
    const int nn = c + sl + se;
    float3 inc = div3s(make_float3(d.x, d.y, d.z), (float)(nn > 1 ? nn : 1));
    s_extra[i] = 0;
    const float3 x_old = f3(x);
    x.x = x.x + inc.x;
    x.y = x.y + inc.y;
    x.z = x.z + inc.z;
    if (stab) {
      p.x = p.x + inc.x;
      p.y = p.y + inc.y;
      p.z = p.z + inc.z;
    }
    float pni = 0.0f;
    if (fdelta) pni = pn[i] + len3(inc);
    float mus = pa.mus, muk = pa.muk, xoff = 0.0f;
    if (pa.n_scenes > 0) {
      const int sc = min(max(__float2int_rz(x.x * pa.scene_inv_w), 0), pa.n_scenes - 1);
      xoff = (float)sc * pa.scene_w;
      if (pa.scene_mu) {
        const float2 mu = pa.scene_mu[sc];
        mus = mu.x;
        muk = mu.y;
      }
    }
    // a wall's offset in this particle's scene
    auto wall_d = [&](int k) { return pa.n_scenes > 0 ? pa.pl[k].w + pa.pl[k].x * xoff : pa.pl[k].w; };
    for (int k = 0; k < pa.n; ++k) {
      const float3 nrm = make_float3(pa.pl[k].x, pa.pl[k].y, pa.pl[k].z);
      const float sd = dot3(nrm, f3(x)) - wall_d(k) - x.w;
      if (!(sd < 0.0f)) continue;
      x.x = x.x + -sd * nrm.x;
      x.y = x.y + -sd * nrm.y;
      x.z = x.z + -sd * nrm.z;
      if (stab) {
        p.x = p.x + -sd * nrm.x;
        p.y = p.y + -sd * nrm.y;
        p.z = p.z + -sd * nrm.z;
      }
      pni = pni - sd;
    }
    if (fdelta && !stab) {
      // particle contacts: their friction targets averaged, as the normal
      // corrections are
      const float4 fd = fdelta[i];
      const int fc = __float_as_int(fd.w);
      if (fc > 0) {
        const float3 ft = div3s(make_float3(fd.x, fd.y, fd.z), (float)fc);
        const float lt = len3(ft);
        const float f = lt < mus * pni ? 1.0f : fminf(muk * pni / lt, 1.0f);
        x.x = x.x + f * ft.x;
        x.y = x.y + f * ft.y;
        x.z = x.z + f * ft.z;
      }
      // walls in contact (within 1 % of the radius): the tangential slip
      // since the substep began, cancelled in full like their normal
      // projection
      for (int k = 0; k < pa.n; ++k) {
        const float3 nrm = make_float3(pa.pl[k].x, pa.pl[k].y, pa.pl[k].z);
        const float sd = dot3(nrm, f3(x)) - wall_d(k) - x.w;
        if (!(sd < 0.01f * x.w)) continue;
        const float3 drel = sub3(f3(x), f3(p));
        const float3 tn = sub3(drel, smul3(dot3(drel, nrm), nrm));
        const float lt = len3(tn);
        const float f = lt < mus * pni ? 1.0f : fminf(muk * pni / lt, 1.0f);
        x.x = x.x - f * tn.x;
        x.y = x.y - f * tn.y;
        x.z = x.z - f * tn.z;
      }
    }
    if (fdelta) pn[i] = pni;
    if (pa.n || fdelta) inc = sub3(f3(x), x_old);  // the listed sweeps bound the whole change
    xs[i] = x;
    if (stab) pos[i] = p;
    if (last) {
      ncon[i] = nn;
      contacts[i] = c;
    }
    bits = __float_as_uint(fmaxf(fmaxf(fabsf(inc.x), fabsf(inc.y)), fabsf(inc.z)));
    // the increment's length, rounded up past the roundings of the dot
    // product and the root (a relative 3e-7 at most)
    nbits = __float_as_uint(sqrtf(dot3(inc, inc)) * 1.000001f);
  }
  if (cell_inc) {
    // per-cell bound read by the next listed sweep (non-negative float bits
    // order like the values; NaN bits are above every finite value); the
    // lanes of one cell combine first, since sorted neighbours share cells.
    // Each cell's value also goes to its two z neighbours (the adjacent keys
    // of its column), so an entry holds the largest increment over three
    // cells of a column and a stencil needs nine entries, not 27.
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const unsigned m = __reduce_max_sync(peers, nbits);
    if (key != 0xffffffffu && m && (threadIdx.x & 31) == __ffs(peers) - 1) {
      atomicMax(&cell_inc[key], m);
      if ((int)key < C) {
        const int z = (int)(key - udiv(key, div_z) * (uint32_t)nz);
        if (z > 0) atomicMax(&cell_inc[key - 1], m);
        if (z < nz - 1) atomicMax(&cell_inc[key + 1], m);
      }
    }
  }
  block_max_bits_any(inc_bits, bits);
  block_max_bits_any(inc_norm_bits, nbits);
}

gg_status apply(gg_system* S, int it, bool stab, bool last, bool more, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  prof_begin(S, PC_APPLY, st);
  // a listed sweep after this one (more) reads the per-cell increments
  uint32_t* cell_inc = (S->g.cell_inc && more) ? S->g.cell_inc : nullptr;
  if (cell_inc) GG_CUDA(cudaMemsetAsync(cell_inc, 0, sizeof(uint32_t) * ((size_t)S->grid.C + 1), st));
  PlaneArgs pa;
  pa.n = std::max(0, std::min(S->P.n_planes, 8));
  pa.coulomb = S->P.contact_law == 1;
  pa.mus = S->P.mu_static;
  pa.muk = S->P.mu_kinetic;
  for (int k = 0; k < 8; ++k)
    pa.pl[k] = make_float4(S->P.planes[k][0], S->P.planes[k][1], S->P.planes[k][2], S->P.planes[k][3]);
  pa.n_scenes = S->n_scenes;
  pa.scene_w = S->scene_width;
  pa.scene_inv_w = S->scene_width > 0.0f ? 1.0f / S->scene_width : 0.0f;
  pa.scene_mu = S->scene_mu;
  const int ta = S->tune.apply_threads;
  k_apply<<<blocks_for(S->n, ta), ta, 0, st>>>((int)S->n, S->g.xs, S->g.pos[S->g.cur], S->g.delta,
                                                 S->g.s_extra, S->g.ncon, S->g.contacts, stab ? 1 : 0,
                                                 last ? 1 : 0, &S->scal->inc_bits[it], &S->scal->inc_norm_bits[it],
                                                 S->g.keys, cell_inc,
                                                 S->grid.C, S->grid.nz, make_udiv((uint32_t)S->grid.nz), pa,
                                                 pa.coulomb ? S->g.fdelta : nullptr, S->g.pn);
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
  const int tf = S->tune.finalize_threads;
  kern<<<blocks_for(S->n, tf), tf, 0, st>>>((int)S->n, S->g.pos[c], S->g.xs, S->g.vel[c], S->g.als[c], f);
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
//
// Each stencil column is scanned in chunks of 32 candidates.  A cheap pass
// (fused multiply-adds, compared with the support radius squared plus a
// 0.1 % margin) marks the candidates that can carry weight in a 32-bit mask;
// a second pass evaluates the reference's weight for the marked ones only,
// in candidate order, so the sums are the reference's.  A warp then spends
// the weight arithmetic on each lane's own hits instead of on every
// candidate some lane hits.
// 6 resident blocks of 256 (40 registers, no spills): the kernel is bound by
// instruction issue, and 48 warps per SM hide its load latency better than 40.
//
// ALL: the support reaches every candidate of the stencil (a candidate lies
// within 2 cell lengths of the point along each axis, so within sqrt(12) L,
// and the support covers that), as with the reference's radius 0.045 and
// cells of 0.00808; the candidates are then summed without the mask pass,
// exactly as the reference does.
template <bool ALL>
__global__ void __launch_bounds__(256, 6) k_upsample(UpArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const Grid g = a.g;
  const float4 p4 = a.upos[i];
  const float3 p = f3(p4);
  float3 wv = make_float3(0.f, 0.f, 0.f), rep = make_float3(0.f, 0.f, 0.f);
  float gw = 0.f, maxw = 0.f;
  bool near_b = false;
  const int3 q = floor_cell(g, p);
  // The particle sums and the wall sums are separate, so each runs over a
  // stencil column as one index range (the reference's order within each).
  for_each_stencil_column(g, q, [&](int k0, int nc) {
    const int j1 = a.cs[k0 + nc];
    // the reference's weight (Solver.cu:1281-1287) for candidate j
    auto weigh = [&](int j) {
      const float4 xj = a.gpos[j];
      const float3 d = make_float3(p.x - xj.x, p.y - xj.y, p.z - xj.z);
      const float dis = sqrtf(dot3(d, d));
      const float t1 = 1.0f - (dis * dis * a.r9);
      const float w = fmaxf(0.0f, t1 * t1 * t1);
      gw += w;
      const float4 vj = a.gvel[j];
      wv = add3(wv, smul3(w, make_float3(vj.x, vj.y, vj.z)));
      maxw = fmaxf(maxw, w);
    };
    if (ALL) {
      // unrolled by 4: 8.94 to 8.60 ms per launch at 33.5 M render points
      // (2: the former; 8: 8.57, within the noise of 4)
#pragma unroll 4
      for (int j = a.cs[k0]; j < j1; ++j) weigh(j);
    } else {
      for (int c0 = a.cs[k0]; c0 < j1; c0 += 32) {
        const int cn = min(32, j1 - c0);
        unsigned mask = 0u;
#pragma unroll 8
        for (int b = 0; b < cn; ++b) {
          const float4 xj = a.gpos[c0 + b];
          const float dx = p.x - xj.x, dy = p.y - xj.y, dz = p.z - xj.z;
          const float dd = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
          mask |= (dd <= a.cut2 ? 1u : 0u) << b;
        }
        while (mask) {
          const int j = c0 + __ffs(mask) - 1;
          mask &= mask - 1u;
          weigh(j);
        }
      }
    }
    const int k1 = a.bcs[k0 + nc];
    for (int k = a.bcs[k0]; k < k1; ++k) {
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
  });
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
  // every candidate of a point's stencil lies within sqrt(12) cell lengths
  const float reach2 = 12.0f * S->grid.L * S->grid.L * 1.001f;
  const bool all_in = reach2 * S->P.up_inv_h2 < 0.999f;
  prof_begin(S, PC_UPSAMPLE, st);
  if (all_in) k_upsample<true><<<blocks_for(S->nu, 256), 256, 0, st>>>(a);
  else k_upsample<false><<<blocks_for(S->nu, 256), 256, 0, st>>>(a);
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

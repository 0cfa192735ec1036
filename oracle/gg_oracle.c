/*
 * gg_oracle.c — CPU restatement of granular_gpu's per-substep path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this file.  It is the checker the CUDA path is compared against in
 * tests/, in __graft_entry__.smoke() and (as the timed CPU baseline) in
 * bench.py.
 *
 * Parity status: pinned.  The reference ships no tests, fixtures or golden
 * vectors for this path, so the restatement is checked against the
 * reference's own kernels, compiled from its sources into cubins
 * (oracle/ref_cuda_build.py) and run on the GB300 from the same states
 * (tests/test_ref_cuda.py, tests/test_ref_merge_split.py), and against
 * hand-derived known answers (tests/golden).
 *
 * Two builds of this one file:
 *   GGO_FP64=0  (libggoracle32.so)  FP32 state.  Every expression follows the
 *               reference's own mix of float and double arithmetic (the
 *               double literals and __constant__ double pi of Solver.cu:28,
 *               GranularSystem.cu:28), so it is the bit-level model the CUDA
 *               kernels are held to.
 *   GGO_FP64=1  (libggoracle64.so)  the same algorithm with all state and
 *               arithmetic in double: the serial FP64 transcription each FP32
 *               result is measured against.
 *
 * Where the reference races (compute_delta_pos Solver.cu:346-353,399;
 * merge_mark_gpu Solver.cu:609-628; split_gpu slot order Solver.cu:812) this
 * file implements one fixed, legal schedule of the reference kernel; the
 * schedule is stated at each function.
 *
 * Compile with -ffp-contract=off: no fused multiply-adds, so x86 and Arm
 * hosts give identical results.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/gg.h"

#ifndef GGO_FP64
#define GGO_FP64 0
#endif

#if GGO_FP64
typedef double real;
#define R_CBRT cbrt
#define R_EXP exp
#define R_SQRT sqrt
#define R_ACOS acos
#define R_COS cos
#define R_SIN sin
#define R_FLOOR floor
#define R_FMAX fmax
#define R_FMIN fmin
#define GGO_SYM(name) ggo64_##name
#else
typedef float real;
/* transcendentals evaluated in double and rounded once to float */
#define R_CBRT(x) ((float)cbrt((double)(x)))
#define R_EXP(x) ((float)exp((double)(x)))
#define R_SQRT sqrtf
#define R_ACOS(x) ((float)acos((double)(x)))
#define R_COS(x) ((float)cos((double)(x)))
#define R_SIN(x) ((float)sin((double)(x)))
#define R_FLOOR floorf
#define R_FMAX fmaxf
#define R_FMIN fminf
#define GGO_SYM(name) ggo32_##name
#endif

#define GGO_PI_D 3.14159265358979323846         /* Solver.cu:28, GranularSystem.cu:28 */
#define GGO_PI_F 3.14159265358979323846f        /* Global.hpp:7 */
#define GGO_UNITS_PER_MASS (1 << 20)

typedef struct { real x, y, z; } r3;
typedef struct { int x, y, z; } i3;

static inline r3 v3(real x, real y, real z) { r3 r = {x, y, z}; return r; }
static inline r3 add3(r3 a, r3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline r3 sub3(r3 a, r3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline r3 smul3(real s, r3 a) { return v3(s * a.x, s * a.y, s * a.z); }
static inline r3 mul3s(r3 a, real s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline r3 div3s(r3 a, real s) { return v3(a.x / s, a.y / s, a.z / s); }
/* helper_math dot: a.x*b.x + a.y*b.y + a.z*b.z, left to right. */
static inline real dot3(r3 a, r3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline real len3(r3 a) { return R_SQRT(dot3(a, a)); }
/* helper_math normalize: v * rsqrtf(dot(v,v)), the reciprocal square root
 * evaluated in double and rounded once. */
static inline r3 normalize3(r3 a) { return mul3s(a, (real)(1.0 / sqrt((double)dot3(a, a)))); }
/* norm3df(a,b,c): the Euclidean norm, rounded once from double. */
static inline real norm3(real a, real b, real c) {
#if GGO_FP64
  return sqrt(a * a + b * b + c * c);
#else
  double da = a, db = b, dc = c;
  return (float)sqrt(da * da + db * db + dc * dc);
#endif
}

/* Float-to-int conversion with the GPU's cvt.rzi semantics: truncation,
 * saturation at the int range, NaN -> 0.  make_int3(float3) in
 * helper_math.h is this conversion per component. */
static inline int f2i(real v) {
  if (v != v) return 0;
  if (v >= (real)2147483648.0) return INT_MAX;
  if (v <= (real)-2147483648.0) return INT_MIN;
  return (int)v;
}

typedef struct ggo_sys {
  gg_params P;
  real L;
  int nx, ny, nz, C;
  real dt;
  r3 G;
  float rho_f;
  int rho_i;
  int is_move_boundary, is_adaptive;
  int64_t n, cap, n_grid;
  r3 *pos, *vel, *pos_t, *delta;
  real *mass, *scaled_mass, *inv_m, *rc, *rb, *rs;
  int32_t *units;
  int32_t *als, *surface, *remove, *merge_count, *merge_units;
  real *sdist, *merge;
  r3 *merge_vel, *cover;
  int32_t *keys, *perm, *cell_start, *ncon, *contacts, *rev;
  int32_t *tmp_i; real *tmp_r; r3 *tmp_3;
  /* merge scratch */
  int32_t *prop, *winner; real *ldens;
  /* split scratch */
  int32_t *split_flag; r3 *child_pos; int32_t *child_cell;
  r3 *fdelta; int32_t *fcount; real *pn;
  int64_t nb;
  r3 *bpos;
  int32_t *banim, *bkeys, *bcell_start;
  int64_t nu;
  r3 *upos, *uvel;
  int32_t *ukeys;
  int64_t steps;
  int merge_iter;
  int64_t merged_last, split_last, merged_total, split_total;
  int32_t error_word;
  int64_t stats_len, stats_cap;
  int64_t *stats;  /* triples: merged, split, total (Solver.cu:1235-1236) */
} ggo_sys;

/* ------------------------------------------------------------------ grid */

/* particlePos2cellIdx, CUDAFunctions.cuh:71-79. */
static inline int cell_key(const ggo_sys* s, int x, int y, int z) {
  return (x >= 0 && x < s->nx && y >= 0 && y < s->ny && z >= 0 && z < s->nz)
             ? ((x * s->ny) + y) * s->nz + z
             : s->C;
}

/* mapParticles2Cells_CUDA, CUDAFunctions.cuh:91-107: floorf(pos/L). */
static void map_to_cells(const ggo_sys* s, const r3* p, int64_t n, int32_t* keys) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
    keys[i] = cell_key(s, f2i(R_FLOOR(p[i].x / s->L)), f2i(R_FLOOR(p[i].y / s->L)),
                       f2i(R_FLOOR(p[i].z / s->L)));
}

/* thrust::sort_by_key on int keys is a stable radix sort: a stable
 * counting sort over the C+1 key values gives the same permutation. */
static void stable_sort(int C, const int32_t* keys, int64_t n, int32_t* perm,
                        int32_t* sorted_keys, int32_t* counts /* C+2 */) {
  memset(counts, 0, sizeof(int32_t) * (size_t)(C + 2));
  for (int64_t i = 0; i < n; ++i) counts[keys[i] + 1]++;
  for (int c = 0; c <= C; ++c) counts[c + 1] += counts[c];
  for (int64_t i = 0; i < n; ++i) {
    int32_t k = keys[i];
    int32_t d = counts[k]++;
    perm[d] = (int32_t)i;
    if (sorted_keys) sorted_keys[d] = k;
  }
}

/* countingInCell_CUDA + exclusive_scan over C+1 entries
 * (CUDAFunctions.cuh:54-61, GranularSystem.cu:147-170). */
static void build_cell_start(int C, const int32_t* keys, int64_t n, int32_t* cs) {
  memset(cs, 0, sizeof(int32_t) * (size_t)(C + 1));
  for (int64_t i = 0; i < n; ++i) cs[keys[i]]++;
  int32_t run = 0;
  for (int c = 0; c <= C; ++c) {
    int32_t v = cs[c];
    cs[c] = run;
    run += v;
  }
}

#define PERMUTE(T, arr, tmp)                                          \
  do {                                                                \
    for (int64_t q = 0; q < n; ++q) (tmp)[q] = (arr)[s->perm[q]];     \
    memcpy((arr), (tmp), sizeof(T) * (size_t)n);                      \
  } while (0)

/* neighbor_search_granular, GranularSystem.cu:65-173.  The sort carries pos
 * and the index; vel, mass, merge, merge_count and remove are gathered.
 * adaptive_last_step and merge_velocity are NOT permuted (as in the
 * reference). */
static void granular_grid(ggo_sys* s) {
  int64_t n = s->n;
  int32_t* counts = (int32_t*)malloc(sizeof(int32_t) * (size_t)(s->C + 2));
  s->n_grid = n;
  map_to_cells(s, s->pos, n, s->keys);
  stable_sort(s->C, s->keys, n, s->perm, s->tmp_i, counts);
  memcpy(s->keys, s->tmp_i, sizeof(int32_t) * (size_t)n);
  PERMUTE(r3, s->pos, s->tmp_3);
  PERMUTE(r3, s->vel, s->tmp_3);
  PERMUTE(real, s->mass, s->tmp_r);
  PERMUTE(real, s->merge, s->tmp_r);
  {
    int32_t* t = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
    PERMUTE(int32_t, s->units, t);
    PERMUTE(int32_t, s->merge_units, t);
    PERMUTE(int32_t, s->merge_count, t);
    PERMUTE(int32_t, s->remove, t);
    free(t);
  }
  build_cell_start(s->C, s->keys, n, s->cell_start);
  free(counts);
}

/* neighbor_search_boundary, GranularSystem.cu:174-280: sort (pos, is_animated). */
static void boundary_grid(ggo_sys* s) {
  int64_t n = s->nb;
  if (n == 0) {
    build_cell_start(s->C, s->bkeys, 0, s->bcell_start);
    return;
  }
  int32_t* counts = (int32_t*)malloc(sizeof(int32_t) * (size_t)(s->C + 2));
  int32_t* perm = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  int32_t* sk = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  r3* tp = (r3*)malloc(sizeof(r3) * (size_t)n);
  int32_t* ta = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  map_to_cells(s, s->bpos, n, s->bkeys);
  stable_sort(s->C, s->bkeys, n, perm, sk, counts);
  for (int64_t q = 0; q < n; ++q) { tp[q] = s->bpos[perm[q]]; ta[q] = s->banim[perm[q]]; }
  memcpy(s->bpos, tp, sizeof(r3) * (size_t)n);
  memcpy(s->banim, ta, sizeof(int32_t) * (size_t)n);
  memcpy(s->bkeys, sk, sizeof(int32_t) * (size_t)n);
  build_cell_start(s->C, s->bkeys, n, s->bcell_start);
  free(counts); free(perm); free(sk); free(tp); free(ta);
}

/* neighbor_search_upsampled, GranularSystem.cu:282-395: pos and vel sorted
 * by the same stable permutation.  Its cell table is never read by the
 * reference, so it is not built. */
static void upsampled_grid(ggo_sys* s) {
  int64_t n = s->nu;
  if (n == 0) return;
  int32_t* counts = (int32_t*)malloc(sizeof(int32_t) * (size_t)(s->C + 2));
  int32_t* perm = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  r3* t = (r3*)malloc(sizeof(r3) * (size_t)n);
  map_to_cells(s, s->upos, n, s->ukeys);
  stable_sort(s->C, s->ukeys, n, perm, NULL, counts);
  for (int64_t q = 0; q < n; ++q) t[q] = s->upos[perm[q]];
  memcpy(s->upos, t, sizeof(r3) * (size_t)n);
  for (int64_t q = 0; q < n; ++q) t[q] = s->uvel[perm[q]];
  memcpy(s->uvel, t, sizeof(r3) * (size_t)n);
  free(counts); free(perm); free(t);
}

/* ----------------------------------------------------------- radius laws */

/* cbrtf((3 * m) / (4 * pi * density)) with `int density` and double pi, as
 * compute_delta_pos passes it (Solver.cu:311,320-321,367). */
static inline real radius_contact(const ggo_sys* s, real m) {
  return R_CBRT((real)((double)((real)3 * m) / (4.0 * GGO_PI_D * (double)s->rho_i)));
}
/* The same law with float density (GranularSystem.cu:518,536,570,588). */
static inline real radius_surface(const ggo_sys* s, real m) {
  return R_CBRT((real)((double)((real)3 * m) / (4.0 * GGO_PI_D * (double)s->rho_f)));
}
/* All-float law with the PI macro, split_gpu (Solver.cu:799). */
static inline real radius_split(const ggo_sys* s, real m) {
  return R_CBRT(((real)3 * m) / (((real)4 * (real)GGO_PI_F) * (real)s->rho_f));
}

static void refresh_radii(ggo_sys* s) {
  const real minr = (real)s->P.boundary_min_radius;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < s->n; ++i) {
    real m = s->mass[i];
    s->rc[i] = radius_contact(s, m);
    s->rb[i] = R_FMAX(s->rc[i], minr);
    s->rs[i] = radius_surface(s, m);
  }
}

/* ------------------------------------------------------------- PBD solve */

static inline i3 trunc_cell(const ggo_sys* s, r3 p) {
  /* make_int3(pos / cell_length): float3 / float then truncation. */
  i3 c = {f2i(p.x / s->L), f2i(p.y / s->L), f2i(p.z / s->L)};
  return c;
}
static inline i3 floor_cell(const ggo_sys* s, r3 p) {
  i3 c = {f2i(R_FLOOR(p.x / s->L)), f2i(R_FLOOR(p.y / s->L)), f2i(R_FLOOR(p.z / s->L))};
  return c;
}

/*
 * One sweep of compute_delta_pos (Solver.cu:361-401) with
 * boundary_constraint (:272-307) and particles_constraint (:309-359).
 *
 * Schedule: every thread's scatters into delta_pos[j] land before thread
 * j's final `delta_pos[i] = dp` (Solver.cu:399), so they are overwritten;
 * every constraint-count increment lands.  Hence
 *   delta_i = the corrections thread i computes for itself (loop order),
 *   n_i     = (contacts i finds) + (number of particles that find i).
 * This is the race outcome when the whole grid is resident, which is the
 * reference's own launch shape for its scenes.
 */
static void sweep(ggo_sys* s) {
  const int64_t n = s->n;
  const double brad = s->P.boundary_radius;
  const double fcap = s->P.friction_cap;
  const int coulomb = s->P.contact_law == 1;
  memset(s->rev, 0, sizeof(int32_t) * (size_t)n);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    r3 xi = s->pos_t[i];
    const r3 x0i = s->pos[i];
    r3 dp = v3(0, 0, 0);
    r3 df = v3(0, 0, 0); /* Coulomb law: friction corrections, averaged on their own */
    int c = 0, fc = 0;
    const i3 q = trunc_cell(s, xi);
    const real rb_i = s->rb[i];
    const real rc_i = s->rc[i];
    const real inv_mi = s->inv_m[i];
    for (int m = 0; m < 27; ++m) {
      const int cell = cell_key(s, q.x + m / 9 - 1, q.y + (m % 9) / 3 - 1, q.z + m % 3 - 1);
      if (cell == s->C) continue;
      for (int32_t b = s->bcell_start[cell]; b < s->bcell_start[cell + 1]; ++b) {
        const r3 pb = s->bpos[b];
        const real dis = norm3(xi.x - pb.x, xi.y - pb.y, xi.z - pb.z);
        const real mag = (real)((double)dis - (brad + (double)rb_i));
        const r3 p12 = sub3(xi, pb);
        if (mag < 0 && coulomb) {
          /* configured mode (gg_params.contact_law = 1): the normal push,
           * and the friction target, cancelling the tangential displacement
           * since the substep began (the apply step limits the average) */
          const r3 dpi = smul3(mag / dis, p12);
          const r3 drel = sub3(xi, x0i);
          const real dn = dot3(drel, p12) / (dis * dis);
          const r3 dtan = sub3(drel, smul3(dn, p12));
          dp = sub3(dp, dpi);
          df = sub3(df, dtan);
          ++fc;
          ++c;
        } else if (mag < 0) {
          const r3 dpi = smul3(mag / dis, p12);
          const r3 perp = sub3(dpi, div3s(smul3(dot3(dpi, p12), p12), dis * dis));
          const real pn = norm3(perp.x, perp.y, perp.z);
          const real minf = (real)fmin((brad + (double)rb_i) * fcap / (double)pn, 1.0);
          if ((double)pn < ((double)rb_i + brad) * fcap) dp = sub3(dp, dpi);
          else dp = sub3(dp, mul3s(dpi, minf));
          ++c;
        }
      }
      for (int32_t j = s->cell_start[cell]; j < s->cell_start[cell + 1]; ++j) {
        if (j == i) continue;
        const r3 xj = s->pos_t[j];
        const r3 p12 = sub3(xi, xj);
        const real inv_mj = s->inv_m[j];
        const real inv_sum = (real)(1.0 / (double)(inv_mi + inv_mj));
        const real rc_j = s->rc[j];
        const real dis = norm3(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        const real mag = (rc_i + rc_j) - dis;
        if (mag >= 0 && coulomb) {
          const real t = mag / dis;
          const real w = inv_sum * inv_mi;
          const r3 x0j = s->pos[j];
          const r3 drel = sub3(sub3(xi, x0i), v3(xj.x - x0j.x, xj.y - x0j.y, xj.z - x0j.z));
          const real dn = dot3(drel, p12) / (dis * dis);
          const r3 dtan = sub3(drel, smul3(dn, p12));
          dp = add3(dp, smul3(w * t, p12));
          df = sub3(df, smul3(w, dtan));
          ++fc;
          ++c;
#pragma omp atomic
          s->rev[j]++;
        } else if (mag >= 0) {
          const real t = mag / dis;
          const r3 dpi = smul3((-inv_sum * inv_mi) * t, p12);
          const r3 dpj = smul3((inv_sum * inv_mj) * t, p12);
          const r3 dpij = sub3(dpi, dpj);
          const r3 perp = sub3(dpij, div3s(smul3(dot3(dpij, p12), p12), dis * dis));
          const real pn = norm3(perp.x, perp.y, perp.z);
          const real minf = (real)fmin((double)(rc_i + rc_j) * fcap / (double)pn, 1.0);
          const real w = inv_sum * inv_mi;
          if ((double)pn < (double)(rc_i + rc_j) * fcap) dp = sub3(dp, smul3(w, dpij));
          else dp = sub3(dp, mul3s(smul3(w, dpij), minf));
          ++c;
#pragma omp atomic
          s->rev[j]++;
        }
      }
    }
    s->delta[i] = dp;
    s->fdelta[i] = df;
    s->fcount[i] = fc;
    s->contacts[i] = c;
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) s->ncon[i] = s->contacts[i] + s->rev[i];
}

/* Solver::step, Solver.cu:82-109, with project :416-513 and final_update
 * :193-270. */
static void solver_step(ggo_sys* s) {
  const int64_t n = s->n;
  const gg_params* P = &s->P;
  const r3 dv = v3(s->dt * s->G.x, s->dt * s->G.y, s->dt * s->G.z);
  refresh_radii(s);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    s->vel[i] = add3(s->vel[i], dv);                               /* :125-131 */
    const r3 x = s->pos[i], v = s->vel[i];
    s->pos_t[i] = v3(x.x + s->dt * v.x, x.y + s->dt * v.y, x.z + s->dt * v.z); /* :133-160 */
    s->scaled_mass[i] = s->mass[i] * R_EXP(-x.y);                  /* :162-191 */
    s->inv_m[i] = (real)1 / s->scaled_mass[i];                     /* :317 */
  }
  const int np = P->n_planes < 0 ? 0 : (P->n_planes > 8 ? 8 : P->n_planes);
  const int coulomb = P->contact_law == 1;
  if (coulomb) memset(s->pn, 0, sizeof(real) * (size_t)n);
  const real mus = (real)P->mu_static, muk = (real)P->mu_kinetic;
  const int total = P->stab_iters + P->iters;
  for (int it = 0; it < total; ++it) {
    const int stab = it < P->stab_iters;
    sweep(s);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {                              /* change_position_functor :403-414 */
      const int nn = s->ncon[i] > 1 ? s->ncon[i] : 1;
      if (stab) s->pos[i] = add3(s->pos[i], div3s(s->delta[i], (real)nn));
      s->pos_t[i] = add3(s->pos_t[i], div3s(s->delta[i], (real)nn));
      /* configured mode: analytic walls as hard constraints; the Coulomb
       * law's friction targets (the particle contacts' averaged, each
       * wall's in full), limited by the normal correction the particle
       * received in this substep (k_apply, kernels_solve.cu) */
      real pni = 0;
      if (coulomb) pni = s->pn[i] + len3(div3s(s->delta[i], (real)nn));
      for (int k = 0; k < np; ++k) {
        const r3 nrm = v3((real)P->planes[k][0], (real)P->planes[k][1], (real)P->planes[k][2]);
        const real sd = dot3(nrm, s->pos_t[i]) - (real)P->planes[k][3] - s->rc[i];
        if (!(sd < 0)) continue;
        s->pos_t[i] = v3(s->pos_t[i].x + -sd * nrm.x, s->pos_t[i].y + -sd * nrm.y, s->pos_t[i].z + -sd * nrm.z);
        if (stab) s->pos[i] = v3(s->pos[i].x + -sd * nrm.x, s->pos[i].y + -sd * nrm.y, s->pos[i].z + -sd * nrm.z);
        pni = pni - sd;
      }
      if (coulomb && !stab) {
        /* particle contacts: their friction targets averaged, as the
         * normal corrections are */
        if (s->fcount[i] > 0) {
          const r3 ft = div3s(s->fdelta[i], (real)s->fcount[i]);
          const real lt = len3(ft);
          const real f = lt < mus * pni ? (real)1 : R_FMIN(muk * pni / lt, (real)1);
          s->pos_t[i] = v3(s->pos_t[i].x + f * ft.x, s->pos_t[i].y + f * ft.y, s->pos_t[i].z + f * ft.z);
        }
        /* walls in contact (within 1 % of the radius): the tangential
         * slip since the substep began, cancelled in full like the
         * walls' normal projection */
        for (int k = 0; k < np; ++k) {
          const r3 nrm = v3((real)P->planes[k][0], (real)P->planes[k][1], (real)P->planes[k][2]);
          const real sd = dot3(nrm, s->pos_t[i]) - (real)P->planes[k][3] - s->rc[i];
          if (!(sd < (real)0.01f * s->rc[i])) continue;
          const r3 drel = sub3(s->pos_t[i], s->pos[i]);
          const r3 tn = sub3(drel, smul3(dot3(drel, nrm), nrm));
          const real lt = len3(tn);
          const real f = lt < mus * pni ? (real)1 : R_FMIN(muk * pni / lt, (real)1);
          s->pos_t[i] = v3(s->pos_t[i].x - f * tn.x, s->pos_t[i].y - f * tn.y, s->pos_t[i].z - f * tn.z);
        }
      }
      if (coulomb) s->pn[i] = pni;
    }
  }
  const real dt_inv = (real)1 / s->dt;
  const real span = (real)P->damp_max_speed - (real)P->damp_min_speed;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {                                /* final_velocity_functor :208-247 */
    const r3 x = s->pos[i], xt = s->pos_t[i];
    r3 v = v3(dt_inv * (xt.x - x.x), dt_inv * (xt.y - x.y), dt_inv * (xt.z - x.z));
    const real speed = len3(v);
    if (speed < (real)P->rest_speed) {
      v = v3(0, 0, 0);
    } else if (speed > (real)P->damp_min_speed) {
      real t = (speed - (real)P->damp_min_speed) / span;
      t = R_FMAX((real)0, R_FMIN(t, (real)1));
      const real damping = (real)P->damp_min + ((real)P->damp_max - (real)P->damp_min) * t;
      const real f = damping + ((real)1 - damping) * R_EXP(-speed * (real)P->damp_exp_rate);
      v = mul3s(v, f);
      if (s->als[i] == 1) v = mul3s(v, (real)P->adaptive_damp);
    }
    s->vel[i] = v;
    s->pos[i] = xt;                                                /* :267-269 */
    s->als[i] = 0;                                                 /* :103-108 */
  }
}

/* update_upsampled_cuda, Solver.cu:1244-1369. */
static void upsample(ggo_sys* s) {
  const gg_params* P = &s->P;
  const r3 gdt = mul3s(v3(0, (real)P->up_gravity_y, 0), (real)P->up_dt);
  const real r9 = (real)P->up_inv_h2;
  const real brad = (real)P->up_boundary_radius;
  const real vmax = (real)P->up_max_velocity;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < s->nu; ++i) {
    const r3 p = s->upos[i];
    r3 wv = v3(0, 0, 0), rep = v3(0, 0, 0);
    real gw = 0, maxw = 0;
    int near_b = 0;
    const i3 q = floor_cell(s, p);
    for (int m = 0; m < 27; ++m) {
      const int cell = cell_key(s, q.x + m / 9 - 1, q.y + (m % 9) / 3 - 1, q.z + m % 3 - 1);
      if (cell == s->C) continue;
      for (int32_t j = s->cell_start[cell]; j < s->cell_start[cell + 1]; ++j) {
        const real dis = len3(sub3(p, s->pos[j]));
        const real t1 = (real)1 - (dis * dis * r9);
        const real w = R_FMAX((real)0, t1 * t1 * t1);
        gw += w;
        wv = add3(wv, smul3(w, s->vel[j]));
        maxw = R_FMAX(maxw, w);
      }
      for (int32_t k = s->bcell_start[cell]; k < s->bcell_start[cell + 1]; ++k) {
        const r3 tb = sub3(p, s->bpos[k]);
        const real dis = len3(tb);
        if (dis < brad) {
          near_b = 1;
          const r3 nrm = div3s(tb, dis + (real)1e-6f);
          const real force = (real)P->up_repulsion * (brad - dis) / brad;
          rep = add3(rep, mul3s(nrm, force));
        }
      }
    }
    r3 nv;
    if (gw > (real)1e-6f) {
      wv = div3s(wv, gw);
      const real alpha = R_FMAX((real)0, (real)1 - maxw);
      nv = add3(smul3(alpha, add3(s->uvel[i], gdt)), smul3((real)1 - alpha, wv));
    } else {
      nv = add3(s->uvel[i], gdt);
      if (near_b) {
        nv = mul3s(nv, (real)P->up_boundary_damping);
        if (p.y < (real)P->up_ground_band) nv.y = nv.y * (real)P->up_ground_damping;
      }
    }
    nv = add3(nv, rep);
    nv.x = R_FMAX(-vmax, R_FMIN(nv.x, vmax));
    nv.y = R_FMAX(-vmax, R_FMIN(nv.y, vmax));
    nv.z = R_FMAX(-vmax, R_FMIN(nv.z, vmax));
    if (nv.x != nv.x || nv.y != nv.y || nv.z != nv.z) nv = v3(0, 0, 0);
    r3 up = add3(p, mul3s(nv, (real)P->up_dt));
    if (up.y < (real)P->up_floor_y) {
      up.y = (real)P->up_floor_y;
      nv.y = 0;
      nv.x = nv.x * (real)P->up_floor_friction;
      nv.z = nv.z * (real)P->up_floor_friction;
    }
    if (up.x < 0) { up.x = 0; nv.x = 0; }
    if (up.z < 0) { up.z = 0; nv.z = 0; }
    s->uvel[i] = nv;
    s->upos[i] = up;
  }
}

/* ------------------------------------------------- surface and distance */

/* find_cover_vector + find_surface + the copy, GranularSystem.cu:506-637. */
static void surface(ggo_sys* s) {
  const gg_params* P = &s->P;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < s->n; ++i) {
    const r3 xi = s->pos[i];
    const real ri = s->rs[i];
    const i3 q = trunc_cell(s, xi);
    r3 cv = v3(0, 0, 0);
    for (int m = 0; m < 27; ++m) {
      const int cell = cell_key(s, q.x + m / 9 - 1, q.y + (m % 9) / 3 - 1, q.z + m % 3 - 1);
      if (cell == s->C) continue;
      for (int32_t j = s->cell_start[cell]; j < s->cell_start[cell + 1]; ++j) {
        if (j == i) continue;
        const real dis = len3(sub3(xi, s->pos[j]));
        if (dis > (real)2 * (ri + s->rs[j])) continue;
        cv = add3(cv, normalize3(sub3(xi, s->pos[j])));
      }
    }
    s->cover[i] = cv;
  }
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < s->n; ++i) {
    const r3 xi = s->pos[i];
    const real ri = s->rs[i];
    const i3 q = trunc_cell(s, xi);
    const r3 cv = normalize3(s->cover[i]);
    int vote = 0;
    unsigned nn = 0;
    for (int m = 0; m < 27; ++m) {
      const int cell = cell_key(s, q.x + m / 9 - 1, q.y + (m % 9) / 3 - 1, q.z + m % 3 - 1);
      if (cell == s->C) continue;
      for (int32_t j = s->cell_start[cell]; j < s->cell_start[cell + 1]; ++j) {
        if (j == i) continue;
        r3 b = sub3(s->pos[j], xi);
        const real dis = len3(b);
        if (dis > (real)2 * (ri + s->rs[j])) continue;
        b = normalize3(b);
        if (R_ACOS(dot3(b, cv)) <= (real)P->surface_cone) vote = 1;
        ++nn;
      }
    }
    s->surface[i] = (nn <= (unsigned)P->surface_min_neighbors || !vote) ? 1 : 0;
  }
}

/* compute_distance_to_surface, GranularSystem.cu:639-699. */
static void surface_distance(ggo_sys* s) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < s->n; ++i) {
    if (s->surface[i] == 1) { s->sdist[i] = 0; continue; }
    const r3 xi = s->pos[i];
    const i3 q = trunc_cell(s, xi);
    real best = (real)s->P.no_surface_distance;
    for (int m = 0; m < 27; ++m) {
      const int cell = cell_key(s, q.x + m / 9 - 1, q.y + (m % 9) / 3 - 1, q.z + m % 3 - 1);
      if (cell == s->C) continue;
      for (int32_t j = s->cell_start[cell]; j < s->cell_start[cell + 1]; ++j) {
        if (j == i || s->surface[j] == 0) continue;
        const r3 d = sub3(xi, s->pos[j]);
        const real d2 = dot3(d, d);
        if (d2 < best) best = d2;
      }
    }
    s->sdist[i] = best;
  }
}

static void* xcalloc(size_t n, size_t sz);

/* --------------------------------------------------------- merge / split */

static inline int units_of(real m) { return (int)lrint((double)m * GGO_UNITS_PER_MASS); }
static inline real mass_of_units(int32_t u) { return (real)((double)u / GGO_UNITS_PER_MASS); }

/*
 * merge_mark_gpu, Solver.cu:526-653.
 *
 * Schedule ("warp order with a lag"): every thread finishes its neighbour
 * scan before any thread reaches its compare-and-swaps; then warps of 32
 * consecutive threads issue their CASes in index order, the lanes of a warp
 * together: warp w performs its first CAS (on remove[i]) at time w and its
 * second CAS (on remove[closest]) at time w + merge_cas_lag + 1/2, lanes in
 * lane order.  Under this schedule, in ascending index:
 *   - a proposer i (eligible, closest found) whose own CAS comes after a
 *     successful claim on it is released without acting;
 *   - otherwise it wins its own CAS, and its claim on t succeeds if no lower
 *     proposer claimed t first and t's own first CAS (if t proposes) comes
 *     later, i.e. warp(i) + lag < warp(t).
 * All claimers of t are below t, so the ascending loop settles each
 * winner[t] before t itself is reached.
 */
static void merge_mark(ggo_sys* s) {
  const gg_params* P = &s->P;
  const int64_t n = s->n;
  const real maxm = (real)P->max_mass;
  const real sdt = (real)P->surface_dist_threshold;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    s->prop[i] = -1;
    s->ldens[i] = 0;
    const real mi = s->mass[i];
    if (s->surface[i] != 0 || s->remove[i] != 0 || mi < (real)P->min_merge_mass || mi >= maxm ||
        s->sdist[i] < sdt)
      continue;
    const r3 xi = s->pos[i];
    const i3 q = trunc_cell(s, xi);
    real closest = (real)1000.0f;
    int32_t ci = -1;
    real ld = 0;
    int lc = 0;
    for (int m = 0; m < 27; ++m) {
      const int cell = cell_key(s, q.x + m / 9 - 1, q.y + (m % 9) / 3 - 1, q.z + m % 3 - 1);
      if (cell == s->C) continue;
      for (int32_t j = s->cell_start[cell]; j < s->cell_start[cell + 1] && j < n; ++j) {
        const real dis = len3(sub3(xi, s->pos[j]));
        if ((double)dis < P->merge_radius) { ld += s->mass[j]; ++lc; }
        if (j <= i || s->remove[j] != 0 || s->surface[j] != 0 || s->sdist[i] < sdt) continue;
        if (mi + s->mass[j] > maxm) continue;
        if ((double)dis < P->merge_radius && dis < closest) { closest = dis; ci = j; }
      }
    }
    if (lc > 0 && ci != -1) {
      s->prop[i] = ci;
      s->ldens[i] = ld / (real)lc;
    }
  }
  const int64_t lag = P->merge_cas_lag;
  for (int64_t i = 0; i < n; ++i) s->winner[i] = INT_MAX;
  for (int64_t i = 0; i < n; ++i) {
    const int32_t t = s->prop[i];
    if (t < 0) continue;
    if (s->winner[i] != INT_MAX) continue; /* claimed before its own CAS */
    if (!(s->surface[i] == 0 && s->sdist[i] > sdt)) continue;
    if (s->prop[t] >= 0 && (i >> 5) + lag >= ((int64_t)t >> 5)) continue; /* t's own CAS came first */
    if (s->winner[t] == INT_MAX) s->winner[t] = (int32_t)i;
  }
  for (int64_t i = 0; i < n; ++i) {
    const int32_t t = s->prop[i];
    if (t < 0 || s->winner[i] != INT_MAX) continue;
    s->remove[i] = -1; /* first CAS */
    if (!(s->surface[i] == 0 && s->sdist[i] > sdt)) continue; /* stays -1 */
    if (s->winner[t] != (int32_t)i) { s->remove[i] = 0; continue; }
    s->remove[t] = -1; /* second CAS */
    if (!(s->surface[t] == 0 && s->sdist[t] > sdt)) { s->remove[i] = 0; continue; }
    const real mi = s->mass[i], mt = s->mass[t];
    s->merge[t] = mi;
    s->merge[i] = -mi;
    s->merge_units[t] = s->units[i];
    s->merge_units[i] = -s->units[i];
    const real m_t = (real)1 / (mi + mt);
    const r3 vt = smul3(m_t, add3(smul3(mi, s->vel[i]), smul3(mt, s->vel[t])));
    s->merge_vel[i] = v3(-vt.x, -vt.y, -vt.z);
    const real df = R_FMIN((real)1, s->ldens[i] / (real)P->target_density);
    s->merge_vel[t] = mul3s(vt, (real)1 + ((real)1 - df) * (real)0.1f);
  }
}

/* merge_count_gpu, Solver.cu:658-699.  With mass_ledger the transfer of
 * step k (k = 0..blend-1) is floor(M(k+1)/B) - floor(Mk/B) units, so the
 * B transfers sum to M exactly and giver and receiver change by opposite
 * amounts. */
static void merge_count(ggo_sys* s) {
  const gg_params* P = &s->P;
  const int B = P->blend_factor;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < s->n; ++i) {
    if (s->remove[i] != -1) continue;
    const int old = s->merge_count[i]++;
    const r3 dvel = div3s(s->merge_vel[i], (real)B);
    if (P->mass_ledger) {
      const int64_t M = s->merge_units[i] < 0 ? -(int64_t)s->merge_units[i] : s->merge_units[i];
      int64_t amt = (M * (old + 1)) / B - (M * old) / B;
      if (s->merge_units[i] < 0) amt = -amt;
      s->units[i] += (int32_t)amt;
      s->mass[i] = mass_of_units(s->units[i]);
    } else {
      const real delta = s->merge[i] / (real)B;
      s->mass[i] = s->mass[i] + delta;
    }
    s->als[i] = 1;
    s->vel[i] = add3(s->vel[i], dvel);
    if (old + 1 == B) {
      const int giver = P->mass_ledger ? (s->merge_units[i] < 0) : (s->merge[i] < (real)0);
      if (giver) { s->remove[i] = 1; s->als[i] = 0; }
      else s->remove[i] = 0;
      s->merge_count[i] = 0;
      s->merge[i] = 0;
      s->merge_units[i] = 0;
    }
  }
}

/* check_neighborhood, Solver.cu:708-778. */
static int check_neighborhood(const ggo_sys* s, r3 pos, real r_i, r3* center, int* center_cell) {
  int found = 0;
  const real max_dist = (real)2 * r_i;
  const i3 q = trunc_cell(s, pos);
  for (int m = 0; m < 27; ++m) {
    const int cx = q.x + m / 9 - 1, cy = q.y + (m % 9) / 3 - 1, cz = q.z + m % 3 - 1;
    const int cell = cell_key(s, cx, cy, cz);
    if (cell == s->C) continue;
    if (!found && m != 13) {
      if (s->cell_start[cell] == s->cell_start[cell + 1] &&
          s->bcell_start[cell] == s->bcell_start[cell + 1]) {
        *center = v3(((real)cx + (real)0.5f) * s->L, ((real)cy + (real)0.5f) * s->L,
                     ((real)cz + (real)0.5f) * s->L);
        *center_cell = cell;
        found = 1;
      }
    }
    for (int32_t j = s->bcell_start[cell]; j < s->bcell_start[cell + 1]; ++j) {
      const real dis = len3(sub3(pos, s->bpos[j]));
      if (dis < max_dist) return 0;
    }
  }
  return found;
}

/* split_gpu, Solver.cu:780-827.  Slot order: children are appended in
 * ascending parent index (the reference's atomicAdd order is arbitrary). */
static int64_t split_mark(ggo_sys* s) {
  const gg_params* P = &s->P;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < s->n; ++i) {
    s->split_flag[i] = 0;
    if (s->remove[i] != 0 || s->surface[i] != 1 || s->mass[i] <= (real)P->split_min_mass) continue;
    const real r_i = radius_split(s, s->mass[i]);
    r3 c;
    int cc = 0;
    if (!check_neighborhood(s, s->pos[i], r_i, &c, &cc)) continue;
    s->split_flag[i] = 1;
    s->child_pos[i] = c;
    s->child_cell[i] = cc;
  }
  if (P->split_claim) {
    /* configured mode: a child claims its cell; the lowest parent wins */
    unsigned char* taken = (unsigned char*)xcalloc((size_t)s->C + 1, 1);
    for (int64_t i = 0; i < s->n; ++i) {
      if (!s->split_flag[i]) continue;
      if (taken[s->child_cell[i]]) s->split_flag[i] = 0;
      else taken[s->child_cell[i]] = 1;
    }
    free(taken);
  }
  int64_t k = 0;
  for (int64_t i = 0; i < s->n; ++i) k += s->split_flag[i];
  return k;
}

/* Solver::adaptive_sampling, Solver.cu:856-1242, with DArray::compact
 * (DArray.hpp:62-122) and the appends (Solver.cu:1168-1221,
 * GranularParticles.hpp:30-95). */
static void adaptive_sampling(ggo_sys* s) {
  const int64_t n = s->n;
  if (n == 0) return;
  if (s->merge_iter == 1) {
    merge_mark(s);
    s->merge_iter = 0;
  }
  s->merge_iter++;
  merge_count(s);
  const int64_t nsplit = split_mark(s);
  /* children data captured before compaction */
  int64_t nc = 0;
  r3* cpos = (r3*)malloc(sizeof(r3) * (size_t)(nsplit ? nsplit : 1));
  r3* cvel = (r3*)malloc(sizeof(r3) * (size_t)(nsplit ? nsplit : 1));
  real* cmass = (real*)malloc(sizeof(real) * (size_t)(nsplit ? nsplit : 1));
  int32_t* cunits = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nsplit ? nsplit : 1));
  for (int64_t i = 0; i < n; ++i) {
    if (!s->split_flag[i]) continue;
    cpos[nc] = s->child_pos[i];
    cvel[nc] = s->vel[i];
    if (s->P.mass_ledger) {
      const int32_t half = s->units[i] / 2;
      cunits[nc] = half;
      s->units[i] -= half;
      cmass[nc] = mass_of_units(half);
      s->mass[i] = mass_of_units(s->units[i]);
    } else {
      const real h = s->mass[i] / (real)2;
      cmass[nc] = h;
      cunits[nc] = 0;
      s->mass[i] = h;
    }
    s->als[i] = 1;
    ++nc;
  }
  /* stream compaction, flag == 1 removed, order kept */
  int64_t w = 0, removed = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (s->remove[i] == 1) { ++removed; continue; }
    s->pos[w] = s->pos[i];
    s->vel[w] = s->vel[i];
    s->mass[w] = s->mass[i];
    s->units[w] = s->units[i];
    s->als[w] = s->als[i];
    s->merge_count[w] = s->merge_count[i];
    s->merge[w] = s->merge[i];
    s->merge_units[w] = s->merge_units[i];
    s->remove[w] = s->remove[i];
    ++w;
  }
  int64_t appended = 0;
  for (int64_t k = 0; k < nc; ++k) {
    if (w >= s->cap) { s->error_word |= 1; break; }
    s->pos[w] = cpos[k];
    s->vel[w] = cvel[k];
    s->mass[w] = cmass[k];
    s->units[w] = cunits[k];
    s->als[w] = 1;
    s->merge_count[w] = 0;
    s->merge[w] = 0;
    s->merge_units[w] = 0;
    s->remove[w] = 0;
    ++w;
    ++appended;
  }
  s->merged_last = removed;
  s->split_last = appended;
  s->merged_total += removed;
  s->split_total += appended;
  if (s->stats_len == s->stats_cap) {
    s->stats_cap = s->stats_cap ? 2 * s->stats_cap : 256;
    s->stats = (int64_t*)realloc(s->stats, sizeof(int64_t) * 3 * (size_t)s->stats_cap);
  }
  s->stats[3 * s->stats_len + 0] = removed;
  s->stats[3 * s->stats_len + 1] = appended;
  s->stats[3 * s->stats_len + 2] = n;
  s->stats_len++;
  s->n = w;
  free(cpos); free(cvel); free(cmass); free(cunits);
}

/* GranularSystem::step, GranularSystem.cu:397-453. */
static void step_once(ggo_sys* s) {
  if (s->is_move_boundary) boundary_grid(s);
  granular_grid(s);
  upsampled_grid(s);
  solver_step(s);
  if (s->P.upsample_enabled) upsample(s);
  if (s->is_adaptive == 1 && s->P.merge_enabled) {
    refresh_radii(s);
    surface(s);
    surface_distance(s);
    adaptive_sampling(s);
  }
  s->steps++;
}

/* -------------------------------------------------------------- public */

static void* xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

void GGO_SYM(default_params)(gg_params* P) {
  memset(P, 0, sizeof(*P));
  P->stab_iters = 3; P->iters = 5;
  P->boundary_radius = 0.01; P->boundary_min_radius = 0.01f; P->friction_cap = 0.8;
  P->rest_speed = 0.01f; P->damp_min_speed = 1.0f; P->damp_max_speed = 10.0f;
  P->damp_min = 0.99f; P->damp_max = 0.99f; P->damp_exp_rate = 0.1f; P->adaptive_damp = 0.98f;
  P->max_mass = 4.0f; P->min_merge_mass = 1.0f; P->merge_radius = 0.035;
  P->surface_dist_threshold = 100.0f; P->target_density = 100.0f; P->blend_factor = 40;
  P->split_min_mass = 2.0f; P->surface_cone = 1.047197551f; P->surface_min_neighbors = 5;
  P->no_surface_distance = 100000.0f;
  P->up_inv_h2 = 493.8271605f; P->up_dt = 0.002f; P->up_gravity_y = -9.8f;
  P->up_boundary_radius = 0.015f; P->up_repulsion = 3.0f; P->up_max_velocity = 7.0f;
  P->up_floor_y = 0.04f; P->up_floor_friction = 0.95f; P->up_boundary_damping = 0.8f;
  P->up_ground_band = 0.1f; P->up_ground_damping = 0.5f;
  P->mass_ledger = 0; P->merge_enabled = 1; P->upsample_enabled = 1;
  P->merge_cas_lag = 4;
  P->contact_law = 0; P->mu_static = 0.5f; P->mu_kinetic = 0.4f; P->split_claim = 0; P->n_planes = 0;
}

ggo_sys* GGO_SYM(create)(const gg_desc* d) {
  ggo_sys* s = (ggo_sys*)calloc(1, sizeof(ggo_sys));
  s->P = d->params;
  s->L = (real)d->cell_length;
  s->nx = d->cell_size[0]; s->ny = d->cell_size[1]; s->nz = d->cell_size[2];
  s->C = s->nx * s->ny * s->nz;
  s->dt = (real)d->dt;
  s->G = v3((real)d->gravity[0], (real)d->gravity[1], (real)d->gravity[2]);
  s->rho_f = d->density;
  s->rho_i = (int)d->density;
  s->is_move_boundary = d->is_move_boundary;
  s->is_adaptive = d->is_adaptive;
  s->n = d->n_particles;
  s->cap = d->max_particles > 0 ? d->max_particles : 2 * d->n_particles;
  if (s->cap < s->n) s->cap = s->n;
  const size_t cap = (size_t)s->cap;
  s->pos = (r3*)xcalloc(cap, sizeof(r3)); s->vel = (r3*)xcalloc(cap, sizeof(r3));
  s->pos_t = (r3*)xcalloc(cap, sizeof(r3)); s->delta = (r3*)xcalloc(cap, sizeof(r3));
  s->mass = (real*)xcalloc(cap, sizeof(real)); s->scaled_mass = (real*)xcalloc(cap, sizeof(real));
  s->inv_m = (real*)xcalloc(cap, sizeof(real)); s->rc = (real*)xcalloc(cap, sizeof(real));
  s->rb = (real*)xcalloc(cap, sizeof(real)); s->rs = (real*)xcalloc(cap, sizeof(real));
  s->units = (int32_t*)xcalloc(cap, sizeof(int32_t));
  s->als = (int32_t*)xcalloc(cap, sizeof(int32_t)); s->surface = (int32_t*)xcalloc(cap, sizeof(int32_t));
  s->remove = (int32_t*)xcalloc(cap, sizeof(int32_t)); s->merge_count = (int32_t*)xcalloc(cap, sizeof(int32_t));
  s->merge_units = (int32_t*)xcalloc(cap, sizeof(int32_t));
  s->sdist = (real*)xcalloc(cap, sizeof(real)); s->merge = (real*)xcalloc(cap, sizeof(real));
  s->merge_vel = (r3*)xcalloc(cap, sizeof(r3)); s->cover = (r3*)xcalloc(cap, sizeof(r3));
  s->keys = (int32_t*)xcalloc(cap, sizeof(int32_t)); s->perm = (int32_t*)xcalloc(cap, sizeof(int32_t));
  s->cell_start = (int32_t*)xcalloc((size_t)s->C + 1, sizeof(int32_t));
  s->ncon = (int32_t*)xcalloc(cap, sizeof(int32_t)); s->contacts = (int32_t*)xcalloc(cap, sizeof(int32_t));
  s->rev = (int32_t*)xcalloc(cap, sizeof(int32_t));
  s->tmp_i = (int32_t*)xcalloc(cap, sizeof(int32_t)); s->tmp_r = (real*)xcalloc(cap, sizeof(real));
  s->tmp_3 = (r3*)xcalloc(cap, sizeof(r3));
  s->prop = (int32_t*)xcalloc(cap, sizeof(int32_t)); s->winner = (int32_t*)xcalloc(cap, sizeof(int32_t));
  s->ldens = (real*)xcalloc(cap, sizeof(real));
  s->split_flag = (int32_t*)xcalloc(cap, sizeof(int32_t)); s->child_pos = (r3*)xcalloc(cap, sizeof(r3));
  s->child_cell = (int32_t*)xcalloc(cap, sizeof(int32_t));
  s->fdelta = (r3*)xcalloc(cap, sizeof(r3)); s->fcount = (int32_t*)xcalloc(cap, sizeof(int32_t));
  s->pn = (real*)xcalloc(cap, sizeof(real));
  for (int64_t i = 0; i < s->n; ++i) {
    s->pos[i] = v3((real)d->particles[3 * i], (real)d->particles[3 * i + 1], (real)d->particles[3 * i + 2]);
    const real m = d->masses ? (real)d->masses[i] : (real)1;
    s->mass[i] = m;
    s->units[i] = units_of(m);
    if (s->P.mass_ledger) s->mass[i] = mass_of_units(s->units[i]);
  }
  s->nb = d->n_boundary;
  s->bpos = (r3*)xcalloc((size_t)s->nb, sizeof(r3));
  s->banim = (int32_t*)xcalloc((size_t)s->nb, sizeof(int32_t));
  s->bkeys = (int32_t*)xcalloc((size_t)s->nb, sizeof(int32_t));
  s->bcell_start = (int32_t*)xcalloc((size_t)s->C + 1, sizeof(int32_t));
  for (int64_t i = 0; i < s->nb; ++i) {
    s->bpos[i] = v3((real)d->boundary[3 * i], (real)d->boundary[3 * i + 1], (real)d->boundary[3 * i + 2]);
    s->banim[i] = d->boundary_animated ? d->boundary_animated[i] : 0;
  }
  s->nu = d->n_upsampled;
  s->upos = (r3*)xcalloc((size_t)s->nu, sizeof(r3));
  s->uvel = (r3*)xcalloc((size_t)s->nu, sizeof(r3));
  s->ukeys = (int32_t*)xcalloc((size_t)s->nu, sizeof(int32_t));
  for (int64_t i = 0; i < s->nu; ++i)
    s->upos[i] = v3((real)d->upsampled[3 * i], (real)d->upsampled[3 * i + 1], (real)d->upsampled[3 * i + 2]);
  /* constructor sequence, GranularSystem.cu:54-62 */
  boundary_grid(s);
  granular_grid(s);
  upsampled_grid(s);
  if (!d->skip_initial_step) step_once(s);
  return s;
}

void GGO_SYM(step)(ggo_sys* s, int nsub) {
  for (int k = 0; k < nsub; ++k) step_once(s);
}

int64_t GGO_SYM(size)(const ggo_sys* s, int set) {
  return set == GG_SET_GRANULAR ? s->n : set == GG_SET_BOUNDARY ? s->nb : s->nu;
}

int64_t GGO_SYM(steps)(const ggo_sys* s) { return s->steps; }
int64_t GGO_SYM(n_grid)(const ggo_sys* s) { return s->n_grid; }
int64_t GGO_SYM(merged_last)(const ggo_sys* s) { return s->merged_last; }
int64_t GGO_SYM(split_last)(const ggo_sys* s) { return s->split_last; }

static void out3(const r3* src, int64_t n, float* dst) {
  for (int64_t i = 0; i < n; ++i) {
    dst[3 * i] = (float)src[i].x; dst[3 * i + 1] = (float)src[i].y; dst[3 * i + 2] = (float)src[i].z;
  }
}
static void out1(const real* src, int64_t n, float* dst) {
  for (int64_t i = 0; i < n; ++i) dst[i] = (float)src[i];
}

/* Copies a field into dst (float or int32 per gg.h); returns the element
 * count, or -1 when the field does not exist for the set. */
int64_t GGO_SYM(read)(const ggo_sys* s, int set, int field, void* dst) {
  const int64_t n = GGO_SYM(size)(s, set);
  float* f = (float*)dst;
  int32_t* iv = (int32_t*)dst;
  if (set == GG_SET_GRANULAR) {
    switch (field) {
      case GG_FIELD_POS: out3(s->pos, n, f); return n;
      case GG_FIELD_VEL: out3(s->vel, n, f); return n;
      case GG_FIELD_MASS: out1(s->mass, n, f); return n;
      case GG_FIELD_MASS_UNITS: memcpy(iv, s->units, sizeof(int32_t) * (size_t)n); return n;
      case GG_FIELD_SURFACE: memcpy(iv, s->surface, sizeof(int32_t) * (size_t)n); return n;
      case GG_FIELD_SURFACE_DISTANCE: out1(s->sdist, n, f); return n;
      case GG_FIELD_CELL_KEY: memcpy(iv, s->keys, sizeof(int32_t) * (size_t)s->n_grid); return s->n_grid;
      case GG_FIELD_PERM: memcpy(iv, s->perm, sizeof(int32_t) * (size_t)s->n_grid); return s->n_grid;
      case GG_FIELD_CELL_START: memcpy(iv, s->cell_start, sizeof(int32_t) * (size_t)(s->C + 1)); return s->C + 1;
      case GG_FIELD_REMOVE: memcpy(iv, s->remove, sizeof(int32_t) * (size_t)n); return n;
      case GG_FIELD_MERGE: out1(s->merge, n, f); return n;
      case GG_FIELD_MERGE_COUNT: memcpy(iv, s->merge_count, sizeof(int32_t) * (size_t)n); return n;
      case GG_FIELD_MERGE_VELOCITY: out3(s->merge_vel, n, f); return n;
      case GG_FIELD_ADAPTIVE_LAST_STEP: memcpy(iv, s->als, sizeof(int32_t) * (size_t)n); return n;
      case GG_FIELD_CONTACTS: memcpy(iv, s->contacts, sizeof(int32_t) * (size_t)n); return n;
      case GG_FIELD_NUM_CONSTRAINTS: memcpy(iv, s->ncon, sizeof(int32_t) * (size_t)n); return n;
      default: return -1;
    }
  } else if (set == GG_SET_BOUNDARY) {
    switch (field) {
      case GG_FIELD_POS: out3(s->bpos, n, f); return n;
      case GG_FIELD_IS_ANIMATED: memcpy(iv, s->banim, sizeof(int32_t) * (size_t)n); return n;
      case GG_FIELD_CELL_KEY: memcpy(iv, s->bkeys, sizeof(int32_t) * (size_t)n); return n;
      case GG_FIELD_CELL_START: memcpy(iv, s->bcell_start, sizeof(int32_t) * (size_t)(s->C + 1)); return s->C + 1;
      default: return -1;
    }
  } else {
    switch (field) {
      case GG_FIELD_POS: out3(s->upos, n, f); return n;
      case GG_FIELD_VEL: out3(s->uvel, n, f); return n;
      default: return -1;
    }
  }
}

/* Overwrites pos/vel of a set (to start both implementations from one state). */
int GGO_SYM(write)(ggo_sys* s, int set, int field, const float* src, int64_t n) {
  r3* dst = NULL;
  if (set == GG_SET_GRANULAR) dst = field == GG_FIELD_POS ? s->pos : field == GG_FIELD_VEL ? s->vel : NULL;
  else if (set == GG_SET_UPSAMPLED) dst = field == GG_FIELD_POS ? s->upos : field == GG_FIELD_VEL ? s->uvel : NULL;
  if (!dst || n != GGO_SYM(size)(s, set)) return -1;
  for (int64_t i = 0; i < n; ++i) dst[i] = v3((real)src[3 * i], (real)src[3 * i + 1], (real)src[3 * i + 2]);
  return 0;
}

/* animateParticles, main.cu:1175-1208: the flagged walls move by t, then
 * turn by rotation_deg about the z axis through c.  The angle is
 * rotation * M_PI / 180.0f as the reference evaluates it (double, rounded
 * to float). */
void GGO_SYM(animate_walls)(ggo_sys* s, const float t[3], float rotation_deg, const float c[3]) {
  const real angle = (real)(float)((double)rotation_deg * GGO_PI_D / 180.0);
  const real ct = R_COS(angle), st = R_SIN(angle);
  for (int64_t i = 0; i < s->nb; ++i) {
    if (s->banim[i] != 1) continue;
    r3 p = s->bpos[i];
    p = v3(p.x + (real)t[0], p.y + (real)t[1], p.z + (real)t[2]);
    if (rotation_deg != 0.0f) {
      p.x = p.x - (real)c[0];
      p.y = p.y - (real)c[1];
      const real nx = p.x * ct - p.y * st;
      const real ny = p.x * st + p.y * ct;
      p.x = nx + (real)c[0];
      p.y = ny + (real)c[1];
    }
    s->bpos[i] = p;
  }
}

/* Stand-alone grid: unsorted keys, stable sort, cell start. */
void GGO_SYM(grid_build)(const float* pos, int64_t n, const int32_t cell_size[3], float cell_length,
                         int32_t* keys, int32_t* sorted_keys, int32_t* perm, int32_t* cell_start) {
  ggo_sys s;
  memset(&s, 0, sizeof(s));
  s.nx = cell_size[0]; s.ny = cell_size[1]; s.nz = cell_size[2];
  s.C = s.nx * s.ny * s.nz;
  s.L = (real)cell_length;
  r3* p = (r3*)xcalloc((size_t)n, sizeof(r3));
  for (int64_t i = 0; i < n; ++i) p[i] = v3((real)pos[3 * i], (real)pos[3 * i + 1], (real)pos[3 * i + 2]);
  map_to_cells(&s, p, n, keys);
  int32_t* counts = (int32_t*)xcalloc((size_t)s.C + 2, sizeof(int32_t));
  stable_sort(s.C, keys, n, perm, sorted_keys, counts);
  build_cell_start(s.C, sorted_keys, n, cell_start);
  free(counts);
  free(p);
}

int GGO_SYM(save_particle_stats)(const ggo_sys* s, const char* path) {
  FILE* f = fopen(path, "w");
  if (!f) return -1;
  fprintf(f, "Frame,MergedParticles,SplitParticles,TotalParticles\n");
  for (int64_t i = 0; i < s->stats_len; ++i)
    fprintf(f, "%lld,%lld,%lld,%lld\n", (long long)i, (long long)s->stats[3 * i],
            (long long)s->stats[3 * i + 1], (long long)s->stats[3 * i + 2]);
  fclose(f);
  return 0;
}

int32_t GGO_SYM(error_word)(const ggo_sys* s) { return s->error_word; }

int GGO_SYM(threads)(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void GGO_SYM(destroy)(ggo_sys* s) {
  if (!s) return;
  void* ptrs[] = {s->pos, s->vel, s->pos_t, s->delta, s->mass, s->scaled_mass, s->inv_m, s->rc, s->rb,
                  s->rs, s->units, s->als, s->surface, s->remove, s->merge_count, s->merge_units, s->sdist,
                  s->merge, s->merge_vel, s->cover, s->keys, s->perm, s->cell_start, s->ncon, s->contacts,
                  s->rev, s->tmp_i, s->tmp_r, s->tmp_3, s->prop, s->winner, s->ldens, s->split_flag,
                  s->child_pos, s->child_cell, s->fdelta, s->fcount, s->pn, s->bpos, s->banim, s->bkeys, s->bcell_start, s->upos, s->uvel, s->ukeys,
                  s->stats};
  for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); ++k) free(ptrs[k]);
  free(s);
}

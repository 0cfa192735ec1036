// system.cu — lifetime and per-substep orchestration of a gg_system.
//
// GranularSystem::GranularSystem (GranularSystem.cu:30-63) and
// GranularSystem::step (GranularSystem.cu:397-453) on one stream: every
// buffer is allocated at create time with a particle capacity, so a substep
// allocates nothing and synchronises only to learn the particle count after
// an adaptive step (the reference reads its split count back at the same
// point, Solver.cu:1162-1163).
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>

#include "common.cuh"

namespace gg {

// ------------------------------------------------------------ profiling

static cudaEvent_t prof_event(gg_system* S) {
  if (S->prof_pool_used == S->prof_pool.size()) {
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    S->prof_pool.push_back(e);
  }
  return S->prof_pool[S->prof_pool_used++];
}

void prof_begin(gg_system* S, int cls, cudaStream_t st) {
  if (!S || !S->profiling) return;
  gg_system::ProfEv ev;
  ev.a = prof_event(S);
  ev.b = nullptr;
  ev.cls = cls;
  ev.units = 0;
  cudaEventRecord(ev.a, st);
  S->prof_pending.push_back(ev);
}

void prof_end(gg_system* S, int cls, int64_t units, cudaStream_t st) {
  if (!S || !S->profiling) return;
  for (auto it = S->prof_pending.rbegin(); it != S->prof_pending.rend(); ++it) {
    if (it->cls == cls && it->b == nullptr) {
      it->b = prof_event(S);
      it->units = units;
      cudaEventRecord(it->b, st);
      return;
    }
  }
}

void prof_flush(gg_system* S) {
  if (S->prof_pending.empty()) return;
  cudaStreamSynchronize(S->stream);
  for (auto& e : S->prof_pending) {
    if (!e.b) continue;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e.a, e.b);
    S->prof_ms[e.cls] += ms;
    S->prof_launches[e.cls] += 1;
    S->prof_units[e.cls] += e.units;
  }
  S->prof_pending.clear();
  S->prof_pool_used = 0;
}

const char* prof_name(int cls) {
  static const char* kNames[PC_COUNT] = {"hash", "sort", "reorder", "cell_start", "predict", "sweep",
                                         "apply", "finalize", "upsample", "up_grid", "surface",
                                         "surf_dist", "merge", "split", "compact", "stats",
                                         "features", "mlp", "residual"};
  return (cls >= 0 && cls < PC_COUNT) ? kNames[cls] : "?";
}

// ------------------------------------------------------------ grids

// neighbor_search_boundary, GranularSystem.cu:174-280.
gg_status boundary_grid(gg_system* S) {
  cudaStream_t st = S->stream;
  if (S->nb > 0) {
    gg_status rc = grid_sort(S->grid, S->b.pos, S->nb, S->sort, S->b.keys, S->b.perm, nullptr, st, nullptr);
    if (rc != GG_OK) return rc;
    rc = reorder_boundary(S, S->b.perm, st);
    if (rc != GG_OK) return rc;
  }
  return cell_start_build(S->grid, S->b.keys, S->nb, S->b.cell_start, S->sort, st, nullptr);
}

// neighbor_search_granular, GranularSystem.cu:65-173.
gg_status granular_grid(gg_system* S) {
  cudaStream_t st = S->stream;
  S->n_grid = S->n;
  gg_status rc = grid_sort(S->grid, S->g.pos[S->g.cur], S->n, S->sort, S->g.keys, S->g.perm, nullptr, st, S);
  if (rc != GG_OK) return rc;
  rc = reorder_granular(S, st);
  if (rc != GG_OK) return rc;
  return cell_start_build(S->grid, S->g.keys, S->n, S->g.cell_start, S->sort, st, S);
}

// neighbor_search_upsampled, GranularSystem.cu:282-395.  Its cell table is
// never read by the reference, so only the stable reorder is kept.
gg_status upsampled_grid(gg_system* S) {
  if (S->nu <= 0) return GG_OK;
  cudaStream_t st = S->stream;
  prof_begin(S, PC_UP_GRID, st);
  gg_status rc = grid_sort(S->grid, S->u.pos[S->u.cur], S->nu, S->sort, S->u.keys, S->u.perm, nullptr, st, nullptr);
  if (rc != GG_OK) return rc;
  rc = reorder_upsampled(S, S->u.perm, st);
  prof_end(S, PC_UP_GRID, S->nu, st);
  return rc;
}

// ------------------------------------------------------------ substep

gg_status step_once(gg_system* S) {
  cudaStream_t st = S->stream;
  if (S->frame_timing) cudaEventRecord(S->frame_ev[0], st);
  GG_CUDA(cudaMemsetAsync(S->scal, 0, offsetof(DevScalars, error_word), st));
  gg_status rc = GG_OK;
  if (S->phys.is_move_boundary && (rc = boundary_grid(S)) != GG_OK) return rc;
  if ((rc = granular_grid(S)) != GG_OK) return rc;
  if ((rc = upsampled_grid(S)) != GG_OK) return rc;
  // Solver::step, Solver.cu:82-109
  if ((rc = predict(S, st)) != GG_OK) return rc;
  if (S->P.warm_start == 1 && (rc = warm_start_apply(S, st)) != GG_OK) return rc;
  if (S->P.warm_start == 2 && (rc = warm_start_record(S, st)) != GG_OK) return rc;
  // Coulomb law: the normal correction each particle receives accumulates over the substep
  if (S->P.contact_law == 1 && S->n > 0) GG_CUDA(cudaMemsetAsync(S->g.pn, 0, sizeof(float) * (size_t)S->n, st));
  if (S->P.target_residual > 0.0f) {
    // residual mode: the stabilisation sweeps, then Jacobi sweeps until the
    // largest penetration, measured before each sweep, is within the target
    const int stab = S->P.stab_iters;
    for (int it = 0; it < stab; ++it) {
      if ((rc = sweep(S, it, st)) != GG_OK) return rc;
      if ((rc = apply(S, it, true, false, true, st)) != GG_OK) return rc;
    }
    const int cap = std::max(0, std::min(S->P.max_sweeps, kMaxSweeps - stab));
    int k = 0;
    float res = 0.0f;
    for (;;) {
      if ((rc = residual(S, st, &res)) != GG_OK) return rc;
      if (!(res > S->P.target_residual) || k >= cap) break;
      if ((rc = sweep(S, stab + k, st)) != GG_OK) return rc;
      if ((rc = apply(S, stab + k, false, true, true, st)) != GG_OK) return rc;
      ++k;
    }
    S->last_sweeps = k;
    S->last_residual = res;
  } else {
    const int total = std::min(S->P.stab_iters + S->P.iters, kMaxSweeps);
    for (int it = 0; it < total; ++it) {
      if ((rc = sweep(S, it, st)) != GG_OK) return rc;
      if ((rc = apply(S, it, it < S->P.stab_iters, it == total - 1, it < total - 1, st)) != GG_OK) return rc;
    }
  }
  if (S->P.warm_start == 2 && (rc = warm_start_target(S, st)) != GG_OK) return rc;
  if ((rc = finalize(S, st)) != GG_OK) return rc;
  if (S->P.upsample_enabled && (rc = upsample(S, st)) != GG_OK) return rc;
  if (S->phys.is_adaptive == 1 && S->P.merge_enabled && S->n > 0) {
    if ((rc = surface(S, st)) != GG_OK) return rc;
    if ((rc = surface_distance(S, st)) != GG_OK) return rc;
    // Solver::adaptive_sampling, Solver.cu:856-1242; merge marking is skipped
    // on the first call only (t_merge_iter, Solver.cu:36,910-922), here per
    // system instead of per process.
    if (S->merge_iter == 1) {
      if ((rc = merge_mark(S, st)) != GG_OK) return rc;
      S->merge_iter = 0;
    }
    S->merge_iter++;
    if ((rc = merge_count(S, st)) != GG_OK) return rc;
    if ((rc = split_and_compact(S, st)) != GG_OK) return rc;
    GG_CUDA(cudaMemcpyAsync(S->scal_host, S->scal, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    const int64_t before = S->n;
    // k_compact wrote the other buffers unless nothing was removed or split
    if (!(S->scal_host->n_kept == before && S->scal_host->n_split == 0)) S->g.cur ^= 1;
    S->n = S->scal_host->n_after;
    S->merged_last = S->scal_host->n_removed;
    S->split_last = S->scal_host->n_split;
    S->merged_total += S->merged_last;
    S->split_total += S->split_last;
    S->stats_rows.push_back(S->merged_last);
    S->stats_rows.push_back(S->split_last);
    S->stats_rows.push_back(before);
    S->error_word |= S->scal_host->error_word;
  }
  S->steps++;
  if (S->frame_timing) {
    cudaEventRecord(S->frame_ev[1], st);
    cudaEventSynchronize(S->frame_ev[1]);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, S->frame_ev[0], S->frame_ev[1]);
    S->frame_times.push_back(ms);
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ------------------------------------------------------------ create

template <typename T>
static cudaError_t dalloc(T** p, int64_t n) {
  return cudaMalloc((void**)p, sizeof(T) * (size_t)std::max<int64_t>(n, 1));
}

static void free_all(gg_system* S) {
  Granular& G = S->g;
  for (int k = 0; k < 2; ++k) {
    cudaFree(G.pos[k]); cudaFree(G.vel[k]); cudaFree(G.mass[k]); cudaFree(G.rs[k]);
    cudaFree(G.units[k]); cudaFree(G.merge[k]); cudaFree(G.merge_units[k]);
    cudaFree(G.merge_count[k]); cudaFree(G.remove[k]); cudaFree(G.als[k]);
    cudaFree(S->u.pos[k]); cudaFree(S->u.vel[k]);
  }
  void* ptrs[] = {G.merge_vel, G.surface, G.sdist, G.cover, G.xs, G.inv_m, G.delta, G.s_extra, G.contacts,
                  G.ncon, G.keys, G.perm, G.cell_start, G.cell_surf, G.prop, G.ldens, G.winner, G.split_flag, G.keep_flag,
                  G.split_slot, G.keep_slot, G.child_pos, G.nl_idx, G.nl_meta, G.nl_acc, G.nl_queue, G.cell_inc, G.ld_sum, G.ld_cnt, G.claim_tgt, G.claimed, G.cell_claim, G.child_cell, G.fdelta, G.pn, S->b.pos, S->b.animated, S->b.pos_alt,
                  S->b.animated_alt, S->b.keys, S->b.perm, S->b.cell_start, S->u.keys, S->u.perm, S->scal,
                  S->stats_partial, S->stage, S->feat, S->xs0, S->warm_target, S->scene_fcap,
                  S->scene_acc, S->scene_mu};
  for (void* p : ptrs) cudaFree(p);
  if (S->scal_host) cudaFreeHost(S->scal_host);
  sort_scratch_free(S->sort);
  for (auto e : S->prof_pool) cudaEventDestroy(e);
  for (auto e : S->frame_ev)
    if (e) cudaEventDestroy(e);
  if (S->own_stream && S->stream) cudaStreamDestroy(S->stream);
}

// Packs host float[3] into device float4 (w = 0) with one strided copy.
static cudaError_t upload3(float4* dst, const float* src, int64_t n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(dst, 0, sizeof(float4) * (size_t)n, st);
  if (e != cudaSuccess) return e;
  return cudaMemcpy2DAsync(dst, sizeof(float4), src, 3 * sizeof(float), 3 * sizeof(float), (size_t)n,
                           cudaMemcpyHostToDevice, st);
}

gg_status system_create(const gg_desc* d, gg_system** out) {
  if (!d || !out) {
    set_error("gg_create: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  if (d->n_particles < 0 || d->n_boundary < 0 || d->n_upsampled < 0 ||
      (d->n_particles > 0 && !d->particles) || (d->n_boundary > 0 && !d->boundary) ||
      (d->n_upsampled > 0 && !d->upsampled)) {
    set_error("gg_create: particle counts/pointers are inconsistent");
    return GG_ERR_INVALID_ARGUMENT;
  }
  if (!(d->cell_length > 0.0f) || d->cell_size[0] <= 0 || d->cell_size[1] <= 0 || d->cell_size[2] <= 0) {
    set_error("gg_create: cell_length and cell_size must be positive");
    return GG_ERR_INVALID_ARGUMENT;
  }
  const int64_t C64 = (int64_t)d->cell_size[0] * d->cell_size[1] * d->cell_size[2];
  if (C64 >= (int64_t)1 << 30) {
    set_error("gg_create: grid has too many cells (max 2^30)");
    return GG_ERR_INVALID_ARGUMENT;
  }
  if (d->params.stab_iters < 0 || d->params.iters < 0 || d->params.stab_iters + d->params.iters > 64 ||
      d->params.blend_factor <= 0) {
    set_error("gg_create: iteration counts must be in 0..64 and blend_factor > 0");
    return GG_ERR_INVALID_ARGUMENT;
  }
  if (d->params.merge_cas_lag < 0 || d->params.merge_cas_lag > 65536) {
    set_error("gg_create: merge_cas_lag must be in 0..65536");
    return GG_ERR_INVALID_ARGUMENT;
  }
  if ((d->params.contact_law != 0 && d->params.contact_law != 1) || d->params.n_planes < 0 ||
      d->params.n_planes > 8) {
    set_error("gg_create: contact_law must be 0 or 1 and n_planes in 0..8");
    return GG_ERR_INVALID_ARGUMENT;
  }
  int64_t cap = d->max_particles > 0 ? d->max_particles : 2 * d->n_particles;
  cap = std::max<int64_t>(cap, std::max<int64_t>(d->n_particles, 1));
  // a launch rounds its count up to whole tiles (at most 4,096 items), and
  // thread and tile indices are signed 32-bit: counts stay 2^16 below 2^31
  if (cap > kMaxCount || d->n_upsampled > kMaxCount || d->n_boundary > kMaxCount) {
    set_error("gg_create: particle counts must not exceed 2^31 - 2^16");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(d->device));
  gg_system* S = new gg_system();
  S->device = d->device;
  S->P = d->params;
  S->grid.L = d->cell_length;
  S->grid.nx = d->cell_size[0];
  S->grid.ny = d->cell_size[1];
  S->grid.nz = d->cell_size[2];
  S->grid.C = (int)C64;
  S->phys.dt = d->dt;
  S->phys.g = make_float3(d->gravity[0], d->gravity[1], d->gravity[2]);
  S->phys.density = d->density;
  S->phys.rho_i = (int)d->density;
  for (int k = 0; k < 3; ++k) S->phys.space[k] = d->space_size[k];
  S->phys.upsampled_radius = d->upsampled_radius;
  S->phys.is_move_boundary = d->is_move_boundary;
  S->phys.is_adaptive = d->is_adaptive;
  S->n = d->n_particles;
  S->cap = cap;
  S->nb = d->n_boundary;
  S->nu = d->n_upsampled;
  cudaDeviceGetAttribute(&S->num_sms, cudaDevAttrMultiProcessorCount, d->device);

  cudaError_t e = cudaSuccess;
#define ALLOC(ptr, cnt)                                 \
  do {                                                  \
    if (e == cudaSuccess) e = dalloc(&(ptr), (cnt));    \
  } while (0)
  if (d->stream) {
    S->stream = (cudaStream_t)d->stream;
  } else {
    e = cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking);
    S->own_stream = true;
  }
  Granular& G = S->g;
  const int64_t C1 = C64 + 1;
  for (int k = 0; k < 2; ++k) {
    ALLOC(G.pos[k], cap); ALLOC(G.vel[k], cap); ALLOC(G.mass[k], cap); ALLOC(G.rs[k], cap);
    ALLOC(G.units[k], cap); ALLOC(G.merge[k], cap); ALLOC(G.merge_units[k], cap);
    ALLOC(G.merge_count[k], cap); ALLOC(G.remove[k], cap); ALLOC(G.als[k], cap);
    ALLOC(S->u.pos[k], S->nu); ALLOC(S->u.vel[k], S->nu);
  }
  ALLOC(G.merge_vel, cap); ALLOC(G.surface, cap); ALLOC(G.sdist, cap); ALLOC(G.cover, cap);
  ALLOC(G.xs, cap); ALLOC(G.inv_m, cap); ALLOC(G.delta, cap); ALLOC(G.s_extra, cap);
  ALLOC(G.contacts, cap); ALLOC(G.ncon, cap); ALLOC(G.keys, cap); ALLOC(G.perm, cap);
  ALLOC(G.cell_start, C1); ALLOC(G.cell_surf, C1); ALLOC(G.prop, cap); ALLOC(G.ldens, cap); ALLOC(G.winner, cap);
  ALLOC(G.split_flag, cap); ALLOC(G.keep_flag, cap); ALLOC(G.split_slot, cap); ALLOC(G.keep_slot, cap);
  ALLOC(G.child_pos, cap); ALLOC(G.ld_sum, cap); ALLOC(G.ld_cnt, cap);
  ALLOC(G.claim_tgt, cap); ALLOC(G.claimed, 2 * cap);
  ALLOC(G.cell_claim, C64); ALLOC(G.child_cell, cap); ALLOC(G.fdelta, cap); ALLOC(G.pn, cap);
  if (e == cudaSuccess) e = cudaMemset(G.cell_claim, 0xff, sizeof(uint32_t) * (size_t)std::max<int64_t>(C64, 1));
  // contact lists: a negative skin asks for the automatic one, a tenth of
  // the cell length; zero or NaN turns them off
  S->nl_skin = S->P.nlist_skin < 0.0f ? 0.1f * S->grid.L : S->P.nlist_skin;
  if (!(S->nl_skin > 0.0f) || !std::isfinite(S->nl_skin)) S->nl_skin = 0.0f;
  if (S->nl_skin > 0.0f) {
    ALLOC(G.nl_idx, (int64_t)kNlistMax * cap);
    ALLOC(G.nl_meta, cap);
    ALLOC(G.nl_acc, cap);
    ALLOC(G.nl_queue, cap);
    ALLOC(G.cell_inc, C1);
  }
  ALLOC(S->b.pos, S->nb); ALLOC(S->b.animated, S->nb); ALLOC(S->b.pos_alt, S->nb);
  ALLOC(S->b.animated_alt, S->nb); ALLOC(S->b.keys, S->nb); ALLOC(S->b.perm, S->nb);
  ALLOC(S->b.cell_start, C1);
  ALLOC(S->u.keys, S->nu); ALLOC(S->u.perm, S->nu);
  ALLOC(S->scal, 1);
  S->stats_blocks = std::max(1, std::min(4 * S->num_sms, 1024));
  ALLOC(S->stats_partial, (int64_t)S->stats_blocks * 16);
  ALLOC(S->stage, 3 * std::max<int64_t>(std::max(cap, S->nu), S->nb));
#undef ALLOC
  if (e == cudaSuccess) e = cudaMallocHost((void**)&S->scal_host, sizeof(DevScalars));
  if (e != cudaSuccess) {
    free_all(S);
    delete S;
    cudaGetLastError();
    set_error(std::string("gg_create: device allocation failed: ") + cudaGetErrorString(e));
    return GG_ERR_OUT_OF_MEMORY;
  }
  gg_status rc = sort_scratch_alloc(S->sort, std::max<int64_t>(std::max(cap, S->nu), std::max<int64_t>(S->nb, 1)));
  S->sort.counter = &S->launches;
  if (rc != GG_OK) {
    free_all(S);
    delete S;
    return GG_ERR_OUT_OF_MEMORY;
  }
  cudaEventCreate(&S->frame_ev[0]);
  cudaEventCreate(&S->frame_ev[1]);
  cudaStream_t st = S->stream;
  auto fail = [&](gg_status r) {
    cudaStreamSynchronize(st);
    free_all(S);
    delete S;
    return r;
  };
#define CHK(x)                                                   \
  do {                                                           \
    cudaError_t e2 = (x);                                        \
    if (e2 != cudaSuccess) return fail(cuda_status(e2, #x));     \
  } while (0)
  const int c = G.cur;
  CHK(upload3(G.pos[c], d->particles, S->n, st));
  CHK(cudaMemsetAsync(G.vel[c], 0, sizeof(float4) * cap, st));
  {
    std::vector<float> m((size_t)std::max<int64_t>(S->n, 1), 1.0f);
    std::vector<int32_t> u((size_t)std::max<int64_t>(S->n, 1), 0);
    for (int64_t i = 0; i < S->n; ++i) {
      float mi = d->masses ? d->masses[i] : 1.0f;
      const double units = (double)mi * (double)(1 << 20);
      u[i] = (int32_t)llrint(units);
      if (S->P.mass_ledger) mi = (float)((double)u[i] / (double)(1 << 20));
      m[i] = mi;
    }
    CHK(cudaMemcpyAsync(G.mass[c], m.data(), sizeof(float) * S->n, cudaMemcpyHostToDevice, st));
    CHK(cudaMemcpyAsync(G.units[c], u.data(), sizeof(int32_t) * S->n, cudaMemcpyHostToDevice, st));
    // the host vectors must outlive the async copies
    CHK(cudaStreamSynchronize(st));
  }
  for (int k = 0; k < 2; ++k) {
    CHK(cudaMemsetAsync(G.merge[k], 0, sizeof(float) * cap, st));
    CHK(cudaMemsetAsync(G.merge_units[k], 0, sizeof(int32_t) * cap, st));
    CHK(cudaMemsetAsync(G.merge_count[k], 0, sizeof(int32_t) * cap, st));
    CHK(cudaMemsetAsync(G.remove[k], 0, sizeof(int32_t) * cap, st));
    CHK(cudaMemsetAsync(G.als[k], 0, sizeof(int32_t) * cap, st));
  }
  CHK(cudaMemsetAsync(G.merge_vel, 0, sizeof(float4) * cap, st));
  CHK(cudaMemsetAsync(G.surface, 0, sizeof(int32_t) * cap, st));
  CHK(cudaMemsetAsync(G.sdist, 0, sizeof(float) * cap, st));
  CHK(cudaMemsetAsync(G.s_extra, 0, sizeof(int32_t) * cap, st));
  CHK(cudaMemsetAsync(G.contacts, 0, sizeof(int32_t) * cap, st));
  CHK(cudaMemsetAsync(G.ncon, 0, sizeof(int32_t) * cap, st));
  CHK(cudaMemsetAsync(S->scal, 0, sizeof(DevScalars), st));
  CHK(upload3(S->b.pos, d->boundary, S->nb, st));
  if (S->nb > 0) {
    if (d->boundary_animated)
      CHK(cudaMemcpyAsync(S->b.animated, d->boundary_animated, sizeof(int32_t) * S->nb, cudaMemcpyHostToDevice, st));
    else
      CHK(cudaMemsetAsync(S->b.animated, 0, sizeof(int32_t) * S->nb, st));
  }
  CHK(upload3(S->u.pos[S->u.cur], d->upsampled, S->nu, st));
  if (S->nu > 0) CHK(cudaMemsetAsync(S->u.vel[S->u.cur], 0, sizeof(float4) * S->nu, st));
#undef CHK
  // constructor sequence, GranularSystem.cu:54-62
  if ((rc = radii_all(S, st)) != GG_OK) return fail(rc);
  if ((rc = boundary_grid(S)) != GG_OK) return fail(rc);
  if ((rc = granular_grid(S)) != GG_OK) return fail(rc);
  if ((rc = upsampled_grid(S)) != GG_OK) return fail(rc);
  if (!d->skip_initial_step && (rc = step_once(S)) != GG_OK) return fail(rc);
  cudaError_t se = cudaStreamSynchronize(st);
  if (se != cudaSuccess) return fail(cuda_status(se, "gg_create: initial step"));
  *out = S;
  return GG_OK;
}

void system_destroy(gg_system* S) {
  if (!S) return;
  cudaSetDevice(S->device);
  cudaStreamSynchronize(S->stream);
  if (S->graph_exec) cudaGraphExecDestroy(S->graph_exec);
  free_all(S);
  delete S;
}

// ------------------------------------------------------------ stats

constexpr int kStatSlots = 12;  // mass, units, mom xyz, ke, mx, my, mz, nonfinite, (pad)

__global__ void k_stats_partial(int n, const float4* __restrict__ pos, const float4* __restrict__ vel,
                                const float* __restrict__ mass, const int32_t* __restrict__ units,
                                double* __restrict__ partial) {
  __shared__ double sh[kStatSlots][256];
  double acc[kStatSlots];
#pragma unroll
  for (int k = 0; k < kStatSlots; ++k) acc[k] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double m = mass[i];
    const float4 p = pos[i];
    const float4 v = vel[i];
    acc[0] += m;
    acc[1] += (double)units[i];
    acc[2] += m * v.x;
    acc[3] += m * v.y;
    acc[4] += m * v.z;
    acc[5] += 0.5 * m * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
    acc[6] += m * p.x;
    acc[7] += m * p.y;
    acc[8] += m * p.z;
    acc[9] += (isfinite(p.x) && isfinite(p.y) && isfinite(p.z)) ? 0.0 : 1.0;
  }
#pragma unroll
  for (int k = 0; k < kStatSlots; ++k) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
#pragma unroll
      for (int k = 0; k < kStatSlots; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x < kStatSlots) partial[blockIdx.x * 16 + threadIdx.x] = sh[threadIdx.x][0];
}

// max over found contacts of r_i + r_j - |x_i - x_j| on the current grid.
__global__ void k_penetration(Grid g, int n, const float4* __restrict__ pos, const int32_t* __restrict__ cs,
                              unsigned int* __restrict__ out_bits) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float best = 0.0f;
  if (i < n) {
    const float4 xi = pos[i];
    const int3 q = trunc_cell(g, f3(xi));
    for (int m = 0; m < 27; ++m) {
      const int cell = cell_key(g, q.x + m / 9 - 1, q.y + (m % 9) / 3 - 1, q.z + m % 3 - 1);
      if (cell == g.C) continue;
      for (int j = cs[cell]; j < cs[cell + 1]; ++j) {
        if (j == i) continue;
        const float4 xj = pos[j];
        const float pen = (xi.w + xj.w) - norm3df(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        if (pen > best) best = pen;
      }
    }
  }
  warp_max_bits(out_bits, __float_as_uint(best));
}

gg_status stats_compute(gg_system* S, gg_stats_t* out) {
  memset(out, 0, sizeof(*out));
  cudaStream_t st = S->stream;
  const int c = S->g.cur;
  out->n_particles = S->n;
  out->n_boundary = S->nb;
  out->n_upsampled = S->nu;
  out->steps = S->steps;
  out->merged_last = S->merged_last;
  out->split_last = S->split_last;
  out->merged_total = S->merged_total;
  out->split_total = S->split_total;
  out->launches = S->launches;
  std::vector<double> part((size_t)S->stats_blocks * 16, 0.0);
  unsigned int pen_bits = 0;
  if (S->n > 0) {
    k_stats_partial<<<S->stats_blocks, 256, 0, st>>>((int)S->n, S->g.pos[c], S->g.vel[c], S->g.mass[c],
                                                     S->g.units[c], S->stats_partial);
    GG_CUDA(cudaMemsetAsync(&S->scal->rmax_bits, 0, sizeof(unsigned int), st));
    k_penetration<<<blocks_for(S->n, 256), 256, 0, st>>>(S->grid, (int)S->n, S->g.pos[c], S->g.cell_start,
                                                         &S->scal->rmax_bits);
    count_launches(S, 2);
    GG_CUDA(cudaMemcpyAsync(part.data(), S->stats_partial, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaMemcpyAsync(S->scal_host, S->scal, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
  }
  GG_CUDA(cudaStreamSynchronize(st));
  if (S->n > 0) pen_bits = S->scal_host->rmax_bits;
  double acc[kStatSlots] = {0};
  for (int b = 0; b < S->stats_blocks; ++b)
    for (int k = 0; k < kStatSlots; ++k) acc[k] += part[(size_t)b * 16 + k];
  out->total_mass = acc[0];
  out->total_mass_units = (int64_t)llround(acc[1]);
  for (int k = 0; k < 3; ++k) out->momentum[k] = acc[2 + k];
  out->kinetic_energy = acc[5];
  for (int k = 0; k < 3; ++k) out->center_of_mass[k] = acc[0] > 0 ? acc[6 + k] / acc[0] : 0.0;
  out->nonfinite = (int32_t)acc[9];
  float pen;
  memcpy(&pen, &pen_bits, sizeof(pen));
  out->max_penetration = pen;
  out->error_word = S->error_word;
  out->last_sweeps = S->last_sweeps;
  out->last_residual = S->last_residual;
  out->last_residual_max = S->last_residual_max;
  return GG_OK;
}

}  // namespace gg

// ------------------------------------------------------------ host copies

namespace gg {

constexpr int kPackThreads = 256;

// float4 -> packed float[3]: each block stages its 256 elements in shared
// memory and writes them back as 768 consecutive floats (coalesced).
__global__ void __launch_bounds__(kPackThreads) k_pack3(const float4* __restrict__ src, float* __restrict__ dst,
                                                         int64_t n) {
  __shared__ float s[3 * kPackThreads];
  const int64_t base = (int64_t)blockIdx.x * kPackThreads;
  const int t = threadIdx.x;
  if (base + t < n) {
    const float4 v = src[base + t];
    s[3 * t] = v.x;
    s[3 * t + 1] = v.y;
    s[3 * t + 2] = v.z;
  }
  __syncthreads();
  const int cnt = 3 * (int)(n - base < kPackThreads ? n - base : kPackThreads);
  for (int k = t; k < cnt; k += kPackThreads) dst[3 * base + k] = s[k];
}

__global__ void __launch_bounds__(kPackThreads) k_unpack3(const float* __restrict__ src, float4* __restrict__ dst,
                                                           int64_t n) {
  __shared__ float s[3 * kPackThreads];
  const int64_t base = (int64_t)blockIdx.x * kPackThreads;
  const int t = threadIdx.x;
  const int cnt = 3 * (int)(n - base < kPackThreads ? n - base : kPackThreads);
  for (int k = t; k < cnt; k += kPackThreads) s[k] = src[3 * base + k];
  __syncthreads();
  if (base + t < n) {
    float4 v = dst[base + t];
    v.x = s[3 * t];
    v.y = s[3 * t + 1];
    v.z = s[3 * t + 2];
    dst[base + t] = v;
  }
}

cudaError_t pack3(gg_system* S, const float4* src, float* dst, int64_t n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_pack3<<<(unsigned)((n + kPackThreads - 1) / kPackThreads), kPackThreads, 0, st>>>(src, dst, n);
  count_launches(S, 1);
  return cudaGetLastError();
}

cudaError_t unpack3(gg_system* S, const float* src, float4* dst, int64_t n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_unpack3<<<(unsigned)((n + kPackThreads - 1) / kPackThreads), kPackThreads, 0, st>>>(src, dst, n);
  count_launches(S, 1);
  return cudaGetLastError();
}

}  // namespace gg

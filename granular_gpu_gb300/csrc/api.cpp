// api.cpp — the extern "C" surface of libgg.so (include/gg.h).
//
// Every entry point validates its arguments, converts CUDA and C++ failures
// into a gg_status and records a message for gg_last_error(); nothing throws
// across the ABI.  The reference's equivalents print and continue
// (CUDA_CALL, Global.hpp:8-16) or throw std::runtime_error (DArray.hpp:18-44).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "gg_internal.h"
#include "scene.h"

namespace gg {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

gg_status cuda_status(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return GG_ERR_OUT_OF_MEMORY;
  return GG_ERR_CUDA;
}

gg_status system_create(const gg_desc* d, gg_system** out);
void system_destroy(gg_system* S);
gg_status step_once(gg_system* S);
void prof_flush(gg_system* S);
const char* prof_name(int cls);
gg_status boundary_grid(gg_system* S);
gg_status granular_grid(gg_system* S);

}  // namespace gg

using namespace gg;

#define GG_GUARD_BEGIN try {
#define GG_GUARD_END                                           \
  }                                                            \
  catch (const std::exception& ex) {                           \
    set_error(std::string("internal error: ") + ex.what());    \
    return GG_ERR_INVALID_ARGUMENT;                            \
  }                                                            \
  catch (...) {                                                \
    set_error("internal error");                               \
    return GG_ERR_INVALID_ARGUMENT;                            \
  }

#define REQUIRE(cond, msg)                \
  do {                                    \
    if (!(cond)) {                        \
      set_error(msg);                     \
      return GG_ERR_INVALID_ARGUMENT;     \
    }                                     \
  } while (0)

extern "C" {

int32_t gg_abi_version(void) { return GG_ABI_VERSION; }

gg_status gg_struct_sizes(int64_t* sizes, int32_t n) {
  REQUIRE(sizes && n >= 0, "gg_struct_sizes: null buffer");
  const int64_t s[5] = {(int64_t)sizeof(gg_params), (int64_t)sizeof(gg_desc), (int64_t)sizeof(gg_overrides),
                        (int64_t)sizeof(gg_stats_t), (int64_t)sizeof(gg_profile_t)};
  for (int i = 0; i < n && i < 5; ++i) sizes[i] = s[i];
  return GG_OK;
}

const char* gg_last_error(void) { return g_last_error.c_str(); }

gg_status gg_default_params(gg_params* P) {
  REQUIRE(P, "gg_default_params: null");
  memset(P, 0, sizeof(*P));
  P->stab_iters = 3;
  P->iters = 5;
  P->boundary_radius = 0.01;
  P->boundary_min_radius = 0.01f;
  P->friction_cap = 0.8;
  P->rest_speed = 0.01f;
  P->damp_min_speed = 1.0f;
  P->damp_max_speed = 10.0f;
  P->damp_min = 0.99f;
  P->damp_max = 0.99f;
  P->damp_exp_rate = 0.1f;
  P->adaptive_damp = 0.98f;
  P->max_mass = 4.0f;
  P->min_merge_mass = 1.0f;
  P->merge_radius = 0.035;
  P->surface_dist_threshold = 100.0f;
  P->target_density = 100.0f;
  P->blend_factor = 40;
  P->split_min_mass = 2.0f;
  P->surface_cone = 1.047197551f;
  P->surface_min_neighbors = 5;
  P->no_surface_distance = 100000.0f;
  P->up_inv_h2 = 493.8271605f;
  P->up_dt = 0.002f;
  P->up_gravity_y = -9.8f;
  P->up_boundary_radius = 0.015f;
  P->up_repulsion = 3.0f;
  P->up_max_velocity = 7.0f;
  P->up_floor_y = 0.04f;
  P->up_floor_friction = 0.95f;
  P->up_boundary_damping = 0.8f;
  P->up_ground_band = 0.1f;
  P->up_ground_damping = 0.5f;
  P->mass_ledger = 0;
  P->merge_enabled = 1;
  P->upsample_enabled = 1;
  P->nlist_skin = -1.0f;
  P->target_residual = 0.0f;
  P->max_sweeps = 200;
  P->warm_start = 0;
  P->warm_start_scale = 1.0f;
  P->merge_cas_lag = 4;
  P->contact_law = 0;
  P->mu_static = 0.5f;
  P->mu_kinetic = 0.4f;
  P->split_claim = 0;
  P->n_planes = 0;
  for (int k = 0; k < 8; ++k)
    for (int c = 0; c < 4; ++c) P->planes[k][c] = 0.0f;
  return GG_OK;
}

gg_status gg_create(const gg_desc* desc, gg_system** out) {
  GG_GUARD_BEGIN
  return system_create(desc, out);
  GG_GUARD_END
}

gg_status gg_scene_build(const char* json_path, const char* base_dir, float* particles, int64_t* n_particles,
                         float* boundary, int32_t* boundary_animated, int64_t* n_boundary, float* upsampled,
                         int64_t* n_upsampled, gg_desc* desc_out) {
  GG_GUARD_BEGIN
  REQUIRE(json_path && n_particles && n_boundary && n_upsampled, "gg_scene_build: null argument");
  SceneData sc;
  gg_status rc = scene_build(json_path, base_dir, sc);
  if (rc != GG_OK) return rc;
  const int64_t np = (int64_t)sc.particles.size() / 3, nb = (int64_t)sc.boundary.size() / 3,
                nu = (int64_t)sc.upsampled.size() / 3;
  const bool copy = particles != nullptr;
  if (copy) {
    REQUIRE(*n_particles >= np && *n_boundary >= nb && *n_upsampled >= nu, "gg_scene_build: buffers too small");
    memcpy(particles, sc.particles.data(), sizeof(float) * 3 * np);
    if (boundary) memcpy(boundary, sc.boundary.data(), sizeof(float) * 3 * nb);
    if (boundary_animated) memcpy(boundary_animated, sc.animated.data(), sizeof(int32_t) * nb);
    if (upsampled) memcpy(upsampled, sc.upsampled.data(), sizeof(float) * 3 * nu);
  }
  *n_particles = np;
  *n_boundary = nb;
  *n_upsampled = nu;
  if (desc_out) {
    *desc_out = sc.desc;
    desc_out->particles = copy ? particles : nullptr;
    desc_out->boundary = copy ? boundary : nullptr;
    desc_out->boundary_animated = copy ? boundary_animated : nullptr;
    desc_out->upsampled = copy ? upsampled : nullptr;
    desc_out->n_particles = np;
    desc_out->n_boundary = nb;
    desc_out->n_upsampled = nu;
  }
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_create_from_scene(const char* json_path, const gg_overrides* ov, gg_system** out) {
  GG_GUARD_BEGIN
  REQUIRE(json_path && out, "gg_create_from_scene: null argument");
  SceneData sc;
  gg_status rc = scene_build(json_path, ov ? ov->base_dir : nullptr, sc);
  if (rc != GG_OK) return rc;
  gg_desc d = sc.desc;
  d.particles = sc.particles.data();
  d.n_particles = (int64_t)sc.particles.size() / 3;
  d.boundary = sc.boundary.empty() ? nullptr : sc.boundary.data();
  d.n_boundary = (int64_t)sc.boundary.size() / 3;
  d.boundary_animated = sc.animated.empty() ? nullptr : sc.animated.data();
  d.upsampled = sc.upsampled.empty() ? nullptr : sc.upsampled.data();
  d.n_upsampled = (int64_t)sc.upsampled.size() / 3;
  if (ov) {
    if (ov->has_params) d.params = ov->params;
    d.device = ov->device;
    d.max_particles = ov->max_particles;
    d.stream = ov->stream;
    d.skip_initial_step = ov->skip_initial_step;
  }
  return system_create(&d, out);
  GG_GUARD_END
}

gg_status gg_step(gg_system* S, int32_t n_substeps) {
  GG_GUARD_BEGIN
  REQUIRE(S && n_substeps >= 0, "gg_step: invalid argument");
  GG_CUDA(cudaSetDevice(S->device));
  for (int32_t k = 0; k < n_substeps; ++k) {
    gg_status rc = step_once(S);
    if (rc != GG_OK) return rc;
  }
  if (S->error_word & ERR_CAPACITY) {
    set_error("gg_step: splits exceeded max_particles; extra children were dropped");
    S->error_word &= ~ERR_CAPACITY;
    return GG_ERR_CAPACITY;
  }
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_synchronize(gg_system* S) {
  REQUIRE(S, "gg_synchronize: null");
  GG_CUDA(cudaStreamSynchronize(S->stream));
  return GG_OK;
}

gg_status gg_size(gg_system* S, gg_set set, int64_t* n) {
  REQUIRE(S && n, "gg_size: null");
  switch (set) {
    case GG_SET_GRANULAR: *n = S->n; return GG_OK;
    case GG_SET_BOUNDARY: *n = S->nb; return GG_OK;
    case GG_SET_UPSAMPLED: *n = S->nu; return GG_OK;
  }
  set_error("gg_size: unknown set");
  return GG_ERR_INVALID_ARGUMENT;
}

gg_status gg_grid_dims(gg_system* S, int32_t cell_size[3], float* cell_length) {
  REQUIRE(S, "gg_grid_dims: null");
  if (cell_size) {
    cell_size[0] = S->grid.nx;
    cell_size[1] = S->grid.ny;
    cell_size[2] = S->grid.nz;
  }
  if (cell_length) *cell_length = S->grid.L;
  return GG_OK;
}

namespace {

struct FieldView {
  void* ptr = nullptr;
  int64_t count = 0;
  int elem = 4;    // bytes per element on the host side
  int stride = 4;  // bytes per element on the device side
};

bool field_view(gg_system* S, gg_set set, gg_field f, FieldView& v) {
  Granular& G = S->g;
  const int c = G.cur;
  if (set == GG_SET_GRANULAR) {
    v.count = S->n;
    switch (f) {
      case GG_FIELD_POS: v.ptr = G.pos[c]; v.elem = 12; v.stride = 16; return true;
      case GG_FIELD_VEL: v.ptr = G.vel[c]; v.elem = 12; v.stride = 16; return true;
      case GG_FIELD_MASS: v.ptr = G.mass[c]; return true;
      case GG_FIELD_MASS_UNITS: v.ptr = G.units[c]; return true;
      case GG_FIELD_SURFACE: v.ptr = G.surface; return true;
      case GG_FIELD_SURFACE_DISTANCE: v.ptr = G.sdist; return true;
      case GG_FIELD_CELL_KEY: v.ptr = G.keys; v.count = S->n_grid; return true;
      case GG_FIELD_PERM: v.ptr = G.perm; v.count = S->n_grid; return true;
      case GG_FIELD_CELL_START: v.ptr = G.cell_start; v.count = (int64_t)S->grid.C + 1; return true;
      case GG_FIELD_REMOVE: v.ptr = G.remove[c]; return true;
      case GG_FIELD_MERGE: v.ptr = G.merge[c]; return true;
      case GG_FIELD_MERGE_COUNT: v.ptr = G.merge_count[c]; return true;
      case GG_FIELD_MERGE_VELOCITY: v.ptr = G.merge_vel; v.elem = 12; v.stride = 16; return true;
      case GG_FIELD_ADAPTIVE_LAST_STEP: v.ptr = G.als[c]; return true;
      case GG_FIELD_CONTACTS: v.ptr = G.contacts; return true;
      case GG_FIELD_NUM_CONSTRAINTS: v.ptr = G.ncon; return true;
      case GG_FIELD_FEATURES:
        if (!S->feat) return false;
        v.ptr = S->feat; v.elem = 96; v.stride = 96; return true;
      case GG_FIELD_WARM_TARGET:
        if (!S->warm_target) return false;
        v.ptr = S->warm_target; v.elem = 12; v.stride = 12; return true;
      default: return false;
    }
  }
  if (set == GG_SET_BOUNDARY) {
    v.count = S->nb;
    switch (f) {
      case GG_FIELD_POS: v.ptr = S->b.pos; v.elem = 12; v.stride = 16; return true;
      case GG_FIELD_IS_ANIMATED: v.ptr = S->b.animated; return true;
      case GG_FIELD_CELL_KEY: v.ptr = S->b.keys; return true;
      case GG_FIELD_PERM: v.ptr = S->b.perm; return true;
      case GG_FIELD_CELL_START: v.ptr = S->b.cell_start; v.count = (int64_t)S->grid.C + 1; return true;
      default: return false;
    }
  }
  if (set == GG_SET_UPSAMPLED) {
    v.count = S->nu;
    switch (f) {
      case GG_FIELD_POS: v.ptr = S->u.pos[S->u.cur]; v.elem = 12; v.stride = 16; return true;
      case GG_FIELD_VEL: v.ptr = S->u.vel[S->u.cur]; v.elem = 12; v.stride = 16; return true;
      case GG_FIELD_CELL_KEY: v.ptr = S->u.keys; return true;
      case GG_FIELD_PERM: v.ptr = S->u.perm; return true;
      default: return false;
    }
  }
  return false;
}

// The device address of pinned (page-locked, mapped) host memory, or null
// for memory the device cannot address directly.
void* mapped_host(const void* host) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();  // unregistered memory on older runtimes
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// Device float4 fields cross to the host as packed float[3].  Pinned host
// buffers are written (read) by the packing kernel itself over the
// host-device link; other buffers go through the device staging buffer and
// one contiguous copy (a pitched copy with 12-byte rows runs far below the
// link's bandwidth).
cudaError_t copy_out(gg_system* S, const FieldView& v, void* dst, int64_t count, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  if (v.elem == v.stride)
    return cudaMemcpyAsync(dst, v.ptr, (size_t)v.elem * count, cudaMemcpyDeviceToHost, st);
  if (void* mapped = mapped_host(dst)) return pack3(S, (const float4*)v.ptr, (float*)mapped, count, st);
  cudaError_t e = pack3(S, (const float4*)v.ptr, S->stage, count, st);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(dst, S->stage, (size_t)12 * count, cudaMemcpyDeviceToHost, st);
}

cudaError_t copy_in(gg_system* S, const FieldView& v, const void* src, int64_t count, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  if (v.elem == v.stride)
    return cudaMemcpyAsync(v.ptr, src, (size_t)v.elem * count, cudaMemcpyHostToDevice, st);
  if (void* mapped = mapped_host(src)) return unpack3(S, (const float*)mapped, (float4*)v.ptr, count, st);
  cudaError_t e = cudaMemcpyAsync(S->stage, src, (size_t)12 * count, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  return unpack3(S, S->stage, (float4*)v.ptr, count, st);
}

}  // namespace

gg_status gg_get_params(gg_system* S, gg_params* out) {
  REQUIRE(S && out, "gg_get_params: null argument");
  *out = S->P;
  return GG_OK;
}

gg_status gg_set_params(gg_system* S, const gg_params* P) {
  REQUIRE(S && P, "gg_set_params: null argument");
  if (!(P->nlist_skin == S->P.nlist_skin || (std::isnan(P->nlist_skin) && std::isnan(S->P.nlist_skin)))) {
    set_error("gg_set_params: nlist_skin cannot change after gg_create");
    return GG_ERR_NOT_SUPPORTED;
  }
  REQUIRE(P->stab_iters >= 0 && P->iters >= 0 && P->max_sweeps >= 0, "gg_set_params: negative sweep count");
  REQUIRE(P->merge_cas_lag >= 0 && P->merge_cas_lag <= 65536, "gg_set_params: merge_cas_lag must be in 0..65536");
  REQUIRE((P->contact_law == 0 || P->contact_law == 1) && P->n_planes >= 0 && P->n_planes <= 8,
          "gg_set_params: contact_law must be 0 or 1 and n_planes in 0..8");
  S->P = *P;
  return GG_OK;
}

gg_status gg_read(gg_system* S, gg_set set, gg_field field, void* host_dst, int64_t capacity, int64_t* n) {
  GG_GUARD_BEGIN
  REQUIRE(S, "gg_read: null system");
  FieldView v;
  REQUIRE(field_view(S, set, field, v), "gg_read: field not available for this set");
  if (n) *n = v.count;
  if (!host_dst) return GG_OK;
  REQUIRE(capacity >= v.count, "gg_read: destination capacity too small");
  GG_CUDA(cudaSetDevice(S->device));
  GG_CUDA(copy_out(S, v, host_dst, v.count, S->stream));
  GG_CUDA(cudaStreamSynchronize(S->stream));
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_device_ptr(gg_system* S, gg_set set, gg_field field, void** dptr, int64_t* n, int32_t* stride_bytes) {
  REQUIRE(S && dptr, "gg_device_ptr: null argument");
  FieldView v;
  REQUIRE(field_view(S, set, field, v), "gg_device_ptr: field not available for this set");
  *dptr = v.ptr;
  if (n) *n = v.count;
  if (stride_bytes) *stride_bytes = v.stride;
  return GG_OK;
}

gg_status gg_write(gg_system* S, gg_set set, gg_field field, const void* host_src, int64_t n) {
  GG_GUARD_BEGIN
  REQUIRE(S && host_src, "gg_write: null argument");
  REQUIRE(field == GG_FIELD_POS || field == GG_FIELD_VEL, "gg_write: only positions and velocities are writable");
  FieldView v;
  REQUIRE(field_view(S, set, field, v), "gg_write: field not available for this set");
  REQUIRE(n == v.count, "gg_write: count must equal the set size");
  GG_CUDA(cudaSetDevice(S->device));
  GG_CUDA(copy_in(S, v, host_src, n, S->stream));
  GG_CUDA(cudaStreamSynchronize(S->stream));
  // positions of the boundary determine its grid
  if (set == GG_SET_BOUNDARY) return boundary_grid(S);
  return GG_OK;
  GG_GUARD_END
}

// ------------------------------------------------------------ snapshots

namespace {

const char kMagic[8] = {'G', 'G', 'S', 'N', 'A', 'P', '0', '1'};

struct SnapHeader {
  char magic[8];
  int32_t abi;
  int32_t merge_iter;
  int64_t n, cap, nb, nu;
  int32_t nx, ny, nz, pad;
  float L;
  float pad2;
  int64_t steps, merged_last, split_last, merged_total, split_total;
  int32_t error_word;
  int32_t ucur_pad;
  int64_t stats_rows;
  int64_t n_grid;
  gg_params P;
  Physics phys;
};

struct Blob {
  void* dptr;
  size_t bytes;
};

std::vector<Blob> snapshot_blobs(gg_system* S) {
  Granular& G = S->g;
  const int c = G.cur;
  const size_t n = (size_t)S->n, nb = (size_t)S->nb, nu = (size_t)S->nu, C1 = (size_t)S->grid.C + 1;
  return {{G.pos[c], 16 * n},       {G.vel[c], 16 * n},         {G.mass[c], 4 * n},
          {G.rs[c], 4 * n},         {G.units[c], 4 * n},        {G.merge[c], 4 * n},
          {G.merge_units[c], 4 * n}, {G.merge_count[c], 4 * n}, {G.remove[c], 4 * n},
          {G.als[c], 4 * n},        {G.merge_vel, 16 * n},      {G.surface, 4 * n},
          {G.sdist, 4 * n},         {G.keys, 4 * (size_t)S->n_grid}, {G.perm, 4 * (size_t)S->n_grid},
          {G.contacts, 4 * n},      {G.ncon, 4 * n},            {G.cell_start, 4 * C1},
          {S->b.pos, 16 * nb},      {S->b.animated, 4 * nb},    {S->b.keys, 4 * nb},
          {S->b.perm, 4 * nb},      {S->b.cell_start, 4 * C1},  {S->u.pos[S->u.cur], 16 * nu},
          {S->u.vel[S->u.cur], 16 * nu}, {S->u.keys, 4 * nu},   {S->u.perm, 4 * nu}};
}

}  // namespace

gg_status gg_save(gg_system* S, const char* path) {
  GG_GUARD_BEGIN
  REQUIRE(S && path, "gg_save: null argument");
  GG_CUDA(cudaSetDevice(S->device));
  GG_CUDA(cudaStreamSynchronize(S->stream));
  FILE* f = fopen(path, "wb");
  if (!f) {
    set_error(std::string("gg_save: cannot open ") + path);
    return GG_ERR_IO;
  }
  SnapHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, kMagic, 8);
  h.abi = GG_ABI_VERSION;
  h.merge_iter = S->merge_iter;
  h.n = S->n; h.cap = S->cap; h.nb = S->nb; h.nu = S->nu;
  h.nx = S->grid.nx; h.ny = S->grid.ny; h.nz = S->grid.nz; h.L = S->grid.L;
  h.steps = S->steps; h.merged_last = S->merged_last; h.split_last = S->split_last;
  h.merged_total = S->merged_total; h.split_total = S->split_total;
  h.error_word = S->error_word;
  h.stats_rows = (int64_t)S->stats_rows.size();
  h.n_grid = S->n_grid;
  h.P = S->P;
  h.phys = S->phys;
  bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
  if (ok && !S->stats_rows.empty())
    ok = fwrite(S->stats_rows.data(), sizeof(int64_t), S->stats_rows.size(), f) == S->stats_rows.size();
  std::vector<char> buf;
  for (const Blob& b : snapshot_blobs(S)) {
    if (!ok) break;
    buf.resize(b.bytes);
    if (b.bytes) {
      cudaError_t e = cudaMemcpy(buf.data(), b.dptr, b.bytes, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) {
        fclose(f);
        return cuda_status(e, "gg_save: device read");
      }
      ok = fwrite(buf.data(), 1, b.bytes, f) == b.bytes;
    }
  }
  if (fclose(f) != 0) ok = false;
  if (!ok) {
    set_error(std::string("gg_save: write failed for ") + path);
    return GG_ERR_IO;
  }
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_load(gg_system* S, const char* path) {
  GG_GUARD_BEGIN
  REQUIRE(S && path, "gg_load: null argument");
  FILE* f = fopen(path, "rb");
  if (!f) {
    set_error(std::string("gg_load: cannot open ") + path);
    return GG_ERR_IO;
  }
  SnapHeader h;
  if (fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, kMagic, 8) != 0 || h.abi != GG_ABI_VERSION) {
    fclose(f);
    set_error("gg_load: not a snapshot of this ABI version");
    return GG_ERR_PARSE;
  }
  if (h.nx != S->grid.nx || h.ny != S->grid.ny || h.nz != S->grid.nz || h.nb != S->nb || h.nu != S->nu ||
      h.n > S->cap || h.n < 0 || h.stats_rows < 0 || h.stats_rows > ((int64_t)1 << 32)) {
    fclose(f);
    set_error("gg_load: snapshot does not fit this system (grid, set sizes or capacity differ)");
    return GG_ERR_INVALID_ARGUMENT;
  }
  std::vector<int64_t> rows((size_t)h.stats_rows);
  if (h.stats_rows && fread(rows.data(), sizeof(int64_t), rows.size(), f) != rows.size()) {
    fclose(f);
    set_error("gg_load: truncated snapshot");
    return GG_ERR_PARSE;
  }
  GG_CUDA(cudaSetDevice(S->device));
  GG_CUDA(cudaStreamSynchronize(S->stream));
  const int64_t n_old = S->n, ng_old = S->n_grid;
  if (h.n_grid < 0 || h.n_grid > S->cap) {
    fclose(f);
    set_error("gg_load: corrupt snapshot");
    return GG_ERR_PARSE;
  }
  S->n = h.n;
  S->n_grid = h.n_grid;
  std::vector<char> buf;
  for (const Blob& b : snapshot_blobs(S)) {
    buf.resize(b.bytes);
    if (b.bytes && fread(buf.data(), 1, b.bytes, f) != b.bytes) {
      fclose(f);
      S->n = n_old;
      S->n_grid = ng_old;
      set_error("gg_load: truncated snapshot");
      return GG_ERR_PARSE;
    }
    if (b.bytes) {
      cudaError_t e = cudaMemcpy(b.dptr, buf.data(), b.bytes, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        fclose(f);
        return cuda_status(e, "gg_load: device write");
      }
    }
  }
  fclose(f);
  S->merge_iter = h.merge_iter;
  S->steps = h.steps;
  S->merged_last = h.merged_last;
  S->split_last = h.split_last;
  S->merged_total = h.merged_total;
  S->split_total = h.split_total;
  S->error_word = h.error_word;
  S->stats_rows = rows;
  S->P = h.P;
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_stats(gg_system* S, gg_stats_t* out) {
  GG_GUARD_BEGIN
  REQUIRE(S && out, "gg_stats: null argument");
  GG_CUDA(cudaSetDevice(S->device));
  return stats_compute(S, out);
  GG_GUARD_END
}

gg_status gg_save_particle_stats(gg_system* S, const char* path) {
  GG_GUARD_BEGIN
  REQUIRE(S && path, "gg_save_particle_stats: null argument");
  FILE* f = fopen(path, "w");
  if (!f) {
    set_error(std::string("gg_save_particle_stats: cannot open ") + path);
    return GG_ERR_IO;
  }
  fprintf(f, "Frame,MergedParticles,SplitParticles,TotalParticles\n");
  for (size_t i = 0; 3 * i + 2 < S->stats_rows.size(); ++i) {
    fprintf(f, "%zu,%lld,%lld,%lld\n", i, (long long)S->stats_rows[3 * i], (long long)S->stats_rows[3 * i + 1],
            (long long)S->stats_rows[3 * i + 2]);
  }
  fclose(f);
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_write_vtk(gg_system* S, gg_set set, const char* path, int32_t swap_yz) {
  GG_GUARD_BEGIN
  REQUIRE(S && path, "gg_write_vtk: null argument");
  FieldView v;
  REQUIRE(field_view(S, set, GG_FIELD_POS, v), "gg_write_vtk: unknown set");
  std::vector<float> p((size_t)std::max<int64_t>(v.count, 1) * 3);
  GG_CUDA(cudaSetDevice(S->device));
  GG_CUDA(copy_out(S, v, p.data(), v.count, S->stream));
  GG_CUDA(cudaStreamSynchronize(S->stream));
  std::vector<size_t> keep;
  keep.reserve((size_t)v.count);
  for (int64_t i = 0; i < v.count; ++i)
    if (!std::isnan(p[3 * i]) && !std::isnan(p[3 * i + 1]) && !std::isnan(p[3 * i + 2])) keep.push_back((size_t)i);
  std::ofstream out(path);
  if (!out.is_open()) {
    set_error(std::string("gg_write_vtk: cannot open ") + path);
    return GG_ERR_IO;
  }
  out << "# vtk DataFile Version 3.0\n";
  out << "Upsampled Granular Particles\n";
  out << "ASCII\n";
  out << "DATASET UNSTRUCTURED_GRID\n";
  out << "POINTS " << keep.size() << " float\n";
  for (size_t i : keep) {
    const float x = p[3 * i], y = p[3 * i + 1], z = p[3 * i + 2];
    if (swap_yz) out << x << " " << z << " " << y << "\n";
    else out << x << " " << y << " " << z << "\n";
  }
  out << "CELLS " << keep.size() << " " << keep.size() * 2 << "\n";
  for (size_t i = 0; i < keep.size(); ++i) out << "1 " << i << "\n";
  out << "CELL_TYPES " << keep.size() << "\n";
  for (size_t i = 0; i < keep.size(); ++i) out << "1\n";
  if (!out.good()) {
    set_error(std::string("gg_write_vtk: write failed for ") + path);
    return GG_ERR_IO;
  }
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_set_frame_timing(gg_system* S, int32_t enabled) {
  REQUIRE(S, "gg_set_frame_timing: null");
  S->frame_timing = enabled != 0;
  return GG_OK;
}

gg_status gg_frame_times(gg_system* S, float* dst, int64_t capacity, int64_t* n) {
  REQUIRE(S, "gg_frame_times: null");
  const int64_t cnt = (int64_t)S->frame_times.size();
  if (n) *n = cnt;
  if (dst) {
    REQUIRE(capacity >= cnt, "gg_frame_times: capacity too small");
    memcpy(dst, S->frame_times.data(), sizeof(float) * cnt);
  }
  return GG_OK;
}

gg_status gg_trigger_explosion(gg_system* S, float force) {
  GG_GUARD_BEGIN
  REQUIRE(S, "gg_trigger_explosion: null");
  GG_CUDA(cudaSetDevice(S->device));
  gg_status rc = explosion(S, force, S->stream);
  if (rc != GG_OK) return rc;
  GG_CUDA(cudaStreamSynchronize(S->stream));
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_profile_begin(gg_system* S) {
  REQUIRE(S, "gg_profile_begin: null");
  for (int k = 0; k < PC_COUNT; ++k) {
    S->prof_ms[k] = 0;
    S->prof_launches[k] = 0;
    S->prof_units[k] = 0;
  }
  S->prof_pending.clear();
  S->prof_pool_used = 0;
  S->prof_launch_base = S->launches;
  S->profiling = true;
  if (cudaMemsetAsync(&S->scal->nlist_rebuilds, 0, sizeof(S->scal->nlist_rebuilds), S->stream) != cudaSuccess) {
    set_error("gg_profile_begin: cannot reset the device counters");
    return GG_ERR_CUDA;
  }
  return GG_OK;
}

gg_status gg_profile_end(gg_system* S, gg_profile_t* out) {
  GG_GUARD_BEGIN
  REQUIRE(S && out, "gg_profile_end: null");
  prof_flush(S);
  S->profiling = false;
  memset(out, 0, sizeof(*out));
  out->n_classes = PC_COUNT;
  out->kernel_launches = S->launches - S->prof_launch_base;
  unsigned long long rebuilds = 0;
  if (cudaMemcpyAsync(&rebuilds, &S->scal->nlist_rebuilds, sizeof(rebuilds), cudaMemcpyDeviceToHost, S->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(S->stream) != cudaSuccess) {
    set_error("gg_profile_end: cannot read the device counters");
    return GG_ERR_CUDA;
  }
  out->nlist_rebuilds = (int64_t)rebuilds;
  for (int k = 0; k < PC_COUNT && k < GG_PROF_MAX; ++k) {
    strncpy(out->names[k], prof_name(k), 23);
    out->launches[k] = S->prof_launches[k];
    out->ms[k] = S->prof_ms[k];
    out->units[k] = S->prof_units[k];
  }
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_stream(gg_system* S, void** stream) {
  REQUIRE(S && stream, "gg_stream: null");
  *stream = (void*)S->stream;
  return GG_OK;
}

void gg_destroy(gg_system* S) {
  try {
    system_destroy(S);
  } catch (...) {
  }
}

// ------------------------------------------------------------ stand-alone grid

gg_status gg_grid_create(int32_t device, int64_t capacity, const int32_t cell_size[3], float cell_length,
                         gg_grid** out) {
  GG_GUARD_BEGIN
  REQUIRE(out && cell_size && capacity > 0 && cell_length > 0, "gg_grid_create: invalid argument");
  REQUIRE(cell_size[0] > 0 && cell_size[1] > 0 && cell_size[2] > 0, "gg_grid_create: cell_size must be positive");
  const int64_t C64 = (int64_t)cell_size[0] * cell_size[1] * cell_size[2];
  REQUIRE(C64 < ((int64_t)1 << 30) && capacity <= kMaxCount, "gg_grid_create: grid or capacity too large");
  GG_CUDA(cudaSetDevice(device));
  gg_grid* g = new gg_grid();
  g->device = device;
  g->grid.L = cell_length;
  g->grid.nx = cell_size[0];
  g->grid.ny = cell_size[1];
  g->grid.nz = cell_size[2];
  g->grid.C = (int)C64;
  g->cap = capacity;
  cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&g->pos, sizeof(float4) * capacity);
  if (e == cudaSuccess) e = cudaMalloc(&g->keys_unsorted, sizeof(uint32_t) * capacity);
  if (e == cudaSuccess) e = cudaMalloc(&g->cell_start, sizeof(int32_t) * (C64 + 1));
  if (e == cudaSuccess) e = cudaMalloc(&g->sorted_keys, sizeof(uint32_t) * capacity);
  if (e == cudaSuccess) e = cudaMalloc(&g->perm, sizeof(uint32_t) * capacity);
  gg_status rc = e == cudaSuccess ? sort_scratch_alloc(g->sort, capacity) : GG_ERR_OUT_OF_MEMORY;
  if (rc != GG_OK || e != cudaSuccess) {
    gg_grid_destroy(g);
    set_error("gg_grid_create: device allocation failed");
    return GG_ERR_OUT_OF_MEMORY;
  }
  *out = g;
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_grid_build(gg_grid* g, const float* pos, int64_t n, int32_t* keys, int32_t* sorted_keys, int32_t* perm,
                        int32_t* cell_start) {
  GG_GUARD_BEGIN
  REQUIRE(g && (pos || n == 0) && n >= 0 && n <= g->cap, "gg_grid_build: invalid argument");
  GG_CUDA(cudaSetDevice(g->device));
  cudaStream_t st = g->stream;
  if (n > 0) {
    GG_CUDA(cudaMemsetAsync(g->pos, 0, sizeof(float4) * n, st));
    GG_CUDA(cudaMemcpy2DAsync(g->pos, sizeof(float4), pos, 12, 12, (size_t)n, cudaMemcpyHostToDevice, st));
  }
  uint32_t* sk = g->sorted_keys;
  uint32_t* pm = g->perm;
  gg_status rc = grid_sort(g->grid, g->pos, n, g->sort, sk, pm, g->keys_unsorted, st, nullptr);
  if (rc == GG_OK) rc = cell_start_build(g->grid, sk, n, g->cell_start, g->sort, st, nullptr);
  if (rc == GG_OK && n > 0) {
    if (keys) GG_CUDA(cudaMemcpyAsync(keys, g->keys_unsorted, 4 * n, cudaMemcpyDeviceToHost, st));
    if (sorted_keys) GG_CUDA(cudaMemcpyAsync(sorted_keys, sk, 4 * n, cudaMemcpyDeviceToHost, st));
    if (perm) GG_CUDA(cudaMemcpyAsync(perm, pm, 4 * n, cudaMemcpyDeviceToHost, st));
  }
  if (rc == GG_OK && cell_start)
    GG_CUDA(cudaMemcpyAsync(cell_start, g->cell_start, 4 * ((int64_t)g->grid.C + 1), cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  return rc;
  GG_GUARD_END
}

void gg_grid_destroy(gg_grid* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  cudaFree(g->pos);
  cudaFree(g->keys_unsorted);
  cudaFree(g->cell_start);
  cudaFree(g->sorted_keys);
  cudaFree(g->perm);
  sort_scratch_free(g->sort);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

}  // extern "C"

// ------------------------------------------------------------ autotuning

gg_status gg_autotune(gg_system* S, int32_t substeps, gg_tuning* out) {
  GG_GUARD_BEGIN
  REQUIRE(S && substeps > 0, "gg_autotune: bad argument");
  REQUIRE(!S->graph_exec, "gg_autotune: tune before capturing a graph (the graph keeps its launch shapes)");
  REQUIRE(!(S->P.target_residual > 0.0f), "gg_autotune: not in residual mode (the sweep count varies)");
  GG_CUDA(cudaSetDevice(S->device));
  cudaStream_t st = S->stream;
  GG_CUDA(cudaStreamSynchronize(st));
  // device copy of the state; every trial starts from it
  const std::vector<Blob> blobs = snapshot_blobs(S);
  size_t total = 0;
  for (const Blob& b : blobs) total += (b.bytes + 255) & ~(size_t)255;
  char* backup = nullptr;
  GG_CUDA(cudaMalloc((void**)&backup, std::max<size_t>(total, 1)));
  auto copy_all = [&](bool save) -> cudaError_t {
    size_t off = 0;
    for (const Blob& b : blobs) {
      cudaError_t e = b.bytes ? cudaMemcpyAsync(save ? backup + off : b.dptr, save ? b.dptr : backup + off, b.bytes,
                                                cudaMemcpyDeviceToDevice, st)
                              : cudaSuccess;
      if (e != cudaSuccess) return e;
      off += (b.bytes + 255) & ~(size_t)255;
    }
    return cudaStreamSynchronize(st);
  };
  const int cur0 = S->g.cur, ucur0 = S->u.cur;
  const int64_t steps0 = S->steps, launches0 = S->launches, n_grid0 = S->n_grid;
  // merge/split moves the particle count and the host-side counters
  const int64_t n0 = S->n, merged_last0 = S->merged_last, split_last0 = S->split_last;
  const int64_t merged_total0 = S->merged_total, split_total0 = S->split_total;
  const int merge_iter0 = S->merge_iter;
  const int32_t error_word0 = S->error_word;
  const size_t stats_rows0 = S->stats_rows.size();
  auto restore_counters = [&]() {
    S->g.cur = cur0;
    S->u.cur = ucur0;
    S->n_grid = n_grid0;
    S->n = n0;
    S->merged_last = merged_last0;
    S->split_last = split_last0;
    S->merged_total = merged_total0;
    S->split_total = split_total0;
    S->merge_iter = merge_iter0;
    S->error_word = error_word0;
    S->stats_rows.resize(stats_rows0);
  };
  const bool timing0 = S->frame_timing;
  S->frame_timing = false;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t ce = copy_all(true);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  gg_status rc = ce == cudaSuccess ? GG_OK : cuda_status(ce, "gg_autotune: state copy");
  int trials = 0;
  // device ms of `substeps` substeps after one warm-up substep, from the saved state
  auto trial = [&](float* ms) -> gg_status {
    restore_counters();
    cudaError_t e = copy_all(false);
    if (e != cudaSuccess) return cuda_status(e, "gg_autotune: restore");
    gg_status r = step_once(S);
    if (r != GG_OK) return r;
    GG_CUDA(cudaEventRecord(e0, st));
    for (int k = 0; k < substeps && r == GG_OK; ++k) r = step_once(S);
    if (r != GG_OK) return r;
    GG_CUDA(cudaEventRecord(e1, st));
    GG_CUDA(cudaEventSynchronize(e1));
    GG_CUDA(cudaEventElapsedTime(ms, e0, e1));
    ++trials;
    return GG_OK;
  };
  float base = 0.0f, best = 0.0f;
  if (rc == GG_OK) rc = trial(&base);
  best = base;
  struct Site {
    int* field;
    std::vector<int> cands;
  };
  Tuning& T = S->tune;
  std::vector<Site> sites = {{&T.sweep_variant, {0, 1}},
                             {&T.keep_threads, {128, 256}},
                             {&T.build_blocks_per_sm, {4, 8, 16, 32}},
                             {&T.apply_threads, {128, 256}},
                             {&T.predict_threads, {128, 256}},
                             {&T.finalize_threads, {64, 128, 256}}};
  for (Site& site : sites) {
    if (rc != GG_OK) break;
    const int keep = *site.field;
    int choice = keep;
    for (int c : site.cands) {
      if (c == keep) continue;
      *site.field = c;
      float ms = 0.0f;
      rc = trial(&ms);
      if (rc != GG_OK) break;
      if (ms < best) {
        best = ms;
        choice = c;
      }
    }
    *site.field = choice;
  }
  // leave the system as it was, with the chosen shapes
  restore_counters();
  cudaError_t re = copy_all(false);
  S->steps = steps0;
  S->launches = launches0;
  S->frame_timing = timing0;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(backup);
  if (rc != GG_OK) return rc;
  GG_CUDA(re);
  if (out) {
    out->predict_threads = T.predict_threads;
    out->apply_threads = T.apply_threads;
    out->finalize_threads = T.finalize_threads;
    out->keep_threads = T.keep_threads;
    out->build_blocks_per_sm = T.build_blocks_per_sm;
    out->sweep_variant = T.sweep_variant;
    out->pad_ = 0;
    out->trials = trials;
    out->ms_default = base;
    out->ms_tuned = best;
  }
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_get_tuning(gg_system* S, gg_tuning* out) {
  GG_GUARD_BEGIN
  REQUIRE(S && out, "gg_get_tuning: null argument");
  const Tuning& T = S->tune;
  std::memset(out, 0, sizeof(*out));
  out->predict_threads = T.predict_threads;
  out->apply_threads = T.apply_threads;
  out->finalize_threads = T.finalize_threads;
  out->keep_threads = T.keep_threads;
  out->build_blocks_per_sm = T.build_blocks_per_sm;
  out->sweep_variant = T.sweep_variant;
  return GG_OK;
  GG_GUARD_END
}

gg_status gg_set_tuning(gg_system* S, const gg_tuning* t) {
  GG_GUARD_BEGIN
  REQUIRE(S && t, "gg_set_tuning: null argument");
  REQUIRE(!S->graph_exec, "gg_set_tuning: set launch shapes before capturing a graph");
  auto threads_ok = [](int v) { return v >= 32 && v <= 1024 && v % 32 == 0; };
  REQUIRE(threads_ok(t->predict_threads) && threads_ok(t->apply_threads) && threads_ok(t->finalize_threads) &&
              threads_ok(t->keep_threads),
          "gg_set_tuning: threads per block must be a multiple of 32 in 32..1024");
  REQUIRE(t->keep_threads <= 256, "gg_set_tuning: keep_threads must be at most 256 (the keep sweep's launch bound)");
  REQUIRE(t->build_blocks_per_sm >= 1 && t->build_blocks_per_sm <= 32,
          "gg_set_tuning: build_blocks_per_sm must be in 1..32");
  REQUIRE(t->sweep_variant == 0 || t->sweep_variant == 1, "gg_set_tuning: sweep_variant must be 0 or 1");
  Tuning& T = S->tune;
  T.predict_threads = t->predict_threads;
  T.apply_threads = t->apply_threads;
  T.finalize_threads = t->finalize_threads;
  T.keep_threads = t->keep_threads;
  T.build_blocks_per_sm = t->build_blocks_per_sm;
  T.sweep_variant = t->sweep_variant;
  return GG_OK;
  GG_GUARD_END
}

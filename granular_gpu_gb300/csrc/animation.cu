// animation.cu — the animated walls: AnimationState, updateAnimation and
// animateParticles (main.cu:100-111, 1175-1277).
//
// The state machine runs on the host in float arithmetic, operation for
// operation as the reference writes it (host code is compiled without
// contraction); the move itself is one kernel over the wall particles.
// The reference reads the wall positions back for the rotation centre when
// the translation ends, and so does gg_update_animation: the centroid is
// taken over the index range the scene construction recorded, in the
// walls' current (cell-sorted) order, as the reference takes it.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "scene.h"

namespace gg {

// animateParticles, main.cu:1175-1208.  angle_rad is rotation * M_PI /
// 180.0f as the reference evaluates it (in double, rounded to float).
template <int MM>
__global__ void k_animate(int n, float4* __restrict__ pos, const int32_t* __restrict__ animated, float3 t,
                          int rotate, float angle_rad, float3 c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || animated[i] != 1) return;
  float4 p = pos[i];
  p.x = p.x + t.x;
  p.y = p.y + t.y;
  p.z = p.z + t.z;
  if (rotate) {
    p.x = p.x - c.x;
    p.y = p.y - c.y;
    const float ct = MM ? (float)cos((double)angle_rad) : cosf(angle_rad);
    const float st = MM ? (float)sin((double)angle_rad) : sinf(angle_rad);
    const float nx = p.x * ct - p.y * st;
    const float ny = p.x * st + p.y * ct;
    p.x = nx + c.x;
    p.y = ny + c.y;
  }
  pos[i] = p;
}

gg_status animate_walls(gg_system* S, const gg_animation_move& m, cudaStream_t st) {
  if (S->nb <= 0) return GG_OK;
  const float3 t = make_float3(m.translation[0], m.translation[1], m.translation[2]);
  const float3 c = make_float3(m.center[0], m.center[1], m.center[2]);
  const float angle = (float)((double)m.rotation * M_PI / 180.0);
  auto kern = S->P.math_mode ? k_animate<1> : k_animate<0>;
  kern<<<blocks_for(S->nb, 256), 256, 0, st>>>((int)S->nb, S->b.pos, S->b.animated, t, m.rotation != 0.0f ? 1 : 0,
                                               angle, c);
  count_launches(S, 1);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

void default_animation(gg_animation* a) {
  memset(a, 0, sizeof(*a));
  a->translation_direction[0] = -0.1f;
  a->translation_speed = 5.0f;
  a->rotation_speed = 90.0f;
}

static bool ends_translation(const gg_animation* a, float dt) {
  if (!a->is_animating || a->translation_complete) return false;
  const float t = a->animation_time + dt;
  return !(t <= 2.5f);
}

// updateAnimation's decisions, main.cu:1210-1262.
static gg_status advance(gg_animation* a, float dt, const float* walls, int64_t nw, gg_animation_move* out) {
  memset(out, 0, sizeof(*out));
  if (!a->is_animating) return GG_OK;
  if (ends_translation(a, dt)) {
    const int64_t s = a->start_index, k = a->num_particles;
    if (!walls || s < 0 || k < 0 || s + k > nw) {
      set_error("gg_animation_advance: the animated range needs the wall positions it lies in");
      return GG_ERR_INVALID_ARGUMENT;
    }
  }
  a->animation_time += dt;
  float tr[3] = {0.0f, 0.0f, 0.0f};
  float rotation = 0.0f;
  if (a->animation_time <= 2.5f && !a->translation_complete) {
    for (int d = 0; d < 3; ++d) tr[d] = a->translation_direction[d] * a->translation_speed * dt;
  } else if (!a->translation_complete) {
    a->translation_complete = 1;
    a->animation_time = 0.0f;
    float cen[3] = {0.0f, 0.0f, 0.0f};
    int count = 0;
    for (int64_t i = a->start_index; i < (int64_t)a->start_index + a->num_particles; ++i) {
      for (int d = 0; d < 3; ++d) cen[d] = cen[d] + walls[3 * i + d];
      ++count;
    }
    if (count > 0)
      for (int d = 0; d < 3; ++d) a->rotation_center[d] = cen[d] / (float)count;
  }
  if (a->translation_complete && a->rotation_angle < 45.0f) {
    const float delta = -a->rotation_speed * dt;
    a->rotation_angle += std::fabs(delta);
    rotation = delta;
    if (a->rotation_angle >= 45.0f) a->is_animating = 0;
  }
  for (int d = 0; d < 3; ++d) {
    out->translation[d] = tr[d];
    out->center[d] = a->rotation_center[d];
  }
  out->rotation = rotation;
  out->apply = a->is_animating ? 1 : 0;
  return GG_OK;
}

}  // namespace gg

using namespace gg;

#define ANIM_GUARD_BEGIN try {
#define ANIM_GUARD_END                                         \
  }                                                            \
  catch (const std::exception& ex) {                           \
    set_error(std::string("internal error: ") + ex.what());    \
    return GG_ERR_INVALID_ARGUMENT;                            \
  }

extern "C" {

gg_status gg_default_animation(gg_animation* out) {
  if (!out) {
    set_error("gg_default_animation: null");
    return GG_ERR_INVALID_ARGUMENT;
  }
  default_animation(out);
  return GG_OK;
}

gg_status gg_scene_animation(const char* json_path, const char* base_dir, gg_animation* out) {
  ANIM_GUARD_BEGIN
  if (!json_path || !out) {
    set_error("gg_scene_animation: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  SceneData sc;
  gg_status rc = scene_build(json_path, base_dir, sc);
  if (rc != GG_OK) return rc;
  *out = sc.animation;
  return GG_OK;
  ANIM_GUARD_END
}

int32_t gg_animation_needs_centroid(const gg_animation* a, float dt) { return a && ends_translation(a, dt) ? 1 : 0; }

gg_status gg_animation_advance(gg_animation* a, float dt, const float* walls, int64_t n_walls,
                               gg_animation_move* out) {
  if (!a || !out) {
    set_error("gg_animation_advance: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  return advance(a, dt, walls, n_walls, out);
}

gg_status gg_animate_walls(gg_system* S, const gg_animation_move* m) {
  ANIM_GUARD_BEGIN
  if (!S || !m) {
    set_error("gg_animate_walls: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(S->device));
  return animate_walls(S, *m, S->stream);
  ANIM_GUARD_END
}

gg_status gg_update_animation(gg_system* S, gg_animation* a, float dt) {
  ANIM_GUARD_BEGIN
  if (!S || !a) {
    set_error("gg_update_animation: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(S->device));
  std::vector<float> walls;
  if (ends_translation(a, dt)) {
    // the readback of main.cu:1231-1233, in the walls' current order
    int64_t n = 0;
    walls.resize(3 * (size_t)S->nb + 3);
    gg_status rc = gg_read(S, GG_SET_BOUNDARY, GG_FIELD_POS, walls.data(), S->nb, &n);
    if (rc != GG_OK) return rc;
  }
  gg_animation_move m;
  gg_status rc = advance(a, dt, walls.empty() ? nullptr : walls.data(), S->nb, &m);
  if (rc != GG_OK) return rc;
  if (!m.apply) return GG_OK;
  return animate_walls(S, m, S->stream);
  ANIM_GUARD_END
}

}  // extern "C"

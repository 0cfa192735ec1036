// granular_system.hpp — header-only C++ class with the reference's
// GranularSystem shape, built only on the C ABI in gg.h.
//
// Source-level drop-in for callers written against src/GranularSystem.hpp,
// src/GranularParticles.hpp and src/Solver.hpp (main.cu's
// init_granular_system / one_step):
//
//   auto particles = std::make_shared<GranularParticles>(pos);
//   auto boundary  = std::make_shared<GranularParticles>(walls);
//   auto upsampled = std::make_shared<GranularParticles>(points);
//   GranularSystem sys(particles, boundary, upsampled, space_size, cell_length,
//                      dt, G, cell_size, density, 0.005f, false, 1);
//   sys.step();
//   std::vector<float3> x = sys.get_particles()->get_pos();
//
// As in the reference, the constructor moves from the caller's shared_ptr
// arguments (they are null afterwards, GranularSystem.cu:38-40) and runs one
// step (GranularSystem.cu:62).  Failures throw std::runtime_error carrying
// gg_last_error(), like DArray's checks (DArray.hpp:18-44).
#pragma once

#include <cuda_runtime.h>  // float3, int3

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gg.h"

namespace gg_shim {

inline void check(gg_status s) {
  if (s != GG_OK) throw std::runtime_error(std::string("granular: ") + gg_last_error());
}

}  // namespace gg_shim

// Host-side particle set handed to the constructor
// (GranularParticles(const std::vector<float3>&), GranularParticles.hpp:7-14).
class GranularParticles {
 public:
  explicit GranularParticles(const std::vector<float3>& p) : pos_(p), is_animated_(p.size(), 0) {}
  unsigned int size() const { return (unsigned int)pos_.size(); }
  // main.cu:973-975 copies animation markers in after construction
  void set_is_animated(const std::vector<int>& flags) { is_animated_ = flags; }
  const std::vector<float3>& host_pos() const { return pos_; }
  const std::vector<int>& host_is_animated() const { return is_animated_; }

 private:
  std::vector<float3> pos_;
  std::vector<int> is_animated_;
};

// Read access to one particle set of a live system: the get_*_ptr() device
// pointers (Particles.hpp:19-20, GranularParticles.hpp:19-26) and host copies.
class ParticleSetView {
 public:
  ParticleSetView(gg_system* s, gg_set set) : s_(s), set_(set) {}
  unsigned int size() const {
    int64_t n = 0;
    gg_shim::check(gg_size(s_, set_, &n));
    return (unsigned int)n;
  }
  std::vector<float3> get_pos() const { return read3(GG_FIELD_POS); }
  std::vector<float3> get_vel() const { return read3(GG_FIELD_VEL); }
  std::vector<float> get_mass() const { return read<float>(GG_FIELD_MASS); }
  std::vector<int> get_surface() const { return read<int>(GG_FIELD_SURFACE); }
  std::vector<float> get_surface_distance() const { return read<float>(GG_FIELD_SURFACE_DISTANCE); }
  std::vector<int> get_adaptive_last_step() const { return read<int>(GG_FIELD_ADAPTIVE_LAST_STEP); }
  // Device pointers.  Positions and velocities are float4 on the device
  // (w = radius for positions): a 16-byte stride where the reference has 12.
  float4* get_pos_ptr() const { return (float4*)dptr(GG_FIELD_POS); }
  float4* get_vel_ptr() const { return (float4*)dptr(GG_FIELD_VEL); }
  // Mass, surface and distance exist for the particles only: the render
  // points' (zero-filled and never written in the reference) read as null.
  float* get_mass_ptr() const { return (float*)dptr_or_null(GG_FIELD_MASS); }
  int* get_surface_ptr() const { return (int*)dptr_or_null(GG_FIELD_SURFACE); }
  float* get_surface_distance_ptr() const { return (float*)dptr_or_null(GG_FIELD_SURFACE_DISTANCE); }
  int* get_particle_2_cell() const { return (int*)dptr(GG_FIELD_CELL_KEY); }
  gg_system* system() const { return s_; }
  gg_set set() const { return set_; }

 private:
  std::vector<float3> read3(gg_field f) const {
    int64_t n = 0;
    gg_shim::check(gg_read(s_, set_, f, nullptr, 0, &n));
    std::vector<float3> out((size_t)n);
    gg_shim::check(gg_read(s_, set_, f, out.data(), n, &n));
    return out;
  }
  template <typename T>
  std::vector<T> read(gg_field f) const {
    int64_t n = 0;
    gg_shim::check(gg_read(s_, set_, f, nullptr, 0, &n));
    std::vector<T> out((size_t)n);
    gg_shim::check(gg_read(s_, set_, f, out.data(), n, &n));
    return out;
  }
  void* dptr(gg_field f) const {
    void* p = nullptr;
    int64_t n = 0;
    int32_t stride = 0;
    gg_shim::check(gg_device_ptr(s_, set_, f, &p, &n, &stride));
    return p;
  }
  void* dptr_or_null(gg_field f) const {
    void* p = nullptr;
    int64_t n = 0;
    int32_t stride = 0;
    return gg_device_ptr(s_, set_, f, &p, &n, &stride) == GG_OK ? p : nullptr;
  }
  gg_system* s_;
  gg_set set_;
};

// GranularSystem::get_solver() (GranularSystem.hpp:56).
class GranularSolver {
 public:
  explicit GranularSolver(gg_system* s) : s_(s) {}
  void save_particle_stats(const std::string& filename) {  // Solver.cu:1444-1462
    gg_shim::check(gg_save_particle_stats(s_, filename.c_str()));
  }
  void trigger_explosion(float explosion_force) {  // Solver.cu:1411-1442
    gg_shim::check(gg_trigger_explosion(s_, explosion_force));
  }

 private:
  gg_system* s_;
};

class GranularSystem {
 public:
  // GranularSystem.hpp:8-14.  `params` defaults to the reference's constants.
  GranularSystem(std::shared_ptr<GranularParticles>& granular_particles,
                 std::shared_ptr<GranularParticles>& boundary_particles,
                 std::shared_ptr<GranularParticles>& upsampled_particles, float3 space_size,
                 float cell_length, float dt, float3 g, int3 cell_size, const float density,
                 const float upsampled_radius, const bool is_move_boundary, const int is_adaptive,
                 const gg_params* params = nullptr, int device = 0)
      : solver_(nullptr) {
    std::shared_ptr<GranularParticles> p = std::move(granular_particles);
    std::shared_ptr<GranularParticles> b = std::move(boundary_particles);
    std::shared_ptr<GranularParticles> u = std::move(upsampled_particles);
    gg_desc d{};
    d.particles = p && p->size() ? &p->host_pos()[0].x : nullptr;
    d.n_particles = p ? p->size() : 0;
    d.boundary = b && b->size() ? &b->host_pos()[0].x : nullptr;
    d.n_boundary = b ? b->size() : 0;
    d.boundary_animated = b && b->size() ? b->host_is_animated().data() : nullptr;
    d.upsampled = u && u->size() ? &u->host_pos()[0].x : nullptr;
    d.n_upsampled = u ? u->size() : 0;
    d.space_size[0] = space_size.x;
    d.space_size[1] = space_size.y;
    d.space_size[2] = space_size.z;
    d.cell_length = cell_length;
    d.dt = dt;
    d.gravity[0] = g.x;
    d.gravity[1] = g.y;
    d.gravity[2] = g.z;
    d.cell_size[0] = cell_size.x;
    d.cell_size[1] = cell_size.y;
    d.cell_size[2] = cell_size.z;
    d.density = density;
    d.upsampled_radius = upsampled_radius;
    d.is_move_boundary = is_move_boundary ? 1 : 0;
    d.is_adaptive = is_adaptive;
    d.device = device;
    if (params) d.params = *params;
    else gg_shim::check(gg_default_params(&d.params));
    gg_shim::check(gg_create(&d, &s_));
    solver_ = GranularSolver(s_);
    gg_shim::check(gg_set_frame_timing(s_, 1));
  }

  // loadSceneConfig + init_granular_system (main.cu:123-167, 746-1173).
  explicit GranularSystem(const std::string& scene_json, const gg_overrides* ov = nullptr) : solver_(nullptr) {
    gg_shim::check(gg_create_from_scene(scene_json.c_str(), ov, &s_));
    solver_ = GranularSolver(s_);
    gg_shim::check(gg_set_frame_timing(s_, 1));
  }

  GranularSystem(const GranularSystem&) = delete;
  GranularSystem& operator=(const GranularSystem&) = delete;
  ~GranularSystem() { gg_destroy(s_); }

  // GranularSystem.cu:397-453: one step, synchronous, returns 1.
  float step() {
    gg_shim::check(gg_step(s_, 1));
    gg_shim::check(gg_synchronize(s_));
    return 1;
  }

  int size() const { return count(GG_SET_GRANULAR); }
  int upsampled_size() const { return count(GG_SET_UPSAMPLED); }
  int boundary_size() const { return count(GG_SET_BOUNDARY); }
  int total_size() const { return size() + boundary_size() + upsampled_size(); }

  std::shared_ptr<ParticleSetView> get_particles() const {
    return std::make_shared<ParticleSetView>(s_, GG_SET_GRANULAR);
  }
  std::shared_ptr<ParticleSetView> get_boundaries() const {
    return std::make_shared<ParticleSetView>(s_, GG_SET_BOUNDARY);
  }
  std::shared_ptr<ParticleSetView> get_upsampled() const {
    return std::make_shared<ParticleSetView>(s_, GG_SET_UPSAMPLED);
  }

  const std::vector<float>& get_frame_times() {
    int64_t n = 0;
    gg_shim::check(gg_frame_times(s_, nullptr, 0, &n));
    frame_times_.resize((size_t)n);
    gg_shim::check(gg_frame_times(s_, frame_times_.data(), n, &n));
    return frame_times_;
  }

  GranularSolver& get_solver() { return solver_; }
  gg_system* handle() const { return s_; }
  // GranularSystem.hpp:44-45: the merge limits the colouring uses.
  float get_max_mass() const { return params().max_mass; }
  float get_min_mass() const { return params().min_merge_mass; }
  gg_params params() const {
    gg_params p;
    gg_shim::check(gg_get_params(s_, &p));
    return p;
  }

 private:
  int count(gg_set set) const {
    int64_t n = 0;
    gg_shim::check(gg_size(s_, set, &n));
    return (int)n;
  }
  gg_system* s_ = nullptr;
  GranularSolver solver_;
  std::vector<float> frame_times_;
};

// updateAnimation (main.cu:1210-1277) with the animation state passed in
// instead of main.cu's global AnimationState; call it once per frame before
// the frame's steps.  The state of a scene comes from gg_scene_animation.
inline void updateAnimation(GranularSystem& sys, gg_animation& state, float dt) {
  gg_shim::check(gg_update_animation(sys.handle(), &state, dt));
}

// generate_dots (VBO.hpp:96-106) over device buffers instead of mapped
// OpenGL buffer objects: positions and colours of the set as float3, the
// colour chosen by show_surface (0 surface flag, 1 surface distance, 2 mass
// between min_mass and max_mass).  The set's own surface array is used, as
// the reference's callers pass it; `surface` is accepted for the signature.
// Synchronous, as the reference.
inline void generate_dots(float3* dot, float3* color, const std::shared_ptr<ParticleSetView>& particles,
                          int* surface, const float max_mass, const float min_mass, int show_surface) {
  (void)surface;
  gg_shim::check(gg_color_buffer(particles->system(), particles->set(), show_surface, min_mass, max_mass,
                                 reinterpret_cast<float*>(dot), reinterpret_cast<float*>(color)));
  gg_shim::check(gg_synchronize(particles->system()));
}


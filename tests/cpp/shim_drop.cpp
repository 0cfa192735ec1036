// A main.cu-style caller of the C++ shim: builds a small box drop the way
// init_granular_system does (lattice + walls + 25 jittered render points per
// particle), steps it and prints counts and the centre of mass per step.
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <random>
#include <vector>

#include "granular_system.hpp"

int main(int argc, char** argv) {
  const int steps = argc > 1 ? atoi(argv[1]) : 5;
  std::vector<float3> pos;
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j)
      for (int k = 0; k < 10; ++k) pos.push_back(make_float3(0.3f + 0.021f * j, 0.2f + 0.021f * i, 0.3f + 0.021f * k));
  std::vector<float3> up;
  std::default_random_engine gen;
  std::uniform_real_distribution<float> dist(-0.01f, 0.01f);
  for (const auto& p : pos)
    for (int n = 0; n < 25; ++n) {
      const float oz = dist(gen), oy = dist(gen), ox = dist(gen);
      up.push_back(make_float3(p.x + ox, p.y + oy, p.z + oz));
    }
  const float L = 0.0404f;
  const int cs = 25;
  std::vector<float3> walls;
  const int c = 2 * cs;
  for (int a = 0; a < c; ++a)
    for (int b = 0; b < c; ++b) {
      const float s = 1.0f / (c - 1);
      walls.push_back(make_float3(0.99f * a * s + 0.005f, 0.005f, 0.99f * b * s + 0.005f));
    }
  auto particles = std::make_shared<GranularParticles>(pos);
  auto boundary = std::make_shared<GranularParticles>(walls);
  auto upsampled = std::make_shared<GranularParticles>(up);
  GranularSystem sys(particles, boundary, upsampled, make_float3(1, 1, 1), L, 0.002f, make_float3(0, -9.8f, 0),
                     make_int3(cs, cs, cs), 238732.4146f, 0.005f, false, 1);
  if (particles) {
    fprintf(stderr, "constructor did not move from its arguments\n");
    return 2;
  }
  for (int s = 0; s < steps; ++s) {
    sys.step();
    std::vector<float3> x = sys.get_particles()->get_pos();
    double cy = 0;
    for (const auto& p : x) cy += p.y;
    printf("step %d n=%d up=%d walls=%d com_y=%.6f\n", s, sys.size(), sys.upsampled_size(), sys.boundary_size(),
           cy / x.size());
  }
  // renderUpsampledParticles / renderParticles (main.cu:1539-1580) into device buffers
  float3 *dd = nullptr, *dc = nullptr;
  const size_t nu = (size_t)sys.upsampled_size(), n = (size_t)sys.size();
  if (cudaMalloc(&dd, sizeof(float3) * nu) != cudaSuccess || cudaMalloc(&dc, sizeof(float3) * nu) != cudaSuccess) {
    fprintf(stderr, "cudaMalloc failed\n");
    return 3;
  }
  generate_dots(dd, dc, sys.get_upsampled(), sys.get_upsampled()->get_surface_ptr(), sys.get_max_mass(),
                sys.get_min_mass(), 2);
  std::vector<float3> cu(nu);
  cudaMemcpy(cu.data(), dc, sizeof(float3) * nu, cudaMemcpyDeviceToHost);
  generate_dots(dd, dc, sys.get_particles(), sys.get_particles()->get_surface_ptr(), sys.get_max_mass(),
                sys.get_min_mass(), 2);
  std::vector<float3> cp(n);
  cudaMemcpy(cp.data(), dc, sizeof(float3) * n, cudaMemcpyDeviceToHost);
  cudaFree(dd);
  cudaFree(dc);
  // render points have no mass (the reference's 6.0 / 255 / 0 colour); unit masses are blue
  printf("dots up_inf=%d p0=(%.3f,%.3f,%.3f)\n", (int)(cu[0].x > 1e30f), cp[0].x, cp[0].y, cp[0].z);
  sys.get_solver().save_particle_stats("/tmp/gg_shim_stats.csv");
  printf("frames=%zu\n", sys.get_frame_times().size());
  return 0;
}

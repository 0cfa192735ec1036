// kernels_view.cu — the headless colour buffer.
//
// Replaces generate_dots / generate_dots_CUDA (VBO.hpp:9-71, called from
// main.cu:1539-1580 on the particles and on the render points), which write
// positions and colours into OpenGL vertex buffers mapped into CUDA.  Here
// the same packed float[3] positions and colours go into device buffers the
// caller owns (a renderer's interop buffers, or plain device memory to read
// back); no graphics API is involved.
#include "common.cuh"

namespace gg {

// generate_dots_CUDA, VBO.hpp:9-71, colour by mode:
//   0: surface particles (surface == 1) blue-grey, others black;
//   1: surface distance 0 blue-grey, >= 100 black, between red;
//   2: mass interpolated from blue (min_mass) to red (max_mass), in the
//      reference's operation order; mass exactly 0 gets the reference's
//      (6.0 / 255 / 0, 214 / 255, 160 / 255), whose first component is +inf.
// Sets whose mass, surface or distance arrays the reference never writes
// (render points) pass null and read 0, as its zero-filled arrays do.
__global__ void k_color_dots(int n, const float4* __restrict__ pos, const float* __restrict__ mass,
                             const int32_t* __restrict__ surface, const float* __restrict__ sdist, int mode,
                             float min_mass, float max_mass, float* __restrict__ dots, float* __restrict__ colors) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos[i];
  dots[3 * i] = p.x;
  dots[3 * i + 1] = p.y;
  dots[3 * i + 2] = p.z;
  const float m = mass ? mass[i] : 0.0f;
  const int sf = surface ? surface[i] : 0;
  const float sd = sdist ? sdist[i] : 0.0f;
  float3 c = make_float3(0.0f, 0.0f, 0.0f);  // modes other than 0-2 leave it unwritten there: black here
  if (mode == 0) {
    c = sf == 1 ? make_float3(0.34f, 0.46f, 0.7f) : make_float3(0.0f, 0.0f, 0.0f);
  } else if (mode == 1) {
    if (sd == 0.0f) c = make_float3(0.34f, 0.46f, 0.7f);
    else if (sd >= 100.0f) c = make_float3(0.0f, 0.0f, 0.0f);
    else c = make_float3(1.0f, 0.0f, 0.0f);
  } else if (mode == 2) {
    const float t = (m - min_mass) / (max_mass - min_mass);
    // (1 - t) * blue + t * red, component by component
    const float3 lo = smul3(1.0f - t, make_float3(0.0f, 0.0f, 1.0f));
    const float3 hi = smul3(t, make_float3(1.0f, 0.0f, 0.0f));
    c = add3(lo, hi);
    if (m == 0.0f) {
      const double zero = 0.0;
      c = make_float3((float)(6.0 / 255 / zero), (float)(214.0 / 255.0), (float)(160.0 / 255.0));
    }
  }
  colors[3 * i] = c.x;
  colors[3 * i + 1] = c.y;
  colors[3 * i + 2] = c.z;
}

}  // namespace gg

extern "C" gg_status gg_color_buffer(gg_system* S, gg_set set, int32_t mode, float min_mass, float max_mass,
                                     float* d_dots, float* d_colors) {
  using namespace gg;
  if (!S || !d_dots || !d_colors || mode < 0 || mode > 2) {
    set_error("gg_color_buffer: null argument or mode outside 0..2");
    return GG_ERR_INVALID_ARGUMENT;
  }
  int64_t n = 0;
  const float4* pos = nullptr;
  const float* mass = nullptr;
  const int32_t* surface = nullptr;
  const float* sdist = nullptr;
  switch (set) {
    case GG_SET_GRANULAR:
      n = S->n;
      pos = S->g.pos[S->g.cur];
      mass = S->g.mass[S->g.cur];
      surface = S->g.surface;
      sdist = S->g.sdist;
      break;
    case GG_SET_UPSAMPLED:
      n = S->nu;
      pos = S->u.pos[S->u.cur];
      break;
    default:
      set_error("gg_color_buffer: the reference colours the particles and the render points only");
      return GG_ERR_INVALID_ARGUMENT;
  }
  if (n <= 0) return GG_OK;
  GG_CUDA(cudaSetDevice(S->device));
  k_color_dots<<<blocks_for(n, 256), 256, 0, S->stream>>>((int)n, pos, mass, surface, sdist, mode, min_mass, max_mass,
                                                         d_dots, d_colors);
  count_launches(S, 1);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

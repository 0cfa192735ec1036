// kernels_batch.cu — many independent scenes in one system.
//
// A batch places its scenes side by side along x, scene k in the slab
// k*w <= x < (k+1)*w with its own box walls and at least one empty cell
// between neighbouring boxes, so one grid, one sort and one launch of each
// kernel serve every scene and no contact crosses from one scene to
// another.  Scenes may differ in particle count and friction (gg_set_scenes);
// FP64 diagnostics are reduced per scene.  A batch of substeps can be
// captured once into a CUDA graph and replayed with one launch
// (gg_graph_capture / gg_graph_launch).  No counterpart in the reference,
// which steps one scene per GranularSystem with a host-driven sequence of
// launches and synchronisations.
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace gg {

constexpr int kSceneStats = 10;  // count, mass, momentum xyz, kinetic energy, mass-weighted x y z, nonfinite
constexpr int kMaxScenes = 1024;

// Per-scene FP64 sums: one shared-memory table per block (shared atomics),
// then one global atomic per scene and field per block.
__global__ void __launch_bounds__(256) k_scene_stats(int n, const float4* __restrict__ pos,
                                                     const float4* __restrict__ vel,
                                                     const float* __restrict__ mass, float inv_w, int n_scenes,
                                                     double* __restrict__ acc) {
  extern __shared__ double sh[];
  for (int k = threadIdx.x; k < n_scenes * kSceneStats; k += blockDim.x) sh[k] = 0.0;
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = pos[i];
    const float4 v = vel[i];
    const double m = mass[i];
    const int s = min(max(__float2int_rz(p.x * inv_w), 0), n_scenes - 1);
    double* t = sh + s * kSceneStats;
    const bool fin = isfinite(p.x) && isfinite(p.y) && isfinite(p.z);
    atomicAdd(&t[0], 1.0);
    atomicAdd(&t[1], m);
    atomicAdd(&t[2], m * v.x);
    atomicAdd(&t[3], m * v.y);
    atomicAdd(&t[4], m * v.z);
    atomicAdd(&t[5], 0.5 * m * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z));
    if (fin) {
      atomicAdd(&t[6], m * p.x);
      atomicAdd(&t[7], m * p.y);
      atomicAdd(&t[8], m * p.z);
    } else {
      atomicAdd(&t[9], 1.0);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n_scenes * kSceneStats; k += blockDim.x)
    if (sh[k] != 0.0) atomicAdd(&acc[k], sh[k]);
}

gg_status step_once(gg_system* S);

}  // namespace gg

using namespace gg;

extern "C" {

gg_status gg_set_scenes(gg_system* S, int32_t n_scenes, float width, const float* friction_cap) {
  if (!S || n_scenes < 0 || n_scenes > kMaxScenes || (n_scenes > 0 && !(width > 0.0f))) {
    set_error("gg_set_scenes: bad argument (at most 1024 scenes, width > 0)");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(S->device));
  GG_CUDA(cudaStreamSynchronize(S->stream));
  cudaFree(S->scene_fcap);
  cudaFree(S->scene_acc);
  cudaFree(S->scene_mu);
  S->scene_fcap = nullptr;
  S->scene_acc = nullptr;
  S->scene_mu = nullptr;
  S->n_scenes = 0;
  S->scene_width = 0.0f;
  if (n_scenes == 0) return GG_OK;
  GG_CUDA(cudaMalloc((void**)&S->scene_acc, sizeof(double) * kSceneStats * n_scenes));
  if (friction_cap) {
    GG_CUDA(cudaMalloc((void**)&S->scene_fcap, sizeof(float) * n_scenes));
    GG_CUDA(cudaMemcpy(S->scene_fcap, friction_cap, sizeof(float) * n_scenes, cudaMemcpyHostToDevice));
  }
  S->n_scenes = n_scenes;
  S->scene_width = width;
  return GG_OK;
}

gg_status gg_set_scene_coulomb(gg_system* S, int32_t n_scenes, const float* mu_static, const float* mu_kinetic) {
  if (!S || n_scenes != S->n_scenes || n_scenes <= 0 || !mu_static != !mu_kinetic) {
    set_error("gg_set_scene_coulomb: set the scenes first (gg_set_scenes), pass their number and both "
              "coefficient arrays (or neither)");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(S->device));
  GG_CUDA(cudaStreamSynchronize(S->stream));
  cudaFree(S->scene_mu);
  S->scene_mu = nullptr;
  if (!mu_static) return GG_OK;
  std::vector<float2> mu((size_t)n_scenes);
  for (int k = 0; k < n_scenes; ++k) {
    if (!(mu_static[k] >= 0.0f) || !(mu_kinetic[k] >= 0.0f)) {
      set_error("gg_set_scene_coulomb: coefficients must be non-negative");
      return GG_ERR_INVALID_ARGUMENT;
    }
    mu[k] = make_float2(mu_static[k], mu_kinetic[k]);
  }
  GG_CUDA(cudaMalloc((void**)&S->scene_mu, sizeof(float2) * n_scenes));
  GG_CUDA(cudaMemcpy(S->scene_mu, mu.data(), sizeof(float2) * n_scenes, cudaMemcpyHostToDevice));
  return GG_OK;
}

gg_status gg_scene_stats(gg_system* S, double* host_out, int32_t n_scenes) {
  if (!S || !host_out || n_scenes != S->n_scenes || n_scenes <= 0) {
    set_error("gg_scene_stats: set the scenes first (gg_set_scenes) and pass their number");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaSetDevice(S->device));
  cudaStream_t st = S->stream;
  const size_t bytes = sizeof(double) * kSceneStats * n_scenes;
  GG_CUDA(cudaMemsetAsync(S->scene_acc, 0, bytes, st));
  if (S->n > 0) {
    const int c = S->g.cur;
    const int blocks = std::max(1, std::min(blocks_for(S->n, 256), 4 * S->num_sms));
    k_scene_stats<<<blocks, 256, bytes, st>>>((int)S->n, S->g.pos[c], S->g.vel[c], S->g.mass[c],
                                              1.0f / S->scene_width, n_scenes, S->scene_acc);
    count_launches(S, 1);
    GG_CUDA(cudaGetLastError());
  }
  std::vector<double> acc((size_t)kSceneStats * n_scenes);
  GG_CUDA(cudaMemcpyAsync(acc.data(), S->scene_acc, bytes, cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  // out per scene: count, mass, momentum xyz, kinetic energy, centre of mass xyz
  for (int s = 0; s < n_scenes; ++s) {
    const double* a = acc.data() + (size_t)s * kSceneStats;
    double* o = host_out + (size_t)s * 9;
    for (int k = 0; k < 6; ++k) o[k] = a[k];
    for (int k = 0; k < 3; ++k) o[6 + k] = a[1] > 0.0 ? a[6 + k] / a[1] : 0.0;
  }
  return GG_OK;
}

gg_status gg_graph_capture(gg_system* S, int32_t n_substeps) {
  // The particle arrays are double-buffered and a substep moves the live
  // copy to the other buffer; the graph replays fixed addresses, so it must
  // end where it began: an even number of substeps.
  if (!S || n_substeps <= 0 || (n_substeps & 1)) {
    set_error("gg_graph_capture: n_substeps must be even and positive");
    return GG_ERR_INVALID_ARGUMENT;
  }
  if ((S->phys.is_adaptive == 1 && S->P.merge_enabled) || S->P.target_residual > 0.0f || S->profiling ||
      S->frame_timing || S->phys.is_move_boundary) {
    set_error("gg_graph_capture: the substep must run without host round trips (no merge/split, no residual "
              "mode, no moving walls, profiling and frame timing off)");
    return GG_ERR_NOT_SUPPORTED;
  }
  GG_CUDA(cudaSetDevice(S->device));
  GG_CUDA(cudaStreamSynchronize(S->stream));
  if (S->graph_exec) {
    cudaGraphExecDestroy(S->graph_exec);
    S->graph_exec = nullptr;
  }
  const int64_t steps0 = S->steps, launches0 = S->launches;
  const int cur0 = S->g.cur, ucur0 = S->u.cur;
  cudaGraph_t graph = nullptr;
  GG_CUDA(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
  gg_status rc = GG_OK;
  for (int k = 0; k < n_substeps && rc == GG_OK; ++k) rc = step_once(S);
  const cudaError_t e = cudaStreamEndCapture(S->stream, &graph);
  S->steps = steps0;
  S->graph_launches = S->launches - launches0;
  S->launches = launches0;
  if (S->g.cur != cur0 || S->u.cur != ucur0) {
    if (graph) cudaGraphDestroy(graph);
    S->g.cur = cur0;
    S->u.cur = ucur0;
    set_error("gg_graph_capture: the captured substeps do not return to the starting buffers");
    return GG_ERR_NOT_SUPPORTED;
  }
  if (rc != GG_OK || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    if (rc == GG_OK) {
      set_error(std::string("gg_graph_capture: capture failed: ") + cudaGetErrorString(e));
      rc = GG_ERR_NOT_SUPPORTED;
    }
    return rc;
  }
  const cudaError_t ie = cudaGraphInstantiate(&S->graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    S->graph_exec = nullptr;
    cudaGetLastError();
    set_error(std::string("gg_graph_capture: instantiation failed: ") + cudaGetErrorString(ie));
    return GG_ERR_CUDA;
  }
  S->graph_substeps = n_substeps;
  return GG_OK;
}

gg_status gg_graph_launch(gg_system* S) {
  if (!S || !S->graph_exec) {
    set_error("gg_graph_launch: no captured graph");
    return GG_ERR_INVALID_ARGUMENT;
  }
  GG_CUDA(cudaGraphLaunch(S->graph_exec, S->stream));
  S->steps += S->graph_substeps;
  S->launches += S->graph_launches;
  return GG_OK;
}

}  // extern "C"

// kernels_grid.cu — uniform-grid neighbour structure.
//
// Replaces neighbor_search_{granular,boundary,upsampled}
// (GranularSystem.cu:65-395) and the primitives of CUDAFunctions.cuh:54-107:
//   cell key per particle  -> stable LSD radix sort of (key, index)
//   -> one gather of every SoA field -> cell_start by count + exclusive scan.
// The sort is stable, as thrust::sort_by_key on int keys is, so the sorted
// order is identical; it sorts only ceil(log2(C+1)) key bits.
#include <mutex>
#include <utility>

#include "common.cuh"

namespace gg {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;   // 4096
constexpr int kScanTopThreads = 1024;
constexpr int kScanTopItems = 16;
constexpr int64_t kScanMaxBlocks = (int64_t)kScanTopThreads * kScanTopItems;

int key_bits(int C) {
  int b = 1;
  while (b < 31 && ((int64_t)1 << b) <= (int64_t)C) ++b;
  return b;  // keys take values 0..C
}

// ------------------------------------------------------------------ hash

// mapParticles2Cells_CUDA (CUDAFunctions.cuh:91-107) with the sort's value
// array (thrust::sequence, GranularSystem.cu:71-73) produced in one pass.
// One block per sort tile: the block also counts the tile's first radix
// digits (bits 0-7), hist0 digit-major [256][tiles], so the sort's first
// pass does not read the keys again for its histogram.
__global__ void __launch_bounds__(kSortThreads) k_hash(Grid g, const float4* __restrict__ pos, int n,
                                                       uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                       uint32_t* __restrict__ keys_copy, int tiles,
                                                       uint32_t* __restrict__ hist0) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * kSortTile;
  const unsigned lt = lanemask_lt();
#pragma unroll 4
  for (int r = 0; r < kSortItems; ++r) {
    const int i = base + r * kSortThreads + threadIdx.x;
    uint32_t d = 0u;
    if (i < n) {
      const float4 p = pos[i];
      const int3 c = floor_cell(g, make_float3(p.x, p.y, p.z));
      const uint32_t k = (uint32_t)cell_key(g, c.x, c.y, c.z);
      keys[i] = k;
      vals[i] = (uint32_t)i;
      if (keys_copy) keys_copy[i] = k;
      d = k & 255u;
    }
    // one shared-memory atomic per distinct digit of the warp (sorted or
    // nearly sorted keys share their digit across the warp)
    const unsigned peers = __match_any_sync(0xffffffffu, i < n ? d : 256u);
    if (i < n && (peers & lt) == 0) atomicAdd(&h[d], (uint32_t)__popc(peers));
  }
  __syncthreads();
  hist0[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// ------------------------------------------------------------ block scan

// Exclusive scan of one int per thread across a block of kThreads threads;
// returns the block total in *total.
template <int kThreads>
__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
  __shared__ int warp_tot[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < kThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kThreads / 32) warp_tot[lane] = w;
  }
  __syncthreads();
  const int warp_prefix = warp ? warp_tot[warp - 1] : 0;
  *total = warp_tot[kThreads / 32 - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

// -------------------------------------------------------- exclusive scan

__global__ void k_scan_reduce(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ bsum) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + k;
    if (i < n) s += in[i];
  }
  int tot;
  block_exclusive_scan<kScanThreads>(s, &tot);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void k_scan_top(int32_t* __restrict__ bsum, int nb, int32_t* __restrict__ total_out) {
  const int base = threadIdx.x * kScanTopItems;
  int v[kScanTopItems];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanTopItems; ++k) {
    v[k] = (base + k < nb) ? bsum[base + k] : 0;
    s += v[k];
  }
  int tot;
  int run = block_exclusive_scan<kScanTopThreads>(s, &tot);
#pragma unroll
  for (int k = 0; k < kScanTopItems; ++k) {
    if (base + k < nb) bsum[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0 && total_out) *total_out = tot;
}

__global__ void k_scan_down(const int32_t* in, int32_t* out, int64_t n, const int32_t* __restrict__ bsum) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  int tot;
  int run = block_exclusive_scan<kScanThreads>(s, &tot) + bsum[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

gg_status exclusive_scan(const int32_t* in, int32_t* out, int64_t n, SortScratch& s, cudaStream_t st,
                         int32_t* total_out_dev) {
  if (n <= 0) {
    if (total_out_dev) GG_CUDA(cudaMemsetAsync(total_out_dev, 0, sizeof(int32_t), st));
    return GG_OK;
  }
  const int64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb > kScanMaxBlocks || nb > s.scan_block_entries) {
    set_error("exclusive_scan: input larger than the scan scratch");
    return GG_ERR_INVALID_ARGUMENT;
  }
  k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, s.scan_blocks);
  k_scan_top<<<1, kScanTopThreads, 0, st>>>(s.scan_blocks, (int)nb, total_out_dev);
  k_scan_down<<<(unsigned)nb, kScanThreads, 0, st>>>(in, out, n, s.scan_blocks);
  if (s.counter) *s.counter += 3;
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// ------------------------------------------------------------ radix sort

// Per-tile histogram of one 8-bit digit; hist is digit-major [256][tiles].
// The thread's 16 keys are loaded before any is counted, so that their
// loads are in flight together; counts are aggregated over the lanes of a
// warp holding the same digit (one shared-memory atomic per digit).
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const uint32_t* __restrict__ keys, int n, int shift,
                                                             int tiles, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  const int base = blockIdx.x * kSortTile;
  uint32_t k[kSortItems];
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const int i = base + r * kSortThreads + threadIdx.x;
    k[r] = i < n ? keys[i] : 0u;
  }
  __syncthreads();
  const unsigned lt = lanemask_lt();
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const bool valid = base + r * kSortThreads + (int)threadIdx.x < n;
    const uint32_t d = (k[r] >> shift) & 255u;
    const unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 256u);
    if (valid && (peers & lt) == 0) atomicAdd(&h[d], (uint32_t)__popc(peers));
  }
  __syncthreads();
  hist[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one digit: items are ranked in index order within the
// tile (rounds of 256 consecutive items; within a round by warp, then by
// lane).  offs holds the exclusive scan of the digit-major [256][tiles]
// histogram.  The thread's 16 keys and values are loaded before the first
// round, so that the rounds wait on no global load.  In a round, the first
// lane of each group of equal digits in a warp posts the group's size in
// wcnt; after the writes it adds the size to the digit's running base and
// clears its entry, so that wcnt is all zero between rounds.
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const uint32_t* __restrict__ kin,
                                                                const uint32_t* __restrict__ vin,
                                                                uint32_t* __restrict__ kout,
                                                                uint32_t* __restrict__ vout, int n, int shift,
                                                                int tiles, const uint32_t* __restrict__ offs) {
  constexpr int W = kSortThreads / 32;
  __shared__ uint32_t base_d[256];
  __shared__ uint32_t wcnt[W][256];
  const int t = threadIdx.x, warp = t >> 5;
  const int base = blockIdx.x * kSortTile;
  uint32_t k[kSortItems], v[kSortItems];
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const int i = base + r * kSortThreads + t;
    k[r] = i < n ? kin[i] : 0u;
    v[r] = i < n ? vin[i] : 0u;
  }
#pragma unroll
  for (int w = 0; w < W; ++w) wcnt[w][t] = 0;
  base_d[t] = offs[t * tiles + blockIdx.x];
  __syncthreads();
  const unsigned lt = lanemask_lt();
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const bool valid = base + r * kSortThreads + t < n;
    const uint32_t d = (k[r] >> shift) & 255u;
    const unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 256u);
    const bool leader = valid && (peers & lt) == 0;
    const uint32_t cnt = (uint32_t)__popc(peers);
    if (leader) wcnt[warp][d] = cnt;
    __syncthreads();
    if (valid) {
      uint32_t dst = base_d[d] + (uint32_t)__popc(peers & lt);
      for (int w = 0; w < warp; ++w) dst += wcnt[w][d];
      kout[dst] = k[r];
      vout[dst] = v[r];
    }
    __syncthreads();
    if (leader) {
      atomicAdd(&base_d[d], cnt);
      wcnt[warp][d] = 0;
    }
    __syncwarp();
  }
}

gg_status sort_scratch_alloc(SortScratch& s, int64_t capacity) {
  if (capacity < 1) capacity = 1;
  s.capacity = capacity;
  const int64_t tiles = (capacity + kSortTile - 1) / kSortTile;
  s.hist_entries = tiles * 256;
  // scan blocks must cover the largest scanned array: hist, cell table, particles
  s.scan_block_entries = kScanMaxBlocks;
  for (int i = 0; i < 2; ++i) {
    GG_CUDA(cudaMalloc(&s.k[i], sizeof(uint32_t) * capacity));
    GG_CUDA(cudaMalloc(&s.v[i], sizeof(uint32_t) * capacity));
  }
  GG_CUDA(cudaMalloc(&s.hist, sizeof(uint32_t) * s.hist_entries));
  GG_CUDA(cudaMalloc(&s.scan_blocks, sizeof(int32_t) * s.scan_block_entries));
  return GG_OK;
}

void sort_scratch_free(SortScratch& s) {
  for (int i = 0; i < 2; ++i) {
    cudaFree(s.k[i]);
    cudaFree(s.v[i]);
    s.k[i] = s.v[i] = nullptr;
  }
  cudaFree(s.hist);
  cudaFree(s.scan_blocks);
  s.hist = nullptr;
  s.scan_blocks = nullptr;
}

// Stable LSD sort of the (key, value) pairs held in s.k[0], s.v[0]; the
// last pass writes keys_out / perm_out.  hist0_ready: s.hist already holds
// the first digit's tile histogram (counted by the hash kernel).
static gg_status radix_sort_pairs(const Grid& g, int64_t n, SortScratch& s, uint32_t* keys_out, uint32_t* perm_out,
                                  cudaStream_t st, bool hist0_ready) {
  const int nn = (int)n;
  const int bits = key_bits(g.C);
  const int passes = (bits + 7) / 8;
  const int tiles = (int)((n + kSortTile - 1) / kSortTile);
  int src = 0;
  for (int p = 0; p < passes; ++p) {
    const int shift = 8 * p;
    const bool last = p == passes - 1;
    uint32_t* ko = last ? keys_out : s.k[src ^ 1];
    uint32_t* vo = last ? perm_out : s.v[src ^ 1];
    if (p > 0 || !hist0_ready) {
      k_radix_hist<<<tiles, kSortThreads, 0, st>>>(s.k[src], nn, shift, tiles, s.hist);
      if (s.counter) *s.counter += 1;
    }
    gg_status rc = exclusive_scan((const int32_t*)s.hist, (int32_t*)s.hist, (int64_t)tiles * 256, s, st, nullptr);
    if (rc != GG_OK) return rc;
    k_radix_scatter<<<tiles, kSortThreads, 0, st>>>(s.k[src], s.v[src], ko, vo, nn, shift, tiles, s.hist);
    if (s.counter) *s.counter += 1;
    src ^= 1;
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

gg_status grid_sort(const Grid& g, const float4* pos, int64_t n, SortScratch& s, uint32_t* keys_out,
                    uint32_t* perm_out, uint32_t* keys_unsorted_out, cudaStream_t st, gg_system* prof) {
  if (n <= 0) return GG_OK;
  if (n > s.capacity) {
    set_error("grid_sort: more elements than the sort scratch holds");
    return GG_ERR_INVALID_ARGUMENT;
  }
  const int nn = (int)n;
  if (prof) prof_begin(prof, PC_HASH, st);
  const int tiles = (int)((n + kSortTile - 1) / kSortTile);
  k_hash<<<tiles, kSortThreads, 0, st>>>(g, pos, nn, s.k[0], s.v[0], keys_unsorted_out, tiles, s.hist);
  if (s.counter) *s.counter += 1;
  if (prof) prof_end(prof, PC_HASH, n, st);
  if (prof) prof_begin(prof, PC_SORT, st);
  gg_status rc = radix_sort_pairs(g, n, s, keys_out, perm_out, st, true);
  if (prof) prof_end(prof, PC_SORT, n, st);
  return rc;
}

// ------------------------------------------------------------ cell start

// countingInCell_CUDA (CUDAFunctions.cuh:54-61) on the sorted keys, one
// atomic per run of equal keys in a warp.
__global__ void k_count_cells(const uint32_t* __restrict__ keys, int n, int32_t* __restrict__ counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t k = i < n ? keys[i] : 0xffffffffu;
  const unsigned peers = __match_any_sync(0xffffffffu, k);
  if (i < n && __popc(peers & lanemask_lt()) == 0) atomicAdd(&counts[k], __popc(peers));
}

gg_status cell_start_build(const Grid& g, const uint32_t* sorted_keys, int64_t n, int32_t* cell_start,
                           SortScratch& s, cudaStream_t st, gg_system* prof) {
  if (prof) prof_begin(prof, PC_CELLSTART, st);
  GG_CUDA(cudaMemsetAsync(cell_start, 0, sizeof(int32_t) * ((int64_t)g.C + 1), st));
  if (n > 0) {
    k_count_cells<<<blocks_for(n, 256), 256, 0, st>>>(sorted_keys, (int)n, cell_start);
    if (s.counter) *s.counter += 1;
  }
  gg_status rc = exclusive_scan(cell_start, cell_start, (int64_t)g.C + 1, s, st, nullptr);
  if (prof) prof_end(prof, PC_CELLSTART, (int64_t)g.C + 1, st);
  GG_CUDA(cudaGetLastError());
  return rc;
}

// --------------------------------------------------------------- reorder

// The gathers of GranularSystem.cu:97-135 for every permuted field in one
// pass.  adaptive_last_step and merge_velocity are not permuted, as in the
// reference.
__global__ void k_reorder_granular(int n, const uint32_t* __restrict__ perm,
                                   const float4* __restrict__ pos_in, float4* __restrict__ pos_out,
                                   const float4* __restrict__ vel_in, float4* __restrict__ vel_out,
                                   const float* __restrict__ mass_in, float* __restrict__ mass_out,
                                   const float* __restrict__ rs_in, float* __restrict__ rs_out,
                                   const int32_t* __restrict__ units_in, int32_t* __restrict__ units_out,
                                   const float* __restrict__ merge_in, float* __restrict__ merge_out,
                                   const int32_t* __restrict__ mu_in, int32_t* __restrict__ mu_out,
                                   const int32_t* __restrict__ mc_in, int32_t* __restrict__ mc_out,
                                   const int32_t* __restrict__ rm_in, int32_t* __restrict__ rm_out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t s = perm[p];
  pos_out[p] = pos_in[s];
  vel_out[p] = vel_in[s];
  mass_out[p] = mass_in[s];
  rs_out[p] = rs_in[s];
  units_out[p] = units_in[s];
  merge_out[p] = merge_in[s];
  mu_out[p] = mu_in[s];
  mc_out[p] = mc_in[s];
  rm_out[p] = rm_in[s];
}

gg_status reorder_granular(gg_system* S, cudaStream_t st) {
  if (S->n <= 0) return GG_OK;
  Granular& G = S->g;
  const int a = G.cur, b = G.cur ^ 1;
  prof_begin(S, PC_REORDER, st);
  k_reorder_granular<<<blocks_for(S->n, 256), 256, 0, st>>>(
      (int)S->n, G.perm, G.pos[a], G.pos[b], G.vel[a], G.vel[b], G.mass[a], G.mass[b], G.rs[a], G.rs[b],
      G.units[a], G.units[b], G.merge[a], G.merge[b], G.merge_units[a], G.merge_units[b],
      G.merge_count[a], G.merge_count[b], G.remove[a], G.remove[b]);
  count_launches(S, 1);
  // adaptive_last_step stays where it is: copy it into the new live buffer
  GG_CUDA(cudaMemcpyAsync(G.als[b], G.als[a], sizeof(int32_t) * S->n, cudaMemcpyDeviceToDevice, st));
  prof_end(S, PC_REORDER, S->n, st);
  G.cur = b;
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

__global__ void k_gather2(int n, const uint32_t* __restrict__ perm, const float4* __restrict__ a_in,
                          float4* __restrict__ a_out, const float4* __restrict__ b_in,
                          float4* __restrict__ b_out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t s = perm[p];
  a_out[p] = a_in[s];
  if (b_in) b_out[p] = b_in[s];
}

__global__ void k_gather_boundary(int n, const uint32_t* __restrict__ perm, const float4* __restrict__ p_in,
                                  float4* __restrict__ p_out, const int32_t* __restrict__ a_in,
                                  int32_t* __restrict__ a_out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t s = perm[p];
  p_out[p] = p_in[s];
  a_out[p] = a_in[s];
}

gg_status reorder_boundary(gg_system* S, const uint32_t* perm, cudaStream_t st) {
  if (S->nb <= 0) return GG_OK;
  k_gather_boundary<<<blocks_for(S->nb, 256), 256, 0, st>>>((int)S->nb, perm, S->b.pos, S->b.pos_alt,
                                                            S->b.animated, S->b.animated_alt);
  count_launches(S, 1);
  std::swap(S->b.pos, S->b.pos_alt);
  std::swap(S->b.animated, S->b.animated_alt);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

gg_status reorder_upsampled(gg_system* S, const uint32_t* perm, cudaStream_t st) {
  if (S->nu <= 0) return GG_OK;
  const int a = S->u.cur, b = a ^ 1;
  k_gather2<<<blocks_for(S->nu, 256), 256, 0, st>>>((int)S->nu, perm, S->u.pos[a], S->u.pos[b], S->u.vel[a],
                                                    S->u.vel[b]);
  count_launches(S, 1);
  S->u.cur = b;
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}


// ------------------------------------------------------------ grid build without allocation
//
// gg_grid_build_noalloc: the grid build above (cell keys, stable radix sort,
// cell start table) for callers that cannot allocate device memory, such as
// code hosted inside an engine or framework that owns every device
// allocation, or a loop that must not allocate once it is running.  The
// caller passes device buffers for the positions and for every output; the
// sort's scratch (two key/value ping-pong buffers, the per-tile digit
// histograms and the scan's block sums) lives in the file-scope array below,
// sized for at most kNoAllocMaxParticles particles and kNoAllocMaxCells
// cells.  Every GPU that loads this library holds that array (about 4.1 MiB)
// until the process exits.

constexpr int64_t kNoAllocMaxParticles = 1 << 18;
constexpr int64_t kNoAllocMaxCells = 1 << 24;
constexpr int64_t kNoAllocTiles = (kNoAllocMaxParticles + kSortTile - 1) / kSortTile;
constexpr size_t kNoAllocPairWords = 4 * (size_t)kNoAllocMaxParticles;   // k0, k1, v0, v1
constexpr size_t kNoAllocHistWords = 256 * (size_t)kNoAllocTiles;
constexpr size_t kNoAllocScanWords = (size_t)kScanMaxBlocks;
constexpr size_t kNoAllocWords = kNoAllocPairWords + kNoAllocHistWords + kNoAllocScanWords;

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

// mapParticles2Cells_CUDA over packed float[3] positions (12-byte stride).
__global__ void k_hash3(Grid g, const float* __restrict__ pos3, int n, uint32_t* __restrict__ keys,
                        uint32_t* __restrict__ vals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float3 p = make_float3(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]);
  const int3 c = floor_cell(g, p);
  keys[i] = (uint32_t)cell_key(g, c.x, c.y, c.z);
  vals[i] = (uint32_t)i;
}

namespace {
// Saves the calling thread's current device and restores it on scope exit.
struct DeviceGuard {
  int saved = 0;
  cudaError_t status;
  DeviceGuard() { status = cudaGetDevice(&saved); }
  ~DeviceGuard() {
    if (status == cudaSuccess) cudaSetDevice(saved);
  }
};

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
uint32_t* g_noalloc_dev[kNoAllocMaxDevices] = {};

// The array's name is a host-side stand-in, not a device address: the
// address is looked up once per device, with that device current.
gg_status noalloc_scratch(int device, uint32_t** out) {
  if (device < 0 || device >= kNoAllocMaxDevices) {
    set_error("gg_grid_build_noalloc: device ordinal out of range");
    return GG_ERR_INVALID_ARGUMENT;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_dev[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e, "gg_grid_build_noalloc: cudaGetSymbolAddress");
    g_noalloc_dev[device] = (uint32_t*)p;
  }
  *out = g_noalloc_dev[device];
  return GG_OK;
}
}  // namespace

}  // namespace gg

extern "C" gg_status gg_grid_build_noalloc(int32_t device, const float* d_pos, int64_t n,
                                           const int32_t cell_size[3], float cell_length,
                                           uint32_t* d_sorted_keys, uint32_t* d_perm, int32_t* d_cell_start,
                                           void* stream) {
  using namespace gg;
  try {
    if (!cell_size || !(cell_length > 0.0f) || n < 0 || (n > 0 && (!d_pos || !d_sorted_keys || !d_perm)) ||
        !d_cell_start) {
      set_error("gg_grid_build_noalloc: null buffer or invalid size");
      return GG_ERR_INVALID_ARGUMENT;
    }
    if (cell_size[0] <= 0 || cell_size[1] <= 0 || cell_size[2] <= 0) {
      set_error("gg_grid_build_noalloc: cell_size must be positive");
      return GG_ERR_INVALID_ARGUMENT;
    }
    const int64_t C = (int64_t)cell_size[0] * cell_size[1] * cell_size[2];
    if (n > kNoAllocMaxParticles || C > kNoAllocMaxCells) {
      set_error("gg_grid_build_noalloc: at most 262144 particles and 16777216 cells (static scratch limit); "
                "use gg_grid_create/gg_grid_build for larger inputs");
      return GG_ERR_CAPACITY;
    }
    // the caller's current device is put back on every return path
    DeviceGuard guard;
    if (guard.status != cudaSuccess) return cuda_status(guard.status, "gg_grid_build_noalloc: cudaGetDevice");
    GG_CUDA(cudaSetDevice(device));
    uint32_t* base = nullptr;
    gg_status rc = noalloc_scratch(device, &base);
    if (rc != GG_OK) return rc;
    SortScratch s;
    s.k[0] = base;
    s.k[1] = base + kNoAllocMaxParticles;
    s.v[0] = base + 2 * kNoAllocMaxParticles;
    s.v[1] = base + 3 * kNoAllocMaxParticles;
    s.hist = base + kNoAllocPairWords;
    s.scan_blocks = (int32_t*)(base + kNoAllocPairWords + kNoAllocHistWords);
    s.capacity = kNoAllocMaxParticles;
    s.hist_entries = (int64_t)kNoAllocHistWords;
    s.scan_block_entries = (int64_t)kNoAllocScanWords;
    Grid g;
    g.L = cell_length;
    g.nx = cell_size[0];
    g.ny = cell_size[1];
    g.nz = cell_size[2];
    g.C = (int)C;
    cudaStream_t st = (cudaStream_t)stream;
    if (n > 0) {
      k_hash3<<<blocks_for(n, 256), 256, 0, st>>>(g, d_pos, (int)n, s.k[0], s.v[0]);
      GG_CUDA(cudaGetLastError());
      rc = radix_sort_pairs(g, n, s, d_sorted_keys, d_perm, st, false);
      if (rc != GG_OK) return rc;
    }
    // cell_start_build clears the caller's table (the counts start at zero)
    // before counting; the histograms and block sums in the scratch are
    // fully written before they are read, so they need no clearing.
    return cell_start_build(g, d_sorted_keys, n, d_cell_start, s, st, nullptr);
  } catch (...) {
    set_error("gg_grid_build_noalloc: internal error");
    return GG_ERR_INVALID_ARGUMENT;
  }
}

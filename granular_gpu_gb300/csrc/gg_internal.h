// gg_internal.h — state of one gg_system and the kernel launchers shared by
// the translation units of libgg.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gg.h"

namespace gg {

// Grid geometry shared by every kernel: cell length and dims.
struct Grid {
  float L;
  int nx, ny, nz;
  int C;  // nx*ny*nz; the out-of-grid key
};

// Unsigned 32-bit division by an invariant d with a multiply-high
// (Granlund and Montgomery, "Division by invariant integers using
// multiplication", 1994; the round-up variant with a 33-bit multiplier):
// n / d = (hi(m n) + ((n - hi(m n)) >> 1)) >> s for every 32-bit n, d >= 2.
struct UDiv {
  uint32_t m = 0;
  int s = 0;
  uint32_t d = 1;
};
inline UDiv make_udiv(uint32_t d) {
  UDiv u;
  u.d = d;
  if (d <= 1) return u;
  int l = 0;
  while (((uint64_t)1 << l) < d) ++l;  // ceil(log2 d)
  u.m = (uint32_t)((((uint64_t)1 << 32) * (((uint64_t)1 << l) - d)) / d + 1);
  u.s = l - 1;
  return u;
}

// Scalars that live on the device so a substep needs no host round trip.
constexpr int kMaxSweeps = 2048;  // sweeps per substep (stabilisation + Jacobi)

struct DevScalars {
  unsigned int rmax_bits;      // max contact radius (float bits), this step
  unsigned int inc_bits[kMaxSweeps];  // per sweep: max |x* increment| per axis (float bits)
  unsigned int inc_norm_bits[kMaxSweeps];  // per sweep: max Euclidean length of an increment (float bits)
  unsigned int disp0_bits;     // max |dt v| of the predict (float bits)
  unsigned int tile_fallback;  // sweep blocks that could not use the shared-memory tile
  int nl_queued[kMaxSweeps];          // per sweep: particles whose contact list is rebuilt
  unsigned int pen_bits;       // residual mode: largest penetration (float bits)
  unsigned int pen_count;      // residual mode: contacts (particle pairs counted once per side, walls)
  double pen_sum;              // residual mode: sum of their penetrations
  int merge_changed[65];       // merge schedule: iteration m changed a claim status (index m, 1..64)
  int merge_final;             // merge schedule: iteration whose statuses are final
  int error_word;              // bit0 capacity, bit1 numeric, bit2 timeout, bit3 merge schedule unresolved
  int n_after;                 // particle count after the adaptive step
  int n_removed;
  int n_split;
  int n_split_appended;
  int n_kept;
  unsigned long long nlist_rebuilds;  // listed-sweep list builds (not reset per substep)
};


enum ErrorBits { ERR_CAPACITY = 1, ERR_NUMERIC = 2, ERR_TIMEOUT = 4, ERR_MERGE_SCHEDULE = 8 };
constexpr int kMergeMaxIter = 64;  // claim-status iterations of the merge schedule

// Largest element count of a set: launches round counts up to whole tiles
// of at most 4,096 items and index them with signed 32-bit integers.
constexpr int64_t kMaxCount = ((int64_t)1 << 31) - ((int64_t)1 << 16);
constexpr int kNlistMax = 64;  // contact candidates kept per particle (walls within reach included)

// Kernel classes timed by gg_profile_*.
enum ProfClass {
  PC_HASH = 0, PC_SORT, PC_REORDER, PC_CELLSTART, PC_PREDICT, PC_SWEEP, PC_APPLY,
  PC_FINALIZE, PC_UPSAMPLE, PC_UP_GRID, PC_SURFACE, PC_SURFDIST, PC_MERGE, PC_SPLIT,
  PC_COMPACT, PC_STATS, PC_FEATURES, PC_MLP, PC_RESIDUAL, PC_COUNT
};

// Double-buffered particle SoA; index `cur` is the live copy.
struct Granular {
  float4* pos[2] = {nullptr, nullptr};    // x, y, z, contact radius
  float4* vel[2] = {nullptr, nullptr};    // x, y, z, unused
  float* mass[2] = {nullptr, nullptr};
  float* rs[2] = {nullptr, nullptr};      // surface-law radius
  int32_t* units[2] = {nullptr, nullptr}; // integer mass ledger
  float* merge[2] = {nullptr, nullptr};
  int32_t* merge_units[2] = {nullptr, nullptr};
  int32_t* merge_count[2] = {nullptr, nullptr};
  int32_t* remove[2] = {nullptr, nullptr};
  int32_t* als[2] = {nullptr, nullptr};   // adaptive_last_step (never permuted by the sort)
  int cur = 0;
  // never permuted or compacted (as in the reference)
  float4* merge_vel = nullptr;
  // recomputed every step
  int32_t* surface = nullptr;
  float* sdist = nullptr;
  float4* cover = nullptr;
  float4* xs = nullptr;       // predicted positions x*, w = contact radius
  float* inv_m = nullptr;     // 1 / (m exp(-y))
  float4* delta = nullptr;    // sweep output: dx, dy, dz, packed counts
  int32_t* s_extra = nullptr; // reverse constraint counts delivered by atomics
  int32_t* contacts = nullptr;
  int32_t* ncon = nullptr;
  int32_t* nl_idx = nullptr;  // contact candidate lists [kNlistMax][cap]
  int4* nl_meta = nullptr;    // query cell at list build, entry count (-1 = overflow)
  float* nl_acc = nullptr;    // displacement bound summed since the particle's list build
  int32_t* nl_queue = nullptr; // particles whose list is rebuilt in this sweep
  uint32_t* cell_inc = nullptr; // per cell (C+1): max |x* increment| of its particles in the last sweep (float bits)
  float* ld_sum = nullptr;       // surface pass: mass within the merge radius, in candidate order
  int32_t* ld_cnt = nullptr;     // and the count (-1: not computed there)
  // grid
  uint32_t* keys = nullptr;   // sorted keys of the last build
  uint32_t* perm = nullptr;   // sort permutation of the last build
  int32_t* cell_start = nullptr;
  uint8_t* cell_surf = nullptr;  // C + 1: cell holds a surface particle (scratch of the surface distance)
  // adaptive scratch
  int32_t* prop = nullptr;
  float* ldens = nullptr;
  int32_t* winner = nullptr;
  int32_t* claim_tgt = nullptr;  // merge schedule: the proposing partner a proposer claims first, or -1
  uint32_t* cell_claim = nullptr; // split claims per cell (C; 0xffffffff = free), configured mode
  float4* fdelta = nullptr;       // Coulomb law: summed friction targets (xyz) and their count (w)
  float* pn = nullptr;            // Coulomb law: normal correction received in the substep so far
  int32_t* child_cell = nullptr;  // cell a split child claimed, or -1
  uint8_t* claimed = nullptr;    // merge schedule: 2 x cap claim statuses (iterations ping-pong)
  int32_t* split_flag = nullptr;
  int32_t* keep_flag = nullptr;
  int32_t* split_slot = nullptr;
  int32_t* keep_slot = nullptr;
  float4* child_pos = nullptr;
};

struct Boundary {
  float4* pos = nullptr;        // live copy
  int32_t* animated = nullptr;
  float4* pos_alt = nullptr;    // reorder target, swapped with the live copy
  int32_t* animated_alt = nullptr;
  uint32_t* keys = nullptr;     // sorted keys of the last build
  uint32_t* perm = nullptr;
  int32_t* cell_start = nullptr;
};

struct Upsampled {
  float4* pos[2] = {nullptr, nullptr};
  float4* vel[2] = {nullptr, nullptr};
  uint32_t* keys = nullptr;     // sorted keys of the last build
  uint32_t* perm = nullptr;
  int cur = 0;
};

// Scratch for the radix sort and scans, sized for max(cap, nu, nb, C+1).
struct SortScratch {
  uint32_t* k[2] = {nullptr, nullptr};
  uint32_t* v[2] = {nullptr, nullptr};
  uint32_t* hist = nullptr;   // 256 x tiles
  int32_t* scan_blocks = nullptr;
  int64_t capacity = 0;
  int64_t hist_entries = 0;
  int64_t scan_block_entries = 0;
  int64_t* counter = nullptr;  // kernel launches are added here when set
};

struct Physics {
  float dt;
  float3 g;
  float density;
  int rho_i;
  float space[3];
  float upsampled_radius;
  int is_move_boundary;
  int is_adaptive;
};

}  // namespace gg

// Launch shapes chosen by gg_autotune (defaults: the shapes written in the
// kernels' launch bounds).
struct Tuning {
  int predict_threads = 256;
  int apply_threads = 256;
  int finalize_threads = 256;
  int keep_threads = 128;  // gg_autotune chose 128 on the column, the pile and the batched scenes
  int build_blocks_per_sm = 16;
  int sweep_variant = 0;  // variant of the default sweep: 0 contact lists, 1 pruned stencil sweep
};

struct gg_system {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  gg::Grid grid{};
  gg_params P{};
  gg::Physics phys{};
  int64_t n = 0, cap = 0, nb = 0, nu = 0;
  int64_t n_grid = 0;  // granular count at the last grid build (length of keys/perm)
  gg::Granular g;
  gg::Boundary b;
  gg::Upsampled u;
  gg::SortScratch sort;
  gg::DevScalars* scal = nullptr;      // device
  gg::DevScalars* scal_host = nullptr; // pinned mirror
  double* stats_partial = nullptr;     // device FP64 partials
  float* stage = nullptr;              // device float[3] staging for host copies (max set size)
  // learned warm start (allocated by gg_set_warm_start)
  gg_mlp* mlp = nullptr;               // attached network (not owned)
  void* feat = nullptr;                // cap x 48 bf16 features of the last substep
  float4* xs0 = nullptr;               // cap: x* after the predict (warm_start = 2)
  float* warm_target = nullptr;        // cap x 3: (x*_final - x*_predict) / (|g| dt^2)
  // batched scenes (gg_set_scenes): scene k is the slab k*width <= x < (k+1)*width
  int n_scenes = 0;
  float scene_width = 0.0f;
  float* scene_fcap = nullptr;         // device, per scene
  float2* scene_mu = nullptr;          // device, per scene: Coulomb mu_static, mu_kinetic
  double* scene_acc = nullptr;         // device, per scene x kSceneStats
  // a captured substep sequence (gg_graph_capture)
  cudaGraphExec_t graph_exec = nullptr;
  int graph_substeps = 0;
  int64_t graph_launches = 0;          // kernels per graph launch
  Tuning tune;
  int32_t last_sweeps = 0;
  float last_residual = 0.0f;         // mean penetration over contacts
  float last_residual_max = 0.0f;     // largest penetration
  int stats_blocks = 0;
  int num_sms = 0;
  int merge_resolve_blocks = 0;  // co-resident blocks of the cooperative merge-schedule kernel
  float nl_skin = 0.0f;                // contact-list skin in use (0 = lists off)
  int64_t steps = 0;
  int64_t launches = 0;                // kernels launched since create
  int merge_iter = 0;
  int64_t merged_last = 0, split_last = 0, merged_total = 0, split_total = 0;
  int32_t error_word = 0;
  std::vector<int64_t> stats_rows;     // merged, split, total per adaptive step
  // timing
  bool frame_timing = false;
  std::vector<float> frame_times;
  cudaEvent_t frame_ev[2] = {nullptr, nullptr};
  bool profiling = false;
  struct ProfEv { cudaEvent_t a, b; int cls; int64_t units; };
  std::vector<ProfEv> prof_pending;
  std::vector<cudaEvent_t> prof_pool;
  size_t prof_pool_used = 0;
  double prof_ms[gg::PC_COUNT] = {};
  int64_t prof_launches[gg::PC_COUNT] = {};
  int64_t prof_units[gg::PC_COUNT] = {};
  int64_t prof_launch_base = 0;
};

struct gg_grid {
  int device = 0;
  cudaStream_t stream = nullptr;
  gg::Grid grid{};
  int64_t cap = 0;
  float4* pos = nullptr;
  uint32_t* keys_unsorted = nullptr;
  uint32_t* sorted_keys = nullptr;
  uint32_t* perm = nullptr;
  int32_t* cell_start = nullptr;
  gg::SortScratch sort;
};

namespace gg {

// ---- error handling (api.cpp) ----
void set_error(const std::string& msg);
gg_status cuda_status(cudaError_t e, const char* what);
#define GG_CUDA(call)                                               \
  do {                                                              \
    cudaError_t e__ = (call);                                       \
    if (e__ != cudaSuccess) return gg::cuda_status(e__, #call);     \
  } while (0)

// ---- launchers (kernels_*.cu) ----
// grid
gg_status sort_scratch_alloc(SortScratch& s, int64_t capacity);
void sort_scratch_free(SortScratch& s);
int key_bits(int C);
// Computes keys of pos[0..n) and the stable sort permutation; sorted keys in
// keys_out, permutation in perm_out (both device, n entries).
gg_status grid_sort(const Grid& g, const float4* pos, int64_t n, SortScratch& s,
                    uint32_t* keys_out, uint32_t* perm_out, uint32_t* keys_unsorted_out,
                    cudaStream_t st, gg_system* prof);
gg_status cell_start_build(const Grid& g, const uint32_t* sorted_keys, int64_t n,
                           int32_t* cell_start, SortScratch& s, cudaStream_t st, gg_system* prof);
gg_status exclusive_scan(const int32_t* in, int32_t* out, int64_t n, SortScratch& s,
                         cudaStream_t st, int32_t* total_out_dev);
gg_status reorder_granular(gg_system* S, cudaStream_t st);
gg_status reorder_boundary(gg_system* S, const uint32_t* perm, cudaStream_t st);
gg_status reorder_upsampled(gg_system* S, const uint32_t* perm, cudaStream_t st);

// solve
gg_status radii_all(gg_system* S, cudaStream_t st);
gg_status predict(gg_system* S, cudaStream_t st);
gg_status sweep(gg_system* S, int it, cudaStream_t st);
// last: write the constraint counts (the substep's last sweep, or every
// sweep of the residual mode); more: another sweep may follow, so record the
// per-cell increments its contact lists are checked against.
gg_status apply(gg_system* S, int it, bool stab, bool last, bool more, cudaStream_t st);
gg_status finalize(gg_system* S, cudaStream_t st);
gg_status upsample(gg_system* S, cudaStream_t st);
gg_status explosion(gg_system* S, float force, cudaStream_t st);

// adaptive
gg_status surface(gg_system* S, cudaStream_t st);
gg_status surface_distance(gg_system* S, cudaStream_t st);
gg_status merge_mark(gg_system* S, cudaStream_t st);
gg_status merge_count(gg_system* S, cudaStream_t st);
gg_status split_and_compact(gg_system* S, cudaStream_t st);
// learned warm start and residual-targeted sweeps (kernels_learn.cu)
gg_status warm_start_apply(gg_system* S, cudaStream_t st);
gg_status warm_start_record(gg_system* S, cudaStream_t st);
gg_status warm_start_target(gg_system* S, cudaStream_t st);
gg_status residual(gg_system* S, cudaStream_t st, float* out);

// stats
gg_status stats_compute(gg_system* S, gg_stats_t* out);
// float4 <-> packed float[3] through S->stage, so a host copy is one
// contiguous transfer (the w component on the device is kept).
cudaError_t pack3(gg_system* S, const float4* src, float* dst, int64_t n, cudaStream_t st);
cudaError_t unpack3(gg_system* S, const float* src, float4* dst, int64_t n, cudaStream_t st);

// profiling hooks (system.cu)
void prof_begin(gg_system* S, int cls, cudaStream_t st);
void prof_end(gg_system* S, int cls, int64_t units, cudaStream_t st);

inline int blocks_for(int64_t n, int threads) {
  return (int)((n + threads - 1) / threads);
}

inline void count_launches(gg_system* S, int k) {
  if (S) S->launches += k;
}

}  // namespace gg

/*
 * gg.h — C ABI of the GB300-native granular substep path.
 *
 * This header is the drop-in boundary for the per-substep simulation path of
 * granular_gpu (src/GranularSystem.{hpp,cu}, src/Solver.{hpp,cu},
 * src/Particles.hpp, src/GranularParticles.hpp).  The reference exposes a C++
 * class, not a C ABI; every entry point below names the reference member it
 * replaces.  A header-only C++ class with the reference's shape lives in
 * granular_system.hpp and is built only on these functions.
 *
 * Conventions
 *  - Every call returns a gg_status and never throws across the ABI.  The
 *    message of the last failure on the calling thread is gg_last_error().
 *  - A gg_system owns all of its device memory; the caller owns every host
 *    buffer it passes.  Nothing is allocated on the device after gg_create.
 *  - One CUDA stream per gg_system.  gg_step is asynchronous on that stream;
 *    gg_read / gg_stats / gg_synchronize wait for it.
 *  - One gg_system must not be used from two host threads at once.
 *  - Positions and velocities cross the ABI as packed float[3] per particle,
 *    the reference's float3 layout (src/Particles.hpp:19-20).
 */
#ifndef GG_H
#define GG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GG_ABI_VERSION 2

typedef struct gg_system gg_system;
typedef struct gg_grid gg_grid;

typedef enum gg_status {
  GG_OK = 0,
  GG_ERR_INVALID_ARGUMENT = 1,
  GG_ERR_CUDA = 2,          /* a CUDA runtime call failed */
  GG_ERR_OUT_OF_MEMORY = 3, /* device allocation at create time failed */
  GG_ERR_CAPACITY = 4,      /* splits would exceed max_particles; extras dropped */
  GG_ERR_IO = 5,            /* file could not be opened / read / written */
  GG_ERR_PARSE = 6,         /* scene JSON or snapshot is malformed */
  GG_ERR_NUMERIC = 7,       /* a NaN/Inf position was produced (reported, not fatal) */
  GG_ERR_NOT_SUPPORTED = 8,
  GG_ERR_TIMEOUT = 9        /* a bounded device-side wait gave up */
} gg_status;

/* The three particle sets of src/GranularSystem.hpp:59-61. */
typedef enum gg_set {
  GG_SET_GRANULAR = 0,
  GG_SET_BOUNDARY = 1,
  GG_SET_UPSAMPLED = 2
} gg_set;

/* Per-particle fields readable with gg_read / gg_device_ptr.  Element types
 * are given in brackets.  Fields marked (granular) exist only for that set. */
typedef enum gg_field {
  GG_FIELD_POS = 0,               /* float[3]  get_pos_ptr            Particles.hpp:19   */
  GG_FIELD_VEL = 1,               /* float[3]  get_vel_ptr            Particles.hpp:20   */
  GG_FIELD_MASS = 2,              /* float     get_mass_ptr  (granular) GranularParticles.hpp:21 */
  GG_FIELD_MASS_UNITS = 3,        /* int32     integer mass ledger, 2^-20 of a unit mass (granular) */
  GG_FIELD_SURFACE = 4,           /* int32     get_surface_ptr (granular) GranularParticles.hpp:23 */
  GG_FIELD_SURFACE_DISTANCE = 5,  /* float     get_surface_distance_ptr (granular) :24 */
  GG_FIELD_CELL_KEY = 6,          /* int32     sorted cell key of the last grid build (particle_2_cell) */
  GG_FIELD_PERM = 7,              /* int32     pre-sort index of each sorted slot, last grid build */
  GG_FIELD_CELL_START = 8,        /* int32[C+1] cell start table (granular or boundary) */
  GG_FIELD_REMOVE = 9,            /* int32     Solver::_buffer_remove   (granular) */
  GG_FIELD_MERGE = 10,            /* float     Solver::_buffer_merge    (granular) */
  GG_FIELD_MERGE_COUNT = 11,      /* int32     Solver::_buffer_merge_count (granular) */
  GG_FIELD_MERGE_VELOCITY = 12,   /* float[3]  Solver::_buffer_merge_velocity (granular) */
  GG_FIELD_ADAPTIVE_LAST_STEP = 13, /* int32   get_adaptive_last_step_ptr (granular) */
  GG_FIELD_IS_ANIMATED = 14,      /* int32     get_is_animated_ptr (boundary) */
  GG_FIELD_CONTACTS = 15,         /* int32     contacts found by each particle in the last sweep (granular) */
  GG_FIELD_NUM_CONSTRAINTS = 16,  /* int32     constraint count n_i of the last sweep (granular) */
  GG_FIELD_FEATURES = 17,         /* uint16[48] bf16 warm-start features of the last substep (granular) */
  GG_FIELD_WARM_TARGET = 18       /* float[3]  correction the sweeps reached, x*_final - x*_predict, in
                                     units of |g| dt^2 (granular, warm_start = 2) */
} gg_field;

/*
 * Every constant the reference hard-codes on this path.  gg_default_params
 * fills the reference's values; each field names where the value comes from.
 */
typedef struct gg_params {
  int32_t stab_iters;          /* 3      pre-stabilisation sweeps, Solver.cu:428 */
  int32_t iters;               /* 5      Jacobi sweeps, Solver.cu:99 (max_iter literal) */
  double boundary_radius;      /* 0.01   wall particle radius (a double literal), Solver.cu:283,295,297 */
  float boundary_min_radius;   /* 0.01   floor of the particle radius against walls, Solver.cu:281 */
  double friction_cap;         /* 0.8    tangential cap factor (a double literal), Solver.cu:295,341 */
  float rest_speed;            /* 0.01   speeds below are zeroed, Solver.cu:223 */
  float damp_min_speed;        /* 1.0    Solver.cu:202 */
  float damp_max_speed;        /* 10.0   Solver.cu:203 */
  float damp_min;              /* 0.99   Solver.cu:204 */
  float damp_max;              /* 0.99   Solver.cu:205 */
  float damp_exp_rate;         /* 0.1    expf(-speed*0.1), Solver.cu:236 */
  float adaptive_damp;         /* 0.98   extra damping after a merge/split, Solver.cu:242 */
  float max_mass;              /* 4      GranularSystem.cu:49 */
  float min_merge_mass;        /* 1      merge eligibility mass_i < 1, Solver.cu:542 */
  double merge_radius;         /* 0.035  merge search radius (a double literal), Solver.cu:572,594 */
  float surface_dist_threshold;/* 100    Solver.cu:543,578,610 */
  float target_density;        /* 100    Solver.cu:31 */
  int32_t blend_factor;        /* 40     Solver.hpp:11 */
  float split_min_mass;        /* 2      split needs mass > 2, Solver.cu:795 */
  float surface_cone;          /* 1.047197551  PI_3, GranularSystem.cu:19,598 */
  int32_t surface_min_neighbors; /* 5    GranularSystem.cu:606 */
  float no_surface_distance;   /* 1e5    FLT_MAX redefined, GranularSystem.cu:26 */
  float up_inv_h2;             /* 493.8271605  r_9 = 1/0.045^2, Solver.cu:29 */
  float up_dt;                 /* 0.002  Solver.cu:1260 */
  float up_gravity_y;          /* -9.8   Solver.cu:1259 */
  float up_boundary_radius;    /* 0.015  Solver.cu:1263 */
  float up_repulsion;          /* 3.0    Solver.cu:1264 */
  float up_max_velocity;       /* 7.0    Solver.cu:1339 */
  float up_floor_y;            /* 0.04   Solver.cu:1354 */
  float up_floor_friction;     /* 0.95   Solver.cu:1357 */
  float up_boundary_damping;   /* 0.8    Solver.cu:1325 */
  float up_ground_band;        /* 0.1    Solver.cu:1329 */
  float up_ground_damping;     /* 0.5    Solver.cu:1330 */
  int32_t mass_ledger;         /* 0 = float masses as the reference (Solver.cu:669-671);
                                  1 = exact integer ledger in 2^-20 units */
  int32_t merge_enabled;       /* 1 = merge/split active when is_adaptive */
  int32_t upsample_enabled;    /* 1 = advect upsampled points each substep */
  int32_t math_mode;           /* 0 = CUDA's cbrtf/expf/norm3df/rsqrtf/acosf, the functions the
                                  reference calls; 1 = each evaluated in double and rounded once
                                  to float (matches the CPU restatement bit for bit) */
  float nlist_skin;            /* skin of the per-particle contact lists reused across the sweeps
                                  of a substep: a length; negative (default) = a tenth of the
                                  cell length; 0 = scan the stencil every sweep.  Results do
                                  not depend on it, only the speed and memory (276 bytes per
                                  particle of capacity: 64 candidates and their bookkeeping) do. */
  float target_residual;       /* > 0: after the stabilisation sweeps, Jacobi sweeps run until the
                                  mean penetration over the contacts at x* (particle pairs
                                  r_i + r_j - |x_i - x_j| > 0 and walls), measured before each sweep,
                                  is at most this length, or max_sweeps sweeps have run; `iters` is
                                  then unused.  0 (default): the fixed `iters` sweeps of the
                                  reference.  No counterpart in the reference. */
  int32_t max_sweeps;          /* cap on the Jacobi sweeps of a substep in residual mode (default 200;
                                  stab_iters + max_sweeps is capped at 2048) */
  int32_t warm_start;          /* 0 (default) off; 1 = before the sweeps, add the attached network's
                                  predicted correction to x* (gg_set_warm_start); 2 = record the
                                  features and, after the sweeps, the correction the sweeps reached
                                  (GG_FIELD_FEATURES, GG_FIELD_WARM_TARGET: training data).  No
                                  counterpart in the reference. */
  float warm_start_scale;      /* multiplies the predicted correction (default 1) */
  int32_t merge_cas_lag;       /* 4      the fixed schedule that replaces the race of merge_mark_gpu's
                                  compare-and-swaps (Solver.cu:608-651): warps of 32 consecutive
                                  particles issue them in index order, the lanes of a warp together,
                                  each warp's second CAS (on its partner) merge_cas_lag warps after its
                                  first (on itself).  0 lets every warp finish before the next starts;
                                  larger values merge less.  4 merges about as many pairs as the
                                  reference's own kernel does on a GB300.  0..65536 */
  /* Configured mode: the contact model the benchmark configurations describe
   * and the reference's constants cannot express.  No counterpart in the
   * reference; the defaults keep its behaviour. */
  int32_t contact_law;         /* 0 (default) the reference's contacts: a tangential cap that is
                                  practically inactive (Solver.cu:272-359); 1 = Coulomb friction:
                                  each contact (particle, wall particle or plane) with penetration
                                  depth d also corrects the relative tangential displacement since
                                  the substep began, t: fully when |t| < mu_static d (sticking),
                                  else by min(mu_kinetic d / |t|, 1) (sliding).  Contacts stay
                                  perfectly inelastic (restitution 0: velocities are (x* - x) / dt) */
  float mu_static;             /* static friction coefficient of contact_law 1 (0.5) */
  float mu_kinetic;            /* kinetic friction coefficient of contact_law 1 (0.4) */
  int32_t split_claim;         /* 1 = a split child claims the empty cell it is placed in, the lowest
                                  parent index winning, so two children never land on one point (the
                                  reference lets them, and its contact law then divides by zero);
                                  0 (default) = the reference's split */
  int32_t n_planes;            /* 0..8 analytic walls: particle i keeps planes[k][0..2] . x >=
                                  planes[k][3] + r_i (unit normal, offset); applied in every sweep
                                  after the particle and wall contacts, with contact_law's friction */
  float planes[8][4];
} gg_params;

/* Arguments of GranularSystem::GranularSystem, GranularSystem.hpp:8-14. */
typedef struct gg_desc {
  const float* particles;      /* n_particles x float[3] (required) */
  int64_t n_particles;
  const float* masses;         /* optional n_particles floats; NULL = 1.0 (GranularSystem.cu:57-58) */
  const float* boundary;       /* n_boundary x float[3] (may be NULL if 0) */
  int64_t n_boundary;
  const int32_t* boundary_animated; /* optional n_boundary flags (main.cu:973-975) */
  const float* upsampled;      /* n_upsampled x float[3] (may be NULL if 0) */
  int64_t n_upsampled;
  float space_size[3];
  float cell_length;
  float dt;
  float gravity[3];
  int32_t cell_size[3];
  float density;
  float upsampled_radius;      /* kept for readback only; unused by the step (as in the reference) */
  int32_t is_move_boundary;
  int32_t is_adaptive;
  int32_t skip_initial_step;   /* 0 = the constructor runs one step (GranularSystem.cu:62) */
  int32_t device;              /* CUDA device ordinal */
  int64_t max_particles;       /* granular capacity; 0 = 2 x n_particles.  Capacity, n_upsampled
                                  and n_boundary are each at most 2^31 - 2^16 */
  void* stream;                /* optional cudaStream_t to run on; NULL = own stream */
  gg_params params;
} gg_desc;

/* Scene-JSON overrides for gg_create_from_scene; zero-initialise and set
 * only the fields you want. */
typedef struct gg_overrides {
  int32_t has_params;          /* 1 = use params below instead of the defaults */
  gg_params params;
  int32_t device;
  int64_t max_particles;
  void* stream;
  int32_t skip_initial_step;
  const char* base_dir;        /* directory obj_file paths are resolved against; NULL = cwd */
} gg_overrides;

typedef struct gg_stats_t {
  int64_t n_particles, n_boundary, n_upsampled;
  int64_t steps;               /* completed substeps (including the constructor's) */
  int64_t merged_last;         /* particles removed by the last adaptive step (Solver.cu:1040) */
  int64_t split_last;          /* children appended by the last adaptive step (Solver.cu:1166) */
  int64_t merged_total, split_total;
  double total_mass;           /* FP64 reduction of the float masses */
  int64_t total_mass_units;    /* integer ledger sum (mass_ledger = 1) */
  double momentum[3];          /* FP64 sum of m v */
  double kinetic_energy;       /* FP64 sum of m |v|^2 / 2 */
  double center_of_mass[3];
  float max_penetration;       /* max over particle pairs of r_i+r_j-|x_i-x_j| (>= 0) */
  int32_t nonfinite;           /* particles with a NaN/Inf position */
  int32_t error_word;          /* device error bits (capacity, timeout) since create */
  int64_t launches;            /* kernels this library launched since create */
  int32_t last_sweeps;         /* Jacobi sweeps of the last substep in residual mode */
  float last_residual;         /* mean penetration over contacts at the last check (residual mode) */
  float last_residual_max;     /* largest penetration at the last check (residual mode) */
  int32_t pad_;
} gg_stats_t;

/* Per-kernel-class timing accumulated between gg_profile_begin/_end. */
#define GG_PROF_MAX 24
typedef struct gg_profile_t {
  int32_t n_classes;
  char names[GG_PROF_MAX][24];
  int64_t launches[GG_PROF_MAX];
  double ms[GG_PROF_MAX];
  int64_t units[GG_PROF_MAX];  /* particles (or points) processed, summed over launches */
  int64_t kernel_launches;     /* kernels launched between begin and end */
  int64_t nlist_rebuilds;      /* contact lists built by listed sweeps (a full stencil scan each) */
} gg_profile_t;

int32_t gg_abi_version(void);
/* sizeof(gg_params), sizeof(gg_desc), sizeof(gg_overrides), sizeof(gg_stats_t),
 * sizeof(gg_profile_t), in that order, for binding checks. */
gg_status gg_struct_sizes(int64_t* sizes, int32_t n);
const char* gg_last_error(void);
gg_status gg_default_params(gg_params* out);

/* GranularSystem::GranularSystem (GranularSystem.cu:30-63).  Unlike the
 * reference, the caller's arrays are copied, not moved from. */
gg_status gg_create(const gg_desc* desc, gg_system** out);

/* loadSceneConfig + init_granular_system + the constructor
 * (main.cu:123-167, 746-1173).  Reads the reference's scene-JSON keys. */
gg_status gg_create_from_scene(const char* json_path, const gg_overrides* ov,
                               gg_system** out);

/* Builds a scene's particle sets on the host only (no GPU): the arrays
 * init_granular_system (main.cu:746-1173) would hand to the constructor.
 * Pass NULL buffers to query sizes.  Buffers hold float[3] per particle. */
gg_status gg_scene_build(const char* json_path, const char* base_dir,
                         float* particles, int64_t* n_particles,
                         float* boundary, int32_t* boundary_animated, int64_t* n_boundary,
                         float* upsampled, int64_t* n_upsampled,
                         gg_desc* desc_out);

/* The parameters in use, and a change of them between substeps (for example
 * switching the warm start or the residual mode).  nlist_skin cannot change
 * after gg_create (it sizes the contact lists): a different value returns
 * GG_ERR_NOT_SUPPORTED.  No counterpart in the reference (its constants are
 * compiled in). */
gg_status gg_get_params(gg_system* sys, gg_params* out);
gg_status gg_set_params(gg_system* sys, const gg_params* params);

/* GranularSystem::step (GranularSystem.cu:397-453), n_substeps times.
 * Asynchronous on the system's stream. */
gg_status gg_step(gg_system* sys, int32_t n_substeps);
gg_status gg_synchronize(gg_system* sys);

/* size() / boundary_size() / upsampled_size(), GranularSystem.hpp:21-27. */
gg_status gg_size(gg_system* sys, gg_set set, int64_t* n);
gg_status gg_grid_dims(gg_system* sys, int32_t cell_size[3], float* cell_length);

/* Copies a field to host memory: the cudaMemcpy a caller of get_*_ptr()
 * performs (main.cu:206-209).  capacity = elements (particles, or cells+1 for
 * GG_FIELD_CELL_START) the buffer holds; *n receives the element count. */
gg_status gg_read(gg_system* sys, gg_set set, gg_field field,
                  void* host_dst, int64_t capacity, int64_t* n);

/* Device pointer of a field for zero-copy use (get_*_ptr).  Valid until the
 * next gg_step.  Positions/velocities are float[4] per particle on device
 * (w = radius for positions); *stride_bytes receives the element stride. */
gg_status gg_device_ptr(gg_system* sys, gg_set set, gg_field field,
                        void** dptr, int64_t* n, int32_t* stride_bytes);

/* Headless colour buffer: generate_dots (VBO.hpp:9-71, main.cu:1539-1580)
 * without the OpenGL buffers.  Writes every particle of `set` (GG_SET_GRANULAR
 * or GG_SET_UPSAMPLED) as a packed float[3] position into d_dots and a packed
 * float[3] colour into d_colors (device buffers of at least 3 * size floats
 * each, e.g. a renderer's interop buffers).  mode 0 colours the surface flag,
 * 1 the surface-distance bands, 2 the mass between min_mass and max_mass (the
 * reference runs mode 2 with 1 and 4).  Render points have no mass, surface
 * or distance arrays in the reference beyond zero-filled ones, and are
 * coloured from zeros.  Enqueued on the system's stream (gg_synchronize). */
gg_status gg_color_buffer(gg_system* sys, gg_set set, int32_t mode, float min_mass, float max_mass,
                          float* d_dots, float* d_colors);

/* Overwrites positions/velocities of a set from host float[3] arrays (same
 * count as the set).  Used to start both implementations from one state. */
gg_status gg_write(gg_system* sys, gg_set set, gg_field field,
                   const void* host_src, int64_t n);

/* Binary snapshot of the full state (all sets, solver buffers, counters). */
gg_status gg_save(gg_system* sys, const char* path);
gg_status gg_load(gg_system* sys, const char* path);

gg_status gg_stats(gg_system* sys, gg_stats_t* out);

/* Solver::save_particle_stats (Solver.cu:1444-1462): writes the per-step
 * "Frame,MergedParticles,SplitParticles,TotalParticles" CSV. */
gg_status gg_save_particle_stats(gg_system* sys, const char* path);

/* ASCII VTK point cloud of one set's positions, as the reference's writers
 * produce it (saveFunnelUpsampledPositionsToVTK, main.cu:190-254): NaN
 * positions are dropped and, with swap_yz, points are written "x z y". */
gg_status gg_write_vtk(gg_system* sys, gg_set set, const char* path, int32_t swap_yz);

/* The reference's other frame writers (main.cu:256-694), ASCII VTK point
 * clouds written "x z y" like gg_write_vtk:
 *   gg_write_vtk_centered           saveUpsampledPositionsToVTK (:588-664): the
 *                                   set's valid points centred on their centroid,
 *                                   the lowest lifted to y = 0;
 *   gg_write_vtk_by_mass            saveParticlesByMass (:256-368): the particles,
 *                                   centred, into <base>_mass_light|_medium|_heavy/
 *                                   <frame_id>.vtk (mass < 2, 2..3, above);
 *   gg_write_vtk_animated_boundary  saveFunnelBoundaryParticlesToVTK (:370-432,
 *                                   centred = 0) / saveBoundaryParticlesToVTK
 *                                   (:434-527, centred on the render points);
 *   gg_write_vtk_points_centered    saveAdditionalBoundaryParticlesToVTK
 *                                   (:529-586): caller points (float[3]), centred
 *                                   on the render points;
 *   gg_write_csv                    saveUpsampledPositionsToCSV (:673-694): "x,y,z";
 *   gg_write_frame_times            saveFrameTimes (:665-671).
 * Writers that find nothing to write leave an empty file, as the reference's. */
gg_status gg_write_vtk_centered(gg_system* sys, gg_set set, const char* path);
gg_status gg_write_vtk_by_mass(gg_system* sys, const char* base, int32_t frame_id);
gg_status gg_write_vtk_animated_boundary(gg_system* sys, const char* path, int32_t centred);
gg_status gg_write_vtk_points_centered(gg_system* sys, const float* points3, int64_t n, const char* path);
gg_status gg_write_csv(gg_system* sys, gg_set set, const char* path);
gg_status gg_write_frame_times(gg_system* sys, const char* path);

/* GranularSystem::get_frame_times (GranularSystem.hpp:48): per-step device
 * milliseconds, recorded when timing is enabled. */
gg_status gg_set_frame_timing(gg_system* sys, int32_t enabled);
gg_status gg_frame_times(gg_system* sys, float* host_dst, int64_t capacity, int64_t* n);

/* Solver::trigger_explosion (Solver.cu:1411-1442). */
gg_status gg_trigger_explosion(gg_system* sys, float explosion_force);

/* ------------------------------------------------ animated walls
 *
 * The excavator's bucket: wall particles flagged is_animated move by
 * updateAnimation (main.cu:1210-1277) once per frame, before the frame's
 * substeps: a translation for the first 2.5 s, then a rotation about the z
 * axis until 45 degrees are turned.  gg_step re-grids the walls every
 * substep when the system was created with is_move_boundary
 * (GranularSystem.cu:402-404). */

/* AnimationState (main.cu:100-111), field for field. */
typedef struct gg_animation {
  int32_t is_animating;
  float animation_time;             /* seconds in the current phase */
  int32_t start_index;              /* wall index range whose centroid becomes */
  int32_t num_particles;            /*   the rotation centre (main.cu:1236-1239) */
  float translation_direction[3];   /* (-0.1, 0, 0) */
  float translation_speed;          /* 5 */
  int32_t translation_complete;
  float rotation_angle;             /* degrees turned so far */
  float rotation_speed;             /* degrees per second, 90 */
  float rotation_center[3];
} gg_animation;

/* One frame's move as updateAnimation decides it: the arguments of
 * animateParticles (main.cu:1175-1208), and whether it runs. */
typedef struct gg_animation_move {
  float translation[3];
  float rotation;                   /* degrees about z through center; 0 = none */
  float center[3];
  int32_t apply;
} gg_animation_move;

/* The initialisers of AnimationState (not animating). */
gg_status gg_default_animation(gg_animation* out);

/* The state the scene construction leaves (main.cu:925-960 for the
 * excavator, 1020-1034 for the funnel): animating, with the range of the
 * walls read from obj_file, when that file exists; else the defaults. */
gg_status gg_scene_animation(const char* json_path, const char* base_dir, gg_animation* out);

/* 1 when gg_animation_advance(a, dt, ...) ends the translation phase and so
 * needs the walls' positions for the rotation centre. */
int32_t gg_animation_needs_centroid(const gg_animation* a, float dt);

/* updateAnimation's host part on the state alone: advances *a by dt and
 * returns the frame's move.  walls (float[3] per wall particle, in the
 * system's current wall order, as the reference reads them back) is read
 * only when gg_animation_needs_centroid says so; then the range
 * [start_index, start_index + num_particles) must lie inside n_walls. */
gg_status gg_animation_advance(gg_animation* a, float dt, const float* walls, int64_t n_walls,
                               gg_animation_move* out);

/* animateParticles (main.cu:1175-1208): moves the flagged wall particles
 * on the device.  cos and sin follow the system's math_mode (0: CUDA's
 * cosf/sinf as the reference; 1: rounded once from double). */
gg_status gg_animate_walls(gg_system* sys, const gg_animation_move* move);

/* updateAnimation (main.cu:1210-1277): advance, reading the walls back
 * when the centroid is needed, then animate the walls if the move applies. */
gg_status gg_update_animation(gg_system* sys, gg_animation* a, float dt);

/* Per-kernel-class timing with CUDA events on the system's stream. */
gg_status gg_profile_begin(gg_system* sys);
gg_status gg_profile_end(gg_system* sys, gg_profile_t* out);

/* The system's cudaStream_t, for callers that time or order work on it. */
gg_status gg_stream(gg_system* sys, void** stream);

void gg_destroy(gg_system* sys);

/*
 * Stand-alone grid build on caller-supplied positions (device-resident
 * scratch owned by a gg_grid).  Replaces the hash / sort_by_key / count /
 * exclusive_scan sequence of neighbor_search_granular
 * (GranularSystem.cu:65-173, CUDAFunctions.cuh:54-107) for parity tests of
 * keys, sorted order and cell ranges on arbitrary inputs.
 */
gg_status gg_grid_create(int32_t device, int64_t capacity, const int32_t cell_size[3],
                         float cell_length, gg_grid** out);
/* pos: n x float[3] host.  Outputs (host, may be NULL): keys[n] (unsorted
 * keys of the input order), sorted_keys[n], perm[n], cell_start[C+1]. */
gg_status gg_grid_build(gg_grid* g, const float* pos, int64_t n,
                        int32_t* keys, int32_t* sorted_keys, int32_t* perm,
                        int32_t* cell_start);
void gg_grid_destroy(gg_grid* g);

/*
 * Grid build that allocates nothing.  This entry point has no counterpart in
 * the reference.  It is for callers that cannot call cudaMalloc: code hosted
 * in an engine or framework that owns every device allocation through its
 * own pool, or a loop that must not allocate once it is running.  Such a
 * caller hands over device buffers it already owns:
 *   d_pos         n x float[3] positions (device)
 *   d_sorted_keys n cell keys in stable sorted order (device, written)
 *   d_perm        n pre-sort indices of the sorted slots (device, written)
 *   d_cell_start  C+1 cell start offsets, C = product of cell_size (device, written)
 * The results equal gg_grid_build's.  The sort's scratch memory is a fixed
 * array inside the library, sized for at most 262,144 particles and
 * 16,777,216 cells; larger inputs return GG_ERR_CAPACITY with a message.
 * Every GPU that loads the library keeps that array (about 4.1 MiB) until
 * the process exits.
 *   - The first call on a device looks up the array's device address; make
 *     that first call before any stream capture on that device.
 *   - Work is queued on `stream` (NULL: the legacy default stream) and the
 *     call returns without waiting.
 *   - The call makes `device` current while it queues the work and puts the
 *     calling thread's previous current device back before it returns, on
 *     every path, errors included.
 *   - All calls on a device share the one array: calls whose work overlaps
 *     on the GPU (other streams, other host threads) race and must be
 *     serialised by the caller.
 */
gg_status gg_grid_build_noalloc(int32_t device, const float* d_pos, int64_t n,
                                const int32_t cell_size[3], float cell_length,
                                uint32_t* d_sorted_keys, uint32_t* d_perm,
                                int32_t* d_cell_start, void* stream);

/*
 * Batched scenes.  No counterpart in the reference (one scene per
 * GranularSystem there).  A batch is one system whose particles and walls
 * hold many independent scenes side by side along x: scene k occupies the
 * slab k*width <= x < (k+1)*width, its box walls inside the slab, with at
 * least one empty cell between neighbouring boxes so that no contact
 * crosses scenes.  One grid, one sort and one launch of each kernel then
 * step every scene.
 */
/* Declares the slabs; friction_cap (optional, n_scenes values) replaces
 * gg_params.friction_cap per scene.  With slabs declared, the analytic
 * walls of gg_params.planes are in each scene's own coordinates (x less
 * k*width for scene k). */
gg_status gg_set_scenes(gg_system* sys, int32_t n_scenes, float width, const float* friction_cap);
/* Configured mode in a batch: Coulomb coefficients per scene (n_scenes
 * values each, after gg_set_scenes with the same n_scenes), replacing
 * gg_params.mu_static / mu_kinetic; NULL for both clears them. */
gg_status gg_set_scene_coulomb(gg_system* sys, int32_t n_scenes, const float* mu_static, const float* mu_kinetic);
/* FP64 per-scene diagnostics, 9 doubles per scene: particle count, mass,
 * momentum x y z, kinetic energy, centre of mass x y z. */
gg_status gg_scene_stats(gg_system* sys, double* host_out, int32_t n_scenes);
/* Captures n_substeps substeps (an even number: the graph replays fixed
 * addresses of the double-buffered arrays) into a CUDA graph on the
 * system's stream (no merge/split, residual mode, moving walls, profiling
 * or frame timing), to be replayed by gg_graph_launch, asynchronously, as
 * often as wanted. */
gg_status gg_graph_capture(gg_system* sys, int32_t n_substeps);
gg_status gg_graph_launch(gg_system* sys);

/* Launch shapes chosen by gg_autotune. */
typedef struct gg_tuning {
  int32_t predict_threads, apply_threads, finalize_threads; /* threads per block */
  int32_t keep_threads;        /* threads per block of the contact-list sweep */
  int32_t build_blocks_per_sm; /* resident blocks per SM of the list-rebuild sweep */
  int32_t trials;              /* timed trials run */
  float ms_default, ms_tuned;  /* device ms of `substeps` substeps with the shapes before and after */
  int32_t sweep_variant;       /* default sweep: 0 contact lists, 1 pruned stencil sweep (same bits) */
  int32_t pad_;
} gg_tuning;
/* Times `substeps` substeps for each candidate launch shape of the
 * substep's tunable kernels and for the default sweep's variant, one choice
 * at a time, every trial from the same saved state (restored afterwards: the
 * system is left as it was, merge/split counters included), and keeps the
 * fastest.  Not in residual mode; call before gg_graph_capture.  Allocates a
 * device copy of the state while it runs. */
gg_status gg_autotune(gg_system* sys, int32_t substeps, gg_tuning* out);
/* The launch shapes in use, and setting them directly, for example to apply
 * shapes an earlier gg_autotune chose on the same workload without timing
 * again.  Results do not depend on them.  gg_set_tuning checks every field
 * (threads per block a multiple of 32 in 32..1024, blocks per SM 1..32,
 * sweep_variant 0 or 1) and ignores trials, ms_default and ms_tuned. */
gg_status gg_get_tuning(gg_system* sys, gg_tuning* out);
gg_status gg_set_tuning(gg_system* sys, const gg_tuning* tuning);

/*
 * Learned warm start.  No counterpart in the reference: a 48 -> 64 -> 64 -> 3
 * MLP (ReLU, BF16 weights on the tensor cores, FP32 accumulation) that
 * predicts a substep's Jacobi position correction from per-particle
 * neighbourhood features (gg_params.warm_start).  Feature and target
 * buffers are device memory: features n x 48 bf16 row-major (16-byte
 * aligned), targets and outputs n x 3 float, in units of |g| dt^2.
 */
typedef struct gg_mlp gg_mlp;
/* He-uniform initial weights from `seed`, zero biases. */
gg_status gg_mlp_create(int32_t device, uint64_t seed, gg_mlp** out);
/* Parameters as one fp32 vector: W1[48][64] b1[64] W2[64][64] b2[64] W3[64][3] b3[3]. */
int64_t gg_mlp_num_params(void);
gg_status gg_mlp_set_params(gg_mlp* mlp, const float* host_params, int64_t n);
gg_status gg_mlp_get_params(gg_mlp* mlp, float* host_params, int64_t n);
/* Prediction for n feature rows; waits for the result. */
gg_status gg_mlp_forward(gg_mlp* mlp, const void* d_features, int64_t n, float* d_out, void* stream);
/* Mean squared error over n samples and its gradient (same layout as the
 * parameters), copied to host buffers (either may be NULL). */
gg_status gg_mlp_gradient(gg_mlp* mlp, const void* d_features, const float* d_targets, int64_t n,
                          float* host_grad, float* host_loss, void* stream);
/* One Adam step (beta 0.9/0.999) on the gradient of n samples. */
gg_status gg_mlp_train_step(gg_mlp* mlp, const void* d_features, const float* d_targets, int64_t n, float lr,
                            float weight_decay, float* host_loss, void* stream);
void gg_mlp_destroy(gg_mlp* mlp);
/* Diagnostic of the failure path of the tensor-core kernels: one block
 * waits, with their bounded mbarrier wait, for a phase that nothing
 * completes.  Returns GG_ERR_TIMEOUT when the wait gave up after `polls`
 * polls (1..2^20, about 0.2 us each) and the error word recorded it, as it
 * must; the device stays usable.  No counterpart in the reference. */
gg_status gg_selftest_bounded_wait(int32_t device, int32_t polls);
/* Attaches a network to a system for gg_params.warm_start = 1 (mlp may be
 * NULL for warm_start = 2) and allocates the warm-start buffers (feature,
 * predicted-position and target arrays: 124 bytes per particle of
 * capacity).  The network must outlive its use by the system. */
gg_status gg_set_warm_start(gg_system* sys, gg_mlp* mlp);

#ifdef __cplusplus
}
#endif

#endif /* GG_H */

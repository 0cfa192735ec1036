"""ctypes mirror of include/gg.h (the C ABI of libgg.so).

Struct layouts here must match the header field for field; the CPU test
suite checks sizeof() of each against the library's own report.
"""
import ctypes as C
import os

GG_OK = 0
GG_ERR_INVALID_ARGUMENT = 1
GG_ERR_CUDA = 2
GG_ERR_OUT_OF_MEMORY = 3
GG_ERR_CAPACITY = 4
GG_ERR_IO = 5
GG_ERR_PARSE = 6
GG_ERR_NUMERIC = 7
GG_ERR_NOT_SUPPORTED = 8
GG_ERR_TIMEOUT = 9

STATUS_NAMES = {
    0: "GG_OK", 1: "GG_ERR_INVALID_ARGUMENT", 2: "GG_ERR_CUDA",
    3: "GG_ERR_OUT_OF_MEMORY", 4: "GG_ERR_CAPACITY", 5: "GG_ERR_IO",
    6: "GG_ERR_PARSE", 7: "GG_ERR_NUMERIC", 8: "GG_ERR_NOT_SUPPORTED",
    9: "GG_ERR_TIMEOUT",
}

SET_GRANULAR, SET_BOUNDARY, SET_UPSAMPLED = 0, 1, 2

FIELD_POS = 0
FIELD_VEL = 1
FIELD_MASS = 2
FIELD_MASS_UNITS = 3
FIELD_SURFACE = 4
FIELD_SURFACE_DISTANCE = 5
FIELD_CELL_KEY = 6
FIELD_PERM = 7
FIELD_CELL_START = 8
FIELD_REMOVE = 9
FIELD_MERGE = 10
FIELD_MERGE_COUNT = 11
FIELD_MERGE_VELOCITY = 12
FIELD_ADAPTIVE_LAST_STEP = 13
FIELD_IS_ANIMATED = 14
FIELD_CONTACTS = 15
FIELD_NUM_CONSTRAINTS = 16
FIELD_FEATURES = 17
FIELD_WARM_TARGET = 18

# (numpy dtype name, components) of each field
FIELD_LAYOUT = {
    FIELD_POS: ("float32", 3), FIELD_VEL: ("float32", 3),
    FIELD_MASS: ("float32", 1), FIELD_MASS_UNITS: ("int32", 1),
    FIELD_SURFACE: ("int32", 1), FIELD_SURFACE_DISTANCE: ("float32", 1),
    FIELD_CELL_KEY: ("int32", 1), FIELD_PERM: ("int32", 1),
    FIELD_CELL_START: ("int32", 1), FIELD_REMOVE: ("int32", 1),
    FIELD_MERGE: ("float32", 1), FIELD_MERGE_COUNT: ("int32", 1),
    FIELD_MERGE_VELOCITY: ("float32", 3), FIELD_ADAPTIVE_LAST_STEP: ("int32", 1),
    FIELD_IS_ANIMATED: ("int32", 1), FIELD_CONTACTS: ("int32", 1),
    FIELD_NUM_CONSTRAINTS: ("int32", 1), FIELD_FEATURES: ("uint16", 48),
    FIELD_WARM_TARGET: ("float32", 3),
}

UNITS_PER_MASS = 1 << 20


class gg_params(C.Structure):
    _fields_ = [
        ("stab_iters", C.c_int32), ("iters", C.c_int32),
        ("boundary_radius", C.c_double), ("boundary_min_radius", C.c_float),
        ("friction_cap", C.c_double), ("rest_speed", C.c_float),
        ("damp_min_speed", C.c_float), ("damp_max_speed", C.c_float),
        ("damp_min", C.c_float), ("damp_max", C.c_float),
        ("damp_exp_rate", C.c_float), ("adaptive_damp", C.c_float),
        ("max_mass", C.c_float), ("min_merge_mass", C.c_float),
        ("merge_radius", C.c_double), ("surface_dist_threshold", C.c_float),
        ("target_density", C.c_float), ("blend_factor", C.c_int32),
        ("split_min_mass", C.c_float), ("surface_cone", C.c_float),
        ("surface_min_neighbors", C.c_int32), ("no_surface_distance", C.c_float),
        ("up_inv_h2", C.c_float), ("up_dt", C.c_float), ("up_gravity_y", C.c_float),
        ("up_boundary_radius", C.c_float), ("up_repulsion", C.c_float),
        ("up_max_velocity", C.c_float), ("up_floor_y", C.c_float),
        ("up_floor_friction", C.c_float), ("up_boundary_damping", C.c_float),
        ("up_ground_band", C.c_float), ("up_ground_damping", C.c_float),
        ("mass_ledger", C.c_int32), ("merge_enabled", C.c_int32),
        ("upsample_enabled", C.c_int32), ("math_mode", C.c_int32), ("nlist_skin", C.c_float),
        ("target_residual", C.c_float), ("max_sweeps", C.c_int32), ("warm_start", C.c_int32),
        ("warm_start_scale", C.c_float), ("merge_cas_lag", C.c_int32),
        ("contact_law", C.c_int32), ("mu_static", C.c_float), ("mu_kinetic", C.c_float),
        ("split_claim", C.c_int32), ("n_planes", C.c_int32), ("planes", (C.c_float * 4) * 8),
    ]


def default_params() -> gg_params:
    """The reference's hard-coded constants (see the comments in gg.h)."""
    p = gg_params()
    p.stab_iters, p.iters = 3, 5
    p.boundary_radius, p.boundary_min_radius, p.friction_cap = 0.01, 0.01, 0.8
    p.rest_speed, p.damp_min_speed, p.damp_max_speed = 0.01, 1.0, 10.0
    p.damp_min, p.damp_max, p.damp_exp_rate, p.adaptive_damp = 0.99, 0.99, 0.1, 0.98
    p.max_mass, p.min_merge_mass, p.merge_radius = 4.0, 1.0, 0.035
    p.surface_dist_threshold, p.target_density, p.blend_factor = 100.0, 100.0, 40
    p.split_min_mass, p.surface_cone, p.surface_min_neighbors = 2.0, 1.047197551, 5
    p.no_surface_distance = 100000.0
    p.up_inv_h2, p.up_dt, p.up_gravity_y = 493.8271605, 0.002, -9.8
    p.up_boundary_radius, p.up_repulsion, p.up_max_velocity = 0.015, 3.0, 7.0
    p.up_floor_y, p.up_floor_friction, p.up_boundary_damping = 0.04, 0.95, 0.8
    p.up_ground_band, p.up_ground_damping = 0.1, 0.5
    p.mass_ledger, p.merge_enabled, p.upsample_enabled = 0, 1, 1
    p.math_mode = 0
    p.nlist_skin = -1.0
    p.target_residual, p.max_sweeps, p.warm_start, p.warm_start_scale = 0.0, 200, 0, 1.0
    p.merge_cas_lag = 4
    p.contact_law, p.mu_static, p.mu_kinetic, p.split_claim, p.n_planes = 0, 0.5, 0.4, 0, 0
    return p


class gg_desc(C.Structure):
    _fields_ = [
        ("particles", C.POINTER(C.c_float)), ("n_particles", C.c_int64),
        ("masses", C.POINTER(C.c_float)),
        ("boundary", C.POINTER(C.c_float)), ("n_boundary", C.c_int64),
        ("boundary_animated", C.POINTER(C.c_int32)),
        ("upsampled", C.POINTER(C.c_float)), ("n_upsampled", C.c_int64),
        ("space_size", C.c_float * 3), ("cell_length", C.c_float), ("dt", C.c_float),
        ("gravity", C.c_float * 3), ("cell_size", C.c_int32 * 3),
        ("density", C.c_float), ("upsampled_radius", C.c_float),
        ("is_move_boundary", C.c_int32), ("is_adaptive", C.c_int32),
        ("skip_initial_step", C.c_int32), ("device", C.c_int32),
        ("max_particles", C.c_int64), ("stream", C.c_void_p),
        ("params", gg_params),
    ]


class gg_overrides(C.Structure):
    _fields_ = [
        ("has_params", C.c_int32), ("params", gg_params), ("device", C.c_int32),
        ("max_particles", C.c_int64), ("stream", C.c_void_p),
        ("skip_initial_step", C.c_int32), ("base_dir", C.c_char_p),
    ]


class gg_stats_t(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int64), ("n_boundary", C.c_int64), ("n_upsampled", C.c_int64),
        ("steps", C.c_int64), ("merged_last", C.c_int64), ("split_last", C.c_int64),
        ("merged_total", C.c_int64), ("split_total", C.c_int64),
        ("total_mass", C.c_double), ("total_mass_units", C.c_int64),
        ("momentum", C.c_double * 3), ("kinetic_energy", C.c_double),
        ("center_of_mass", C.c_double * 3), ("max_penetration", C.c_float),
        ("nonfinite", C.c_int32), ("error_word", C.c_int32), ("launches", C.c_int64),
        ("last_sweeps", C.c_int32), ("last_residual", C.c_float), ("last_residual_max", C.c_float),
        ("pad_", C.c_int32),
    ]


class gg_tuning(C.Structure):
    _fields_ = [("predict_threads", C.c_int32), ("apply_threads", C.c_int32), ("finalize_threads", C.c_int32),
                ("keep_threads", C.c_int32), ("build_blocks_per_sm", C.c_int32), ("trials", C.c_int32),
                ("ms_default", C.c_float), ("ms_tuned", C.c_float), ("sweep_variant", C.c_int32),
                ("pad_", C.c_int32)]


GG_PROF_MAX = 24


class gg_profile_t(C.Structure):
    _fields_ = [
        ("n_classes", C.c_int32), ("names", (C.c_char * 24) * GG_PROF_MAX),
        ("launches", C.c_int64 * GG_PROF_MAX), ("ms", C.c_double * GG_PROF_MAX),
        ("units", C.c_int64 * GG_PROF_MAX), ("kernel_launches", C.c_int64),
        ("nlist_rebuilds", C.c_int64),
    ]


class gg_animation(C.Structure):
    _fields_ = [("is_animating", C.c_int32), ("animation_time", C.c_float), ("start_index", C.c_int32),
                ("num_particles", C.c_int32), ("translation_direction", C.c_float * 3),
                ("translation_speed", C.c_float), ("translation_complete", C.c_int32),
                ("rotation_angle", C.c_float), ("rotation_speed", C.c_float), ("rotation_center", C.c_float * 3)]


class gg_animation_move(C.Structure):
    _fields_ = [("translation", C.c_float * 3), ("rotation", C.c_float), ("center", C.c_float * 3),
                ("apply", C.c_int32)]


# name -> (restype, argtypes) of every function gg.h declares
P_ = C.c_void_p
SIGNATURES = {
    "gg_abi_version": (C.c_int32, []),
    "gg_last_error": (C.c_char_p, []),
    "gg_default_params": (C.c_int, [C.POINTER(gg_params)]),
    "gg_create": (C.c_int, [C.POINTER(gg_desc), C.POINTER(P_)]),
    "gg_create_from_scene": (C.c_int, [C.c_char_p, C.POINTER(gg_overrides), C.POINTER(P_)]),
    "gg_scene_build": (C.c_int, [C.c_char_p, C.c_char_p,
                                 C.POINTER(C.c_float), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_float), C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_float), C.POINTER(C.c_int64),
                                 C.POINTER(gg_desc)]),
    "gg_step": (C.c_int, [P_, C.c_int32]),
    "gg_synchronize": (C.c_int, [P_]),
    "gg_size": (C.c_int, [P_, C.c_int, C.POINTER(C.c_int64)]),
    "gg_grid_dims": (C.c_int, [P_, C.POINTER(C.c_int32), C.POINTER(C.c_float)]),
    "gg_read": (C.c_int, [P_, C.c_int, C.c_int, P_, C.c_int64, C.POINTER(C.c_int64)]),
    "gg_device_ptr": (C.c_int, [P_, C.c_int, C.c_int, C.POINTER(P_), C.POINTER(C.c_int64),
                                C.POINTER(C.c_int32)]),
    "gg_write": (C.c_int, [P_, C.c_int, C.c_int, P_, C.c_int64]),
    "gg_save": (C.c_int, [P_, C.c_char_p]),
    "gg_load": (C.c_int, [P_, C.c_char_p]),
    "gg_stats": (C.c_int, [P_, C.POINTER(gg_stats_t)]),
    "gg_save_particle_stats": (C.c_int, [P_, C.c_char_p]),
    "gg_write_vtk": (C.c_int, [P_, C.c_int, C.c_char_p, C.c_int32]),
    "gg_set_frame_timing": (C.c_int, [P_, C.c_int32]),
    "gg_frame_times": (C.c_int, [P_, C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_int64)]),
    "gg_trigger_explosion": (C.c_int, [P_, C.c_float]),
    "gg_default_animation": (C.c_int, [C.POINTER(gg_animation)]),
    "gg_scene_animation": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(gg_animation)]),
    "gg_animation_needs_centroid": (C.c_int32, [C.POINTER(gg_animation), C.c_float]),
    "gg_animation_advance": (C.c_int, [C.POINTER(gg_animation), C.c_float, C.POINTER(C.c_float), C.c_int64,
                                       C.POINTER(gg_animation_move)]),
    "gg_animate_walls": (C.c_int, [P_, C.POINTER(gg_animation_move)]),
    "gg_update_animation": (C.c_int, [P_, C.POINTER(gg_animation), C.c_float]),
    "gg_profile_begin": (C.c_int, [P_]),
    "gg_profile_end": (C.c_int, [P_, C.POINTER(gg_profile_t)]),
    "gg_stream": (C.c_int, [P_, C.POINTER(P_)]),
    "gg_destroy": (None, [P_]),
    "gg_grid_create": (C.c_int, [C.c_int32, C.c_int64, C.POINTER(C.c_int32), C.c_float,
                                 C.POINTER(P_)]),
    "gg_grid_build": (C.c_int, [P_, C.POINTER(C.c_float), C.c_int64,
                                C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "gg_grid_destroy": (None, [P_]),
    "gg_grid_build_noalloc": (C.c_int, [C.c_int32, P_, C.c_int64, C.POINTER(C.c_int32), C.c_float,
                                        P_, P_, P_, P_]),
    "gg_struct_sizes": (C.c_int, [C.POINTER(C.c_int64), C.c_int32]),
    "gg_mlp_create": (C.c_int, [C.c_int32, C.c_uint64, C.POINTER(P_)]),
    "gg_mlp_num_params": (C.c_int64, []),
    "gg_mlp_set_params": (C.c_int, [P_, C.POINTER(C.c_float), C.c_int64]),
    "gg_mlp_get_params": (C.c_int, [P_, C.POINTER(C.c_float), C.c_int64]),
    "gg_mlp_forward": (C.c_int, [P_, P_, C.c_int64, P_, P_]),
    "gg_mlp_gradient": (C.c_int, [P_, P_, P_, C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_float), P_]),
    "gg_mlp_train_step": (C.c_int, [P_, P_, P_, C.c_int64, C.c_float, C.c_float, C.POINTER(C.c_float), P_]),
    "gg_mlp_destroy": (None, [P_]),
    "gg_selftest_bounded_wait": (C.c_int, [C.c_int32, C.c_int32]),
    "gg_color_buffer": (C.c_int, [P_, C.c_int, C.c_int32, C.c_float, C.c_float, P_, P_]),
    "gg_write_vtk_centered": (C.c_int, [P_, C.c_int, C.c_char_p]),
    "gg_write_vtk_by_mass": (C.c_int, [P_, C.c_char_p, C.c_int32]),
    "gg_write_vtk_animated_boundary": (C.c_int, [P_, C.c_char_p, C.c_int32]),
    "gg_write_vtk_points_centered": (C.c_int, [P_, P_, C.c_int64, C.c_char_p]),
    "gg_write_csv": (C.c_int, [P_, C.c_int, C.c_char_p]),
    "gg_write_frame_times": (C.c_int, [P_, C.c_char_p]),
    "gg_set_warm_start": (C.c_int, [P_, P_]),
    "gg_get_params": (C.c_int, [P_, C.POINTER(gg_params)]),
    "gg_set_scenes": (C.c_int, [P_, C.c_int32, C.c_float, C.POINTER(C.c_float)]),
    "gg_scene_stats": (C.c_int, [P_, C.POINTER(C.c_double), C.c_int32]),
    "gg_set_scene_coulomb": (C.c_int, [P_, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "gg_graph_capture": (C.c_int, [P_, C.c_int32]),
    "gg_graph_launch": (C.c_int, [P_]),
    "gg_autotune": (C.c_int, [P_, C.c_int32, C.POINTER(gg_tuning)]),
    "gg_get_tuning": (C.c_int, [P_, C.POINTER(gg_tuning)]),
    "gg_set_tuning": (C.c_int, [P_, C.POINTER(gg_tuning)]),
    "gg_set_params": (C.c_int, [P_, C.POINTER(gg_params)]),
}

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libgg.so")


class NativeLibraryMissing(RuntimeError):
    pass


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Loads libgg.so and declares every signature.  Raises (no fallback)
    when the library has not been built."""
    if not os.path.exists(path):
        raise NativeLibraryMissing(
            f"{path} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(there is no CPU fallback)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib

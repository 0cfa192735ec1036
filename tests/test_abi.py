"""The C-ABI library loads and matches include/gg.h (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gg.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-zA-Z_][a-zA-Z0-9_]*\s*\**\s+\**(gg_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("gg_create", "gg_create_from_scene", "gg_step", "gg_size", "gg_read", "gg_device_ptr",
                     "gg_save", "gg_load", "gg_stats", "gg_last_error", "gg_destroy", "gg_grid_build"):
        assert required in names


def test_library_exports_every_declared_symbol():
    lib = gg.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared in gg.h but not exported: {missing}"
    # and the Python binding declares a signature for each
    assert not [n for n in declared_functions() if n not in abi.SIGNATURES]


def test_struct_layouts_match_ctypes():
    sizes = (C.c_int64 * 5)()
    assert gg.lib().gg_struct_sizes(sizes, 5) == 0
    assert list(sizes) == [C.sizeof(abi.gg_params), C.sizeof(abi.gg_desc), C.sizeof(abi.gg_overrides),
                           C.sizeof(abi.gg_stats_t), C.sizeof(abi.gg_profile_t)]


def test_default_params_match():
    p = abi.gg_params()
    assert gg.lib().gg_default_params(C.byref(p)) == 0
    q = abi.default_params()
    for name, _ in abi.gg_params._fields_:
        a, b = getattr(p, name), getattr(q, name)
        if name == "planes":
            assert [list(r) for r in a] == [list(r) for r in b]
        elif isinstance(a, float):
            assert C.c_float(a).value == C.c_float(b).value or a == b, name
        else:
            assert a == b, name
    assert gg.lib().gg_abi_version() == 2


def test_invalid_arguments_are_reported_without_a_gpu():
    lib = gg.lib()
    h = C.c_void_p()
    assert lib.gg_create(None, C.byref(h)) == abi.GG_ERR_INVALID_ARGUMENT
    assert b"null" in lib.gg_last_error()
    d = abi.gg_desc()
    d.n_particles = 1
    assert lib.gg_create(C.byref(d), C.byref(h)) == abi.GG_ERR_INVALID_ARGUMENT
    d.particles = (C.c_float * 3)(0.5, 0.5, 0.5)
    d.cell_length = 0.04
    d.cell_size[0] = d.cell_size[1] = d.cell_size[2] = 0
    assert lib.gg_create(C.byref(d), C.byref(h)) == abi.GG_ERR_INVALID_ARGUMENT
    assert b"cell" in lib.gg_last_error()
    d.cell_size[0] = d.cell_size[1] = d.cell_size[2] = 2048
    assert lib.gg_create(C.byref(d), C.byref(h)) == abi.GG_ERR_INVALID_ARGUMENT
    d.cell_size[0] = d.cell_size[1] = d.cell_size[2] = 4
    d.params = abi.default_params()
    d.params.iters = 100
    assert lib.gg_create(C.byref(d), C.byref(h)) == abi.GG_ERR_INVALID_ARGUMENT
    d.params = abi.default_params()
    # counts past 2^31 - 2^16 (launch grids round up to whole tiles of
    # signed 32-bit indices) are refused before any device work
    limit = (1 << 31) - (1 << 16)
    d.upsampled = d.particles
    d.n_upsampled = limit + 1
    assert lib.gg_create(C.byref(d), C.byref(h)) == abi.GG_ERR_INVALID_ARGUMENT
    assert b"2^31" in lib.gg_last_error()
    d.n_upsampled = 0
    d.max_particles = limit + 1
    assert lib.gg_create(C.byref(d), C.byref(h)) == abi.GG_ERR_INVALID_ARGUMENT
    assert lib.gg_step(None, 1) == abi.GG_ERR_INVALID_ARGUMENT


def test_no_fallback_when_library_missing(tmp_path):
    with pytest.raises(abi.NativeLibraryMissing):
        abi.load_library(str(tmp_path / "libgg.so"))


def test_noalloc_grid_build_checks_its_limits_before_touching_a_gpu():
    """gg_grid_build_noalloc rejects inputs beyond its fixed scratch array
    (262,144 particles, 2^24 cells) with GG_ERR_CAPACITY before any CUDA
    call, so this runs without a GPU; the pointers are never dereferenced."""
    lib = gg.lib()
    cs = (C.c_int32 * 3)(4097, 4096, 1)  # 2^24 + 4096 cells
    rc = lib.gg_grid_build_noalloc(0, C.c_void_p(16), 10, cs, C.c_float(0.1),
                                   C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), None)
    assert rc == abi.GG_ERR_CAPACITY
    assert b"16777216" in lib.gg_last_error()
    cs = (C.c_int32 * 3)(1, 1 << 12, 1 << 12)  # exactly 2^24 cells, one particle too many
    rc = lib.gg_grid_build_noalloc(0, C.c_void_p(16), (1 << 18) + 1, cs, C.c_float(0.1),
                                   C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), None)
    assert rc == abi.GG_ERR_CAPACITY
    assert b"262144" in lib.gg_last_error()


def test_new_entry_points_check_their_arguments_without_a_gpu():
    lib = gg.lib()
    # batched scenes in configured mode, animated walls: null systems and
    # states are refused with a message, before any device work
    mu = (C.c_float * 2)(0.5, 0.6)
    assert lib.gg_set_scene_coulomb(None, 2, mu, mu) == abi.GG_ERR_INVALID_ARGUMENT
    assert b"gg_set_scenes" in lib.gg_last_error()
    assert lib.gg_update_animation(None, None, C.c_float(0.1)) == abi.GG_ERR_INVALID_ARGUMENT
    assert lib.gg_animate_walls(None, None) == abi.GG_ERR_INVALID_ARGUMENT
    assert lib.gg_animation_advance(None, C.c_float(0.1), None, 0, None) == abi.GG_ERR_INVALID_ARGUMENT
    assert lib.gg_default_animation(None) == abi.GG_ERR_INVALID_ARGUMENT
    a = abi.gg_animation()
    assert lib.gg_scene_animation(None, None, C.byref(a)) == abi.GG_ERR_INVALID_ARGUMENT
    assert lib.gg_scene_animation(b"/nonexistent/scene.json", None, C.byref(a)) == abi.GG_ERR_IO
    assert lib.gg_animation_needs_centroid(None, C.c_float(0.1)) == 0
    # a state that is not animating moves nothing and needs nothing
    assert lib.gg_default_animation(C.byref(a)) == abi.GG_OK
    m = abi.gg_animation_move()
    assert lib.gg_animation_advance(C.byref(a), C.c_float(0.1), None, 0, C.byref(m)) == abi.GG_OK
    assert m.apply == 0 and a.animation_time == 0.0

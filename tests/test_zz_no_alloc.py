"""gg_grid_build_noalloc: the grid build for callers that cannot allocate
device memory (it uses a fixed scratch array inside the library).

Its results must equal the allocating gg_grid_build and the CPU oracle on
the same positions, on two calls in a row (the second call reuses the
scratch the first one left behind), up to the array's limits: 262,144
particles and 2^24 cells (25-bit keys, four radix passes, a cell table of
2^24 + 1 entries).  Collected last so that a run stopping at the first
failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import abi
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 1 << 18
MAX_CELLS = 1 << 24


def _positions(n, seed, cell_size, L):
    rng = np.random.default_rng(seed)
    span = np.array(cell_size, np.float32) * np.float32(L)
    pos = (rng.uniform(-0.05, 1.05, (n, 3)) * span).astype(np.float32)  # a few out of the grid
    if n > 100:
        pos[: n // 20] = pos[0]  # many equal keys: stability matters
    return pos


def _noalloc(pos, cell_size, L):
    import torch
    n = pos.shape[0]
    ncell = int(np.prod(cell_size))
    d_pos = torch.from_numpy(pos).cuda()
    keys = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    perm = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    cstart = torch.empty(ncell + 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    cs = (C.c_int32 * 3)(*cell_size)
    rc = gg.lib().gg_grid_build_noalloc(0, C.c_void_p(d_pos.data_ptr()), n, cs, C.c_float(L),
                                        C.c_void_p(keys.data_ptr()), C.c_void_p(perm.data_ptr()),
                                        C.c_void_p(cstart.data_ptr()), None)
    torch.cuda.synchronize()
    assert rc == abi.GG_OK, gg.lib().gg_last_error()
    assert torch.cuda.current_device() == 0
    return keys.cpu().numpy()[:n], perm.cpu().numpy()[:n], cstart.cpu().numpy()


def _check_against_both(pos, cell_size, L):
    n = pos.shape[0]
    g = gg.Grid(max(n, 1), cell_size, L)
    _, sk, pm, cst = g.build(pos)
    g.close()
    _, osk, opm, ocst = orc.grid_build(pos, cell_size, L)
    k2, p2, c2 = _noalloc(pos, cell_size, L)
    assert np.array_equal(k2, sk) and np.array_equal(k2, osk[:n])
    assert np.array_equal(p2, pm) and np.array_equal(p2, opm[:n])
    assert np.array_equal(c2, cst) and np.array_equal(c2, ocst)


def test_noalloc_matches_allocating_build_on_two_calls_in_a_row():
    pytest.importorskip("torch")
    cell_size, L = (40, 23, 31), 0.0404
    for n, seed in ((200_000, 11), (37_123, 12)):
        _check_against_both(_positions(n, seed, cell_size, L), cell_size, L)


def test_noalloc_at_its_particle_limit():
    pytest.importorskip("torch")
    cell_size, L = (64, 32, 48), 0.0202
    _check_against_both(_positions(MAX_PARTICLES, 13, cell_size, L), cell_size, L)


def test_noalloc_at_its_cell_limit_four_radix_passes():
    """2^24 cells: keys run to 2^24 (the out-of-grid key), 25 bits, four
    8-bit passes, and a cell scan over 4,097 tiles."""
    pytest.importorskip("torch")
    cell_size, L = (256, 256, 256), 0.004
    assert int(np.prod(cell_size)) == MAX_CELLS
    for n, seed in ((50_000, 14), (1, 15), (0, 16)):
        _check_against_both(_positions(n, seed, cell_size, L), cell_size, L)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    pytest.importorskip("torch")
    cs = (C.c_int32 * 3)(4, 4, 4)
    rc = gg.lib().gg_grid_build_noalloc(0, C.c_void_p(16), MAX_PARTICLES + 1, cs, C.c_float(0.1),
                                        C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), None)
    assert rc == abi.GG_ERR_CAPACITY
    assert b"262144" in gg.lib().gg_last_error()
    cs = (C.c_int32 * 3)(4097, 4096, 1)  # 2^24 + 4096 cells
    rc = gg.lib().gg_grid_build_noalloc(0, C.c_void_p(16), 10, cs, C.c_float(0.1),
                                        C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), None)
    assert rc == abi.GG_ERR_CAPACITY
    assert b"16777216" in gg.lib().gg_last_error()

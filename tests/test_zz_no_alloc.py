"""gg_grid_build_noalloc: the grid build for callers that cannot allocate
device memory (it uses a fixed scratch array inside the library).

Its results must equal the allocating gg_grid_build on the same positions,
on two calls in a row (the second call reuses the scratch the first one
left behind).  Collected last so that a run stopping at the first failure
has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import abi

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 1 << 18


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
    return keys.cpu().numpy()[:n], perm.cpu().numpy()[:n], cstart.cpu().numpy()


def test_noalloc_matches_allocating_build_on_two_calls_in_a_row():
    pytest.importorskip("torch")
    cell_size, L = (40, 23, 31), 0.0404
    for n, seed in ((200_000, 11), (37_123, 12)):
        pos = _positions(n, seed, cell_size, L)
        g = gg.Grid(n, cell_size, L)
        _, sk, pm, cst = g.build(pos)
        g.close()
        k2, p2, c2 = _noalloc(pos, cell_size, L)
        assert np.array_equal(k2, sk)
        assert np.array_equal(p2, pm)
        assert np.array_equal(c2, cst)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    pytest.importorskip("torch")
    cs = (C.c_int32 * 3)(4, 4, 4)
    rc = gg.lib().gg_grid_build_noalloc(0, C.c_void_p(16), MAX_PARTICLES + 1, cs, C.c_float(0.1),
                                        C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), None)
    assert rc == abi.GG_ERR_CAPACITY
    assert b"262144" in gg.lib().gg_last_error()

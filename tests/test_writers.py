"""The reference's frame writers (main.cu:190-694): the library's files against
the text the restatement in oracle/vtk_oracle.py gives for the same state."""
import os

import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import workloads
from oracle import vtk_oracle as vo


def test_restatement_formats_like_the_reference():
    # no GPU: the text layout and the centring arithmetic
    pts = np.array([[0.5, -0.25, 1.0], [1.5, 0.75, 2.0]], np.float32)
    t = vo.vtk_text("T", pts)
    assert t.splitlines()[:7] == ["# vtk DataFile Version 3.0", "T", "ASCII", "DATASET UNSTRUCTURED_GRID",
                                  "POINTS 2 float", "0.5 1 -0.25", "1.5 2 0.75"]
    c, y0 = vo.centring(pts)
    assert np.array_equal(c, np.array([1.0, 0.25, 1.5], np.float32)) and y0 == np.float32(0.5)
    assert vo.csv_text(pts) == "0.5,-0.25,1\n1.5,0.75,2\n"


@pytest.mark.gpu
def test_frame_writers_match_the_restatement(tmp_path):
    desc = workloads.box_drop(n_side=10, substeps=4, iters=5, adaptive=1, upsample_per=2)
    nb = desc["boundary"].shape[0]
    animated = (np.arange(nb) % 7 == 0).astype(np.int32)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), boundary_animated=animated, device=0)
    s.set_frame_timing(True)
    s.step(60)
    up = s.read(gg.FIELD_POS, gg.SET_UPSAMPLED)
    pos, mass = s.read(gg.FIELD_POS), s.read(gg.FIELD_MASS)
    walls = s.read(gg.FIELD_POS, gg.SET_BOUNDARY)
    anim = s.read(gg.FIELD_IS_ANIMATED, gg.SET_BOUNDARY)
    read = lambda p: open(p).read()

    s.write_vtk_centered(str(tmp_path / "up.vtk"))
    v = vo.valid(up)
    c, y0 = vo.centring(v)
    assert read(tmp_path / "up.vtk") == vo.vtk_text("Upsampled Granular Particles", vo.centre(v, c, y0))

    s.write_vtk_by_mass(str(tmp_path / "frame"), 7)
    want = vo.by_mass(pos, mass)
    assert "light" in want
    for k in ("light", "medium", "heavy"):
        p = tmp_path / f"frame_mass_{k}" / "7.vtk"
        assert os.path.isdir(tmp_path / f"frame_mass_{k}")
        assert (read(p) == want[k]) if k in want else not p.exists(), k

    aw = walls[anim == 1]
    s.write_vtk_animated_boundary(str(tmp_path / "walls_raw.vtk"), centred=False)
    assert read(tmp_path / "walls_raw.vtk") == vo.vtk_text("Animated Boundary Particles", aw)
    s.write_vtk_animated_boundary(str(tmp_path / "walls.vtk"), centred=True)
    assert read(tmp_path / "walls.vtk") == vo.vtk_text("Animated Boundary Particles", vo.centre(aw, c, y0))

    extra = np.array([[0.1, 0.2, 0.3], [0.4, 0.5, 0.6]], np.float32)
    s.write_vtk_points_centered(extra, str(tmp_path / "extra.vtk"))
    assert read(tmp_path / "extra.vtk") == vo.vtk_text("Additional Boundary Particles", vo.centre(extra, c, y0))

    s.write_csv(str(tmp_path / "up.csv"))
    assert read(tmp_path / "up.csv") == vo.csv_text(up)

    s.write_frame_times(str(tmp_path / "frame_times.txt"))
    ft = read(tmp_path / "frame_times.txt").split()
    assert len(ft) == 60 and all(float(x) > 0 for x in ft)
    s.close()

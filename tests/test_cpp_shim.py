"""The header-only C++ shim compiles against gg.h and runs (the run needs a GPU)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build(tmp_path):
    exe = str(tmp_path / "shim_drop")
    lib_dir = os.path.join(ROOT, "granular_gpu_gb300", "_build")
    cmd = ["g++", "-std=c++17", "-O1", f"-I{ROOT}/include", f"-I{CUDA}/include",
           os.path.join(ROOT, "tests", "cpp", "shim_drop.cpp"), "-o", exe, f"-L{lib_dir}", "-lgg",
           f"-Wl,-rpath,{lib_dir}", f"-L{CUDA}/lib64", "-lcudart", f"-Wl,-rpath,{CUDA}/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_and_links(tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_shim_runs_reference_style_caller(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "4"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("step")]
    assert len(lines) == 4
    assert "n=1000" in lines[0] and "up=25000" in lines[0]
    ys = [float(l.split("com_y=")[1]) for l in lines]
    assert ys[-1] < ys[0], "the block falls"
    assert "frames=4" in r.stdout  # frame timing starts after the constructor's step
    assert "dots up_inf=1 p0=(0.000,0.000,1.000)" in r.stdout, r.stdout

"""Build recipe of the reference's own CUDA kernels (TEST INFRASTRUCTURE ONLY).

Compiles the reference's `src/Solver.cu` and `src/GranularSystem.cu` from the
reference checkout, unmodified and where they lie, into device-only cubins
for sm_103a.  Nothing from the reference is copied into this repository: the
outputs go to `oracle/_ref/` only (git-ignored; they travel to the GPU host
with the working tree, which has no reference checkout and therefore uses
the prebuilt files).

  solver.cubin, gsystem.cubin, vbo.cubin   the reference's own device flags
                                           (nvcc defaults: -O3, FMA contraction on)
  *_nofma.cubin                            the same with -fmad=false, so every
                                           operation rounds as written, as in
                                           this library's build
  entries.json                             {cubin: {kernel name: mangled entry}}

`src/VBO.hpp` (the colouring kernel of the vertex buffers) is a header that
only `main.cu` includes; it is compiled through a one-line translation unit
written into `oracle/_ref/` that includes it from the reference checkout.

The entry names are read from `ptxas -v`'s "Compiling entry function" lines.
The host side of the reference (its thrust calls, its `GranularSystem`
orchestration) is not built: `oracle/ref_cuda.py` loads the cubins through
the CUDA driver API and drives the `__global__` kernels itself.
"""
import concurrent.futures as cf
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The reference checkout: GG_REFERENCE_DIR when set, else where this
# container mounts it (absent on the GPU host, which uses the prebuilt files).
REF_ROOT = os.environ.get("GG_REFERENCE_DIR") or "/root/reference"
REF_SRC = os.path.join(REF_ROOT, "src")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")

UNITS = {"solver": "Solver.cu", "gsystem": "GranularSystem.cu", "vbo": "VBO.hpp"}
FLAVOURS = {"": [], "_nofma": ["-fmad=false"]}
ENTRY_RE = re.compile(r"Compiling entry function '(_Z(\d+)([A-Za-z_]\w*?)\w*)' for")


def available() -> bool:
    """True when the reference sources can be compiled here."""
    return all(os.path.exists(os.path.join(REF_SRC, f)) for f in UNITS.values())


def _kernel_name(mangled: str):
    m = re.match(r"_Z(\d+)", mangled)
    if not m:
        return None
    n = int(m.group(1))
    start = m.end()
    return mangled[start:start + n]


def _source(unit: str) -> str:
    """The translation unit of `unit`: the reference's .cu file, or for a
    header a generated file that includes it where it lies."""
    src = os.path.join(REF_SRC, UNITS[unit])
    if src.endswith(".cu"):
        return src
    tu = os.path.join(OUT, f"{unit}_ref.cu")
    with open(tu, "w") as f:
        f.write(f'#include "{src}"\n')
    return tu


def _compile(unit: str, flavour: str):
    src = _source(unit)
    dst = os.path.join(OUT, f"{unit}{flavour}.cubin")
    cmd = [NVCC, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
           "--extended-lambda", "-w", "-Xptxas", "-v", "-I", REF_SRC, *FLAVOURS[flavour], src, "-o", dst]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference cubin build failed: {' '.join(cmd)}\n{r.stderr[-4000:]}")
    entries = {}
    for line in (r.stdout + r.stderr).splitlines():
        m = re.search(r"Compiling entry function '([^']+)'", line)
        if not m:
            continue
        mangled = m.group(1)
        if mangled.startswith(("_ZN3cub", "_ZN6thrust", "_ZN4cuda")):
            continue  # library kernels: not driven by the harness
        name = _kernel_name(mangled)
        if name:
            entries[name] = mangled
    return os.path.basename(dst), entries


def build(verbose: bool = False, force: bool = False) -> bool:
    """Builds the cubins when the reference checkout is present; returns
    whether the prebuilt files exist afterwards."""
    meta = os.path.join(OUT, "entries.json")
    if not available():
        return os.path.exists(meta)
    srcs = [os.path.join(REF_SRC, f) for f in UNITS.values()]
    if not force and os.path.exists(meta) and os.path.getmtime(meta) >= max(
            [os.path.getmtime(s) for s in srcs] + [os.path.getmtime(__file__)]):
        return True
    os.makedirs(OUT, exist_ok=True)
    jobs = [(u, f) for u in UNITS for f in FLAVOURS]
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        results = list(ex.map(lambda uf: _compile(*uf), jobs))
    table = {name: ent for name, ent in results}
    with open(meta, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    if verbose:
        for name, ent in table.items():
            print(name, sorted(ent))
    return True


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))

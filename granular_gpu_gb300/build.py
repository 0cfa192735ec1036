"""Build recipe of libgg.so (the CUDA library behind include/gg.h).

Compiles every translation unit in csrc/ in parallel, for sm_103a only:
  .cu  -> nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -fmad=false
  .cpp -> g++ -O2
and links them with the static CUDA runtime into granular_gpu_gb300/_build/libgg.so.
Host code is compiled with -ffp-contract=off and device code with
-fmad=false, so every floating-point operation rounds as written in the
source (the CPU oracle is compiled the same way).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _newer(dst, srcs):
    if not os.path.exists(dst):
        return False
    t = os.path.getmtime(dst)
    return all(os.path.getmtime(s) <= t for s in srcs)


def _headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "gg.h"))
    return hs


def _compile(src, verbose, extra):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if _newer(obj, [src] + _headers()):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-fmad=false", "-std=c++17",
               "-Xcompiler", "-fPIC,-ffp-contract=off", *extra, "-c", src, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
               f"-I{CUDA}/include", "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    return obj


def build(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    """Builds granular_gpu_gb300/_build/libgg.so; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cu", ".cpp")))
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, extra), srcs))
    lib = os.path.join(OUT, "libgg.so")
    if not _newer(lib, objs):
        cmd = ["g++", "-shared", "-o", lib, *objs, f"-L{CUDA}/lib64", "-lcudart_static",
               "-ldl", "-lpthread", "-lrt"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))

"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/gg_oracle.c twice with gcc:
  oracle/_build/libggoracle32.so  FP32 restatement (the bit-level model)
  oracle/_build/libggoracle64.so  FP64 transcription
-ffp-contract=off keeps x86 and Arm results identical (no fused multiply-add).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")


def build(verbose: bool = False) -> None:
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "gg_oracle.c")
    jobs = []
    for fp64, name in ((0, "libggoracle32.so"), (1, "libggoracle64.so")):
        dst = os.path.join(OUT, name)
        if os.path.exists(dst) and os.path.getmtime(dst) >= max(
                os.path.getmtime(src),
                os.path.getmtime(os.path.join(HERE, "..", "include", "gg.h"))):
            continue
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp",
               "-ffp-contract=off", "-fno-fast-math", f"-DGGO_FP64={fp64}",
               src, "-o", dst, "-lm"]
        if verbose:
            print(" ".join(cmd))
        jobs.append(subprocess.Popen(cmd))
    for j in jobs:
        if j.wait() != 0:
            raise RuntimeError("oracle build failed")


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)

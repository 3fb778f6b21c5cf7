"""Build recipe for the CPU oracle (test infrastructure; never part of the product).

Compiles ``oracle/msm_oracle.c`` with gcc into ``oracle/_build/libmsm_oracle.so``.
``-ffp-contract=off`` keeps x86_64 and aarch64 results identical (no FMA contraction);
OpenMP is used when the compiler offers it, for the multi-core CPU baseline.
The reference itself (CUDA Fortran + PGI host Fortran) cannot be compiled here: no Fortran
compiler exists in this image, so there is no ``oracle/_ref`` build.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmsm_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "msm_oracle.c")
    hdr = os.path.join(HERE, "msm_oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) > max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    base = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
            "-Wno-unknown-pragmas"]
    tmp = LIB + ".tmp"
    cmd = base + ["-fopenmp", src, "-o", tmp, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:  # no libgomp: fall back to a serial build
        cmd = base + [src, "-o", tmp, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))

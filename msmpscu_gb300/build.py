"""Builds libmsmgb.so in-tree: nvcc for sm_103a, one object per translation unit, compiled
in parallel, linked with the CUDA runtime statically.  Output:
``msmpscu_gb300/_build/libmsmgb.so``."""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmsmgb.so")
CU_SOURCES = ["context.cu", "nlist.cu", "force64.cu", "force32.cu", "forceff.cu", "vv.cu", "hvp.cu", "adjoint.cu", "noalloc.cu"]
CPP_SOURCES = ["tables.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmsmgb.so")
    return cand


def _deps():
    files = [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES + ["msmgb_internal.cuh"]]
    files.append(os.path.join(HERE, "..", "include", "msmgb.h"))
    return files


def _compile(src, obj, nvcc, extra):
    if src.endswith(".cu"):
        cmd = [nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
               "-diag-suppress", "1444", "-c", src, "-o", obj, *extra]
    else:
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    deps = _deps()
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) > max(os.path.getmtime(f) for f in deps if os.path.exists(f))):
        return LIB
    nvcc = _nvcc()
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose else []
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        for f in CU_SOURCES + CPP_SOURCES:
            src = os.path.join(CSRC, f)
            obj = os.path.join(objdir, os.path.splitext(f)[0] + ".o")
            jobs.append(ex.submit(_compile, src, obj, nvcc, extra))
        objs = [j.result() for j in jobs]
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-cudart", "static", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))

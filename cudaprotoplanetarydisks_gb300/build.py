"""Build recipe of the product: libfargo_gb300.so and the fargo_gb300 driver.

nvcc -gencode arch=compute_103a,code=sm_103a (sm_103a only), one object per
translation unit compiled in parallel, then one shared library and one
executable linked from the same objects.  Outputs stay in this package
directory (git-ignored), so the library that tests and bench.py load is
in-tree.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfargo_gb300.so")
EXE = os.path.join(HERE, "fargo_gb300")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code is compiled without FMA contraction (GCC contracts by default on
# aarch64), so the FP64 set-up is the same IEEE sequence on x86_64 and on Grace
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
CUFLAGS = ARCH + COMMON + ["--expt-relaxed-constexpr", "-Xptxas", "-O3"]

LIB_SOURCES = ["params.cpp", "setup.cpp", "fargo_kernels.cu", "fargo_sg.cu", "fargo_ctx.cu", "output.cpp",
               "fargo_noalloc.cu", "fargo_batch.cu", "fargo_mlp.cu", "fargo_learned.cu",
               "fargo_force_diag.cu", "fargo_peak.cu", "fargo_tc.cu"]
EXE_SOURCES = ["driver.cpp"]
HEADERS = ["fargo_internal.h", "fargo_device.cuh"]


def _obj(src):
    return os.path.join(OBJ, os.path.splitext(src)[0] + ".o")


def _needs(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    path = os.path.join(CSRC, src)
    obj = _obj(src)
    deps = [path] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "fargo_gb300.h")]
    if not _needs(obj, deps):
        return obj
    flags = CUFLAGS if src.endswith(".cu") else ARCH + COMMON + ["-x", "c++"]
    cmd = [NVCC] + flags + ["-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    return obj


def build(force=False, verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    srcs = [s for s in LIB_SOURCES + EXE_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if force:
        for s in srcs:
            if os.path.exists(_obj(s)):
                os.remove(_obj(s))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = dict(zip(srcs, ex.map(lambda s: _compile(s, verbose), srcs)))
    lib_objs = [objs[s] for s in LIB_SOURCES if s in objs]
    if _needs(LIB, lib_objs):
        cmd = [NVCC] + ARCH + ["-shared", "-Xcompiler", "-fPIC"] + lib_objs + ["-o", LIB + ".tmp", "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    exe_objs = [objs[s] for s in EXE_SOURCES if s in objs]
    if exe_objs and _needs(EXE, exe_objs + lib_objs):
        cmd = [NVCC] + ARCH + exe_objs + lib_objs + ["-o", EXE + ".tmp", "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        os.replace(EXE + ".tmp", EXE)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

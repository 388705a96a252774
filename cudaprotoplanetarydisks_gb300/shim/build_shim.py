"""Recipe: the reference's own host driver linked to this library.

Compiles the reference's host-driver sources -- src/Main.cu, Interpret.cu, Psys.cu,
Output.cu, Theo.cu, Init.cu, LowTasks.cu, taken from the copy the reference's CUDA
recipe generates (oracle/_ref/cuda, git-ignored; oracle/ref_cuda/build_ref_cuda.py)
-- unchanged, with the reference Makefile's flags for sm_103a, plus
reference_shim.cu (the functions and globals those files take from the files the
library replaces), and links them against libfargo_gb300.so, with ReadVariables
wrapped at link time so that the shim learns the .par path.  Output:
cudaprotoplanetarydisks_gb300/shim/fargo_ref_driver_gb300 (git-ignored), run as the
reference's binary is: `echo 0 | fargo_ref_driver_gb300 file.par`.

Built only where that copy of the reference exists; build() returns None otherwise.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
REPO = os.path.dirname(PKG)
REF = os.path.join(REPO, "oracle", "_ref", "cuda")
OBJ = os.path.join(HERE, "_build")
EXE = os.path.join(HERE, "fargo_ref_driver_gb300")
LIB = os.path.join(PKG, "libfargo_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
DRIVER = ["Main", "Interpret", "Psys", "Output", "Theo", "Init", "LowTasks"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(" ".join(cmd) + "\n" + (r.stdout + r.stderr)[-4000:])


def build(force=False):
    src_dir, inc = os.path.join(REF, "src"), os.path.join(REF, "include")
    srcs = [os.path.join(src_dir, f + ".cu") for f in DRIVER]
    if not all(os.path.exists(s) for s in srcs) or not os.path.exists(LIB) or shutil.which("nvcc") is None:
        return None
    shim = os.path.join(HERE, "reference_shim.cu")
    deps = srcs + [shim, LIB, os.path.abspath(__file__), os.path.join(REPO, "include", "fargo_gb300.h")]
    if not force and os.path.exists(EXE) and all(os.path.getmtime(d) <= os.path.getmtime(EXE) for d in deps):
        return EXE
    os.makedirs(OBJ, exist_ok=True)
    jobs, objs = [], []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        jobs.append(["nvcc", "-c", "-w", "-I" + inc, s, "-o", o] + ARCH + ["-Xcompiler", "-fopenmp"])
    o = os.path.join(OBJ, "reference_shim.o")
    objs.append(o)
    jobs.append(["nvcc", "-c", "-w", "-std=c++17", "-I" + inc, "-I" + os.path.join(REPO, "include"), shim, "-o", o]
                + ARCH + ["-Xcompiler", "-fopenmp"])
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    _run(["nvcc"] + objs + ["-o", EXE + ".tmp", "-L" + PKG, "-lfargo_gb300", "-Xlinker", "-rpath=$ORIGIN/..",
                            "-lcuda", "-lcudart", "-lcufft"] + ARCH +
         ["-Xcompiler", "-fopenmp", "-lgomp", "-Xlinker", "--wrap=_Z13ReadVariablesPc"])
    os.replace(EXE + ".tmp", EXE)
    return EXE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

"""Recipe: the reference's own CUDA build for sm_103a (TEST INFRASTRUCTURE and the
reference's GPU baseline; never part of the product).

generate() -- only where the reference tree is (FARGO_REFERENCE_DIR, else a
`reference` directory beside this repository): copies src/*.cu and include/*.cuh
into oracle/_ref/cuda/ (git-ignored, never committed) with the two source-compat
fixes nvcc 13 needs and nothing else:
  * src/Kernels.cu:305  __shfl_down(v, o) -> __shfl_down_sync(0xffffffff, v, o)
    (the mask-less form was removed for sm_70+; the call sits in `if (tid < 32)` of
    a 32-thread block, so all 32 lanes take part);
  * src/Main.cu:556,651  array -> ::array (ambiguous with std::array under the
    reference's `using namespace std`).

build() -- wherever oracle/_ref/cuda/src exists and nvcc is on PATH: compiles each
file as the reference's Makefile does (`nvcc -c -w -Iinclude`, default
optimisation, the Makefile's libraries -lcuda -lcudart -lcufft and OpenMP on the
host) for `-gencode arch=compute_103a,code=sm_103a`, plus two link-time wrappers of
oracle/ref_emul: noise_wrap.cpp (the seeded initial noise of the benchmark
workloads, through --wrap on InitGasDensity / InitGasEnergy) and timing_wrap.cpp
(one `REFSTEP dt substeps seconds` line per AlgoGas call on stderr; AlgoGas
synchronises the device after every launch, so host time is its device time).
Output: oracle/_ref/fargoGPU_sm103a, run as `echo 0 | fargoGPU_sm103a file.par`.

Only configurations whose kernels were read for out-of-bounds access may run on a
GPU: disks with closed (WALL) boundaries and no self-gravity, isothermal (C1) or
adiabatic with cooling and alpha viscosity (C3).  Every kernel on those paths
guards i < nrad, j < nsec and indexes inside its allocation; DeviceReduce never
sees N = 1.  The energy path adds ComputeSoundSpeedKernel, Substep3Kernel
(i > 0), Substep3Kernel2 (i == 0 reads rings 1 and 2; the update guards i < nrad),
ComputeTemperatureFieldKernel and Make1DprofileKernel (i < nrad into an NRAD-long
profile), and the host arrays EnergyMed, SigmaMed, CoolingTimeMed, QplusMed and
viscosity_array_d are NRAD + 1 long (src/Kernels.cu:56-115, 167-215, 610-646;
src/Main.cu:623-630, 729-732; src/SourceEuler.cu:412).  The non-reflecting
boundary (NonReflectingBoundaryKernel2, src/Kernels.cu:575, no j < nsec guard) and
self-gravity (Update_sgvelocityKernel, src/Kernels.cu:930, index -1) are not run.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REPO = os.path.dirname(ORACLE)
EMUL = os.path.join(ORACLE, "ref_emul")
OUT = os.path.join(ORACLE, "_ref", "cuda")
GEN_SRC = os.path.join(OUT, "src")
GEN_INC = os.path.join(OUT, "include")
OBJ = os.path.join(OUT, "build")
EXE = os.path.join(ORACLE, "_ref", "fargoGPU_sm103a")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
WRAPS = ["_Z14InitGasDensityPd", "_Z13InitGasEnergyPd",
         "_Z7AlgoGasP5forcePdS1_S1_S1_S1_P16planetary_systemi", "_Z9TransportPdS_S_S_S_d"]

# (file, line, old text, new text): the only changes to the reference's sources
COMPAT = [
    ("Kernels.cu", 305, "mySum += __shfl_down(mySum, offset);", "mySum += __shfl_down_sync(0xffffffff, mySum, offset);"),
    ("Main.cu", 556, "free(array);", "free(::array);"),
    ("Main.cu", 651, "array           = (double *)malloc", "::array           = (double *)malloc"),
]


def reference_dir():
    d = os.environ.get("FARGO_REFERENCE_DIR") or os.path.join(os.path.dirname(REPO), "reference")
    return d if os.path.isdir(os.path.join(d, "src")) and os.path.isdir(os.path.join(d, "include")) else None


def generate():
    ref = reference_dir()
    if ref is None:
        return False
    os.makedirs(GEN_SRC, exist_ok=True)
    os.makedirs(GEN_INC, exist_ok=True)
    for f in sorted(os.listdir(os.path.join(ref, "src"))):
        if not f.endswith(".cu"):
            continue
        lines = open(os.path.join(ref, "src", f)).read().split("\n")
        for name, line, old, new in COMPAT:
            if name == f:
                assert old in lines[line - 1], (f, line, lines[line - 1])
                lines[line - 1] = lines[line - 1].replace(old, new)
        text = "\n".join(lines)
        dst = os.path.join(GEN_SRC, f)
        if not (os.path.exists(dst) and open(dst).read() == text):
            with open(dst, "w") as g:
                g.write(text)
    for f in sorted(os.listdir(os.path.join(ref, "include"))):
        if f.endswith(".cuh"):
            src, dst = os.path.join(ref, "include", f), os.path.join(GEN_INC, f)
            if not (os.path.exists(dst) and open(dst).read() == open(src).read()):
                shutil.copyfile(src, dst)
    return True


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(" ".join(cmd) + "\n" + (r.stdout + r.stderr)[-4000:])


def build(force=False):
    generate()
    if not os.path.isdir(GEN_SRC) or shutil.which("nvcc") is None:
        return None
    srcs = sorted(os.path.join(GEN_SRC, f) for f in os.listdir(GEN_SRC) if f.endswith(".cu"))
    if not srcs:
        return None
    own = [os.path.join(EMUL, "noise_wrap.cpp"), os.path.join(EMUL, "timing_wrap.cpp"), os.path.abspath(__file__)]
    if not force and os.path.exists(EXE) and all(os.path.getmtime(d) <= os.path.getmtime(EXE) for d in srcs + own):
        return EXE
    os.makedirs(OBJ, exist_ok=True)
    jobs, objs = [], []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        jobs.append(["nvcc", "-c", "-w", "-I" + GEN_INC, s, "-o", o] + ARCH + ["-Xcompiler", "-fopenmp"])
    for f in ("noise_wrap.cpp", "timing_wrap.cpp"):
        o = os.path.join(OBJ, f[:-4] + ".o")
        objs.append(o)
        jobs.append(["g++", "-O2", "-c", os.path.join(EMUL, f), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    _run(["nvcc"] + objs + ["-o", EXE + ".tmp", "-lcuda", "-lcudart", "-lcufft"] + ARCH +
         ["-Xcompiler", "-fopenmp", "-lgomp"] + [f"-Xlinker=--wrap={w}" for w in WRAPS])
    os.replace(EXE + ".tmp", EXE)
    return EXE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

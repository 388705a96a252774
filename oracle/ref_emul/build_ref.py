"""Recipe: the reference's own sources, compiled for the CPU (TEST INFRASTRUCTURE).

Two steps.

generate() -- only where the reference tree is (FARGO_REFERENCE_DIR, else a
`reference` directory beside this repository): reads src/*.cu and include/*.cuh
there and writes them into oracle/_ref/ (git-ignored, never committed).  The only
source change is mechanical: each kernel launch `name<<<grid, block[, smem]>>>(args)`
becomes `emu_make([](auto... a) { name(a...); }, grid, block[, smem])(args)`; the
rest of each file is unchanged.

build() -- anywhere oracle/_ref/src exists (here, and on a machine that received a
copy of this working tree): compiles those files with emul.h force-included,
fake_include/ (CUDA runtime, cuFFT, math_constants stand-ins), noise_wrap.cpp
(seeded initial noise through -Wl,--wrap on InitGasDensity / InitGasEnergy),
sg_wrap.cpp (the self-gravity set-up step that stops the reference, replaced at
link time), reduce_wrap.cpp (DeviceReduce's summation order without fibers) and
timing_wrap.cpp (one `REFSTEP dt substeps seconds` line per AlgoGas call on stderr),
into oracle/_ref/fargo_ref_cpu -- the reference's main() on the CPU:

    echo 0 | oracle/_ref/fargo_ref_cpu file.par

FARGO_REF_THREADS=n runs the blocks of each launch on n host threads (emul.cpp).
"""
import concurrent.futures as cf
import filecmp
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REPO = os.path.dirname(ORACLE)
OUT = os.path.join(ORACLE, "_ref")
GEN_SRC = os.path.join(OUT, "src")
GEN_INC = os.path.join(OUT, "include")
EXE = os.path.join(OUT, "fargo_ref_cpu")

LAUNCH = re.compile(r"(\b[A-Za-z_]\w*(?:<[^<>]*>)?)\s*<<<\s*(.*?)\s*>>>\s*\(")
FLAGS = ["-O2", "-std=c++17", "-w", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]
WRAPS = ["_Z14InitGasDensityPd", "_Z13InitGasEnergyPd", "_Z24Init_planetarysys_withSGP16planetary_system",
         "_Z12DeviceReducePdi", "_Z7AlgoGasP5forcePdS1_S1_S1_S1_P16planetary_systemi", "_Z9TransportPdS_S_S_S_d"]


def reference_dir():
    d = os.environ.get("FARGO_REFERENCE_DIR") or os.path.join(os.path.dirname(REPO), "reference")
    return d if os.path.isdir(os.path.join(d, "src")) and os.path.isdir(os.path.join(d, "include")) else None


def transform(text):
    def rep(m):
        name, cfg = m.group(1), m.group(2)
        if name.startswith("DeviceReduceKernel"):  # the one kernel with __syncthreads
            parts = [p.strip() for p in cfg.split(",")]
            while len(parts) < 3:
                parts.append("0")
            cfg = ", ".join(parts) + ", true"
        # a generic lambda resolves overloads at the call, as the launch syntax does
        return f"emu_make([](auto... emu_a) {{ {name}(emu_a...); }}, {cfg})("
    return LAUNCH.sub(rep, text)


def _write_if_changed(path, text):
    if os.path.exists(path) and open(path).read() == text:
        return
    with open(path, "w") as g:
        g.write(text)


def generate():
    ref = reference_dir()
    if ref is None:
        return False
    os.makedirs(GEN_SRC, exist_ok=True)
    os.makedirs(GEN_INC, exist_ok=True)
    for f in sorted(os.listdir(os.path.join(ref, "src"))):
        if f.endswith(".cu"):
            src = os.path.join(ref, "src", f)
            _write_if_changed(os.path.join(GEN_SRC, f[:-3] + ".cpp"),
                              f'#line 1 "{src}"\n' + transform(open(src).read()))
    for f in sorted(os.listdir(os.path.join(ref, "include"))):
        if f.endswith(".cuh"):
            src, dst = os.path.join(ref, "include", f), os.path.join(GEN_INC, f)
            if not (os.path.exists(dst) and filecmp.cmp(src, dst, shallow=False)):
                shutil.copyfile(src, dst)
    return True


def sources():
    if not os.path.isdir(GEN_SRC):
        return []
    return sorted(os.path.join(GEN_SRC, f) for f in os.listdir(GEN_SRC) if f.endswith(".cpp"))


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stderr[-4000:])


def build(force=False):
    generate()
    srcs = sources()
    if not srcs:
        return None
    own = [os.path.join(HERE, f) for f in ("emul.h", "emul.cpp", "noise_wrap.cpp", "sg_wrap.cpp", "reduce_wrap.cpp",
                                           "timing_wrap.cpp", "build_ref.py")]
    if not force and os.path.exists(EXE) and all(os.path.getmtime(d) <= os.path.getmtime(EXE) for d in own + srcs):
        return EXE
    inc = ["-I" + os.path.join(HERE, "fake_include"), "-I" + GEN_INC]
    jobs, objs = [], []
    for cpp in srcs:
        obj = cpp[:-4] + ".o"
        objs.append(obj)
        jobs.append(["g++"] + FLAGS + ["-include", os.path.join(HERE, "emul.h")] + inc + ["-c", cpp, "-o", obj])
    for f in ("emul.cpp", "noise_wrap.cpp", "sg_wrap.cpp", "reduce_wrap.cpp", "timing_wrap.cpp"):
        obj = os.path.join(OUT, f[:-4] + ".o")
        objs.append(obj)
        jobs.append(["g++"] + FLAGS + inc + ["-c", os.path.join(HERE, f), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_compile, jobs))
    _compile(["g++", "-fopenmp"] + objs + ["-o", EXE] + [f"-Wl,--wrap={w}" for w in WRAPS])
    return EXE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

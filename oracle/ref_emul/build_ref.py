"""Recipe: the reference's own sources, compiled for the CPU (TEST INFRASTRUCTURE).

Reads src/*.cu and include/*.cuh where they lie under /root/reference (never
copied into the repository).  The only source change is mechanical: each kernel
launch `name<<<grid, block[, smem]>>>(args)` becomes
`emu_make([](auto... a) { name(a...); }, grid, block[, smem])(args)`, written with the unchanged rest of the file into
oracle/_ref/src/ (git-ignored).  Everything else comes from emul.h (force-included),
fake_include/ (CUDA runtime, cuFFT, math_constants stand-ins) and noise_wrap.cpp
(seeded initial noise through -Wl,--wrap on InitGasDensity / InitGasEnergy).
Output: oracle/_ref/fargo_ref_cpu, the reference's main() on the CPU:

    echo 0 | oracle/_ref/fargo_ref_cpu file.par

Only this container has the reference sources; the GPU machine never runs this.
"""
import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
REF = os.environ.get("FARGO_REFERENCE_DIR", "/root/reference")
EXE = os.path.join(OUT, "fargo_ref_cpu")

LAUNCH = re.compile(r"(\b[A-Za-z_]\w*(?:<[^<>]*>)?)\s*<<<\s*(.*?)\s*>>>\s*\(")
FLAGS = ["-O2", "-std=c++17", "-w", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


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


def sources():
    src = os.path.join(REF, "src")
    return sorted(f for f in os.listdir(src) if f.endswith(".cu"))


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stderr[-4000:])


def build(force=False):
    if not os.path.isdir(os.path.join(REF, "src")):
        return None
    os.makedirs(os.path.join(OUT, "src"), exist_ok=True)
    deps = [os.path.join(HERE, f) for f in ("emul.h", "emul.cpp", "noise_wrap.cpp", "sg_wrap.cpp", "build_ref.py")]
    if not force and os.path.exists(EXE) and all(os.path.getmtime(d) <= os.path.getmtime(EXE) for d in deps):
        return EXE
    inc = ["-include", os.path.join(HERE, "emul.h"), "-I" + os.path.join(HERE, "fake_include"),
           "-I" + os.path.join(REF, "include")]
    jobs, objs = [], []
    for f in sources():
        text = open(os.path.join(REF, "src", f)).read()
        cpp = os.path.join(OUT, "src", f[:-3] + ".cpp")
        with open(cpp, "w") as g:
            g.write(f'#line 1 "{os.path.join(REF, "src", f)}"\n')
            g.write(transform(text))
        obj = cpp[:-4] + ".o"
        objs.append(obj)
        jobs.append(["g++"] + FLAGS + inc + ["-c", cpp, "-o", obj])
    for f in ("emul.cpp", "noise_wrap.cpp", "sg_wrap.cpp"):
        obj = os.path.join(OUT, f[:-4] + ".o")
        objs.append(obj)
        jobs.append(["g++"] + FLAGS + ["-I" + os.path.join(HERE, "fake_include"),
                                       "-I" + os.path.join(REF, "include"), "-c", os.path.join(HERE, f),
                                       "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_compile, jobs))
    link = ["g++", "-fopenmp"] + objs + ["-o", EXE, "-Wl,--wrap=_Z14InitGasDensityPd",
                                         "-Wl,--wrap=_Z13InitGasEnergyPd",
                                         "-Wl,--wrap=_Z24Init_planetarysys_withSGP16planetary_system"]
    _compile(link)
    return EXE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

"""Generate the golden fixtures of tests/test_oracle_pin.py.

Runs the reference's own sources compiled for the CPU (oracle/ref_emul/build_ref.py
-> oracle/_ref/fargo_ref_cpu, built from the reference tree where it lies) on
several .par files, and stores for each output dump (after 1 and 2 DTs):
  * the SHA-256 of every full field (raw FP64 bytes, as dumped),
  * the FP64 ring sums of every field,
  * two full rings of every field,
  * the planet rows (planet0.dat),
plus the .par text itself, so the test rebuilds identical inputs.  Seeded noise
is injected through the reference's InitGasDensity / InitGasEnergy (link-time
wrap, same generator as the SigmaNoise / EnergyNoise keys).

Usage (needs the reference tree; minutes of CPU time):
    python tests/golden/make_golden.py [name ...]
"""
import hashlib
import os
import platform
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

PLANET_FIXED = "Jupiter 1.0 0.001 0.0 NO NO\n"
PLANET_MIGRATING = "Migrator 1.5 5e-4 0.0 YES YES\n"

COMMON = """Transport FARGO
Disk YES
IndirectTerm YES
Nrad 128
Nsec 384
RadialSpacing LOGARITHM
Ntot 2
Ninterm 1
DT 0.05
SigmaNoise 1e-4
NoiseSeed 7
"""

ISO = """AspectRatio 0.05
Sigma0 6.3662e-4
Viscosity 1e-5
SigmaSlope 0.5
ForcedCircular YES
ThicknessSmoothing 0.6
Rmin 0.4
Rmax 2.5
Frame FIXED
"""

CASES = {
    "iso": (ISO + "InnerBoundary WALL\n", PLANET_FIXED),
    "open": (ISO + "InnerBoundary OPEN\n", PLANET_FIXED),
    "evanescent": (ISO + "InnerBoundary EVANESCENT\n", PLANET_FIXED),
    "nonreflecting": (ISO + "InnerBoundary NONREFLECTING\n", PLANET_FIXED),
    "adiabatic_cooling": ("""AspectRatio 0.05
Sigma0 6.3662e-4
AlphaViscosity 1e-3
SigmaSlope 0.5
Adiabatic YES
AdiabaticIndex 1.4
Cooling YES
CoolingTime0 10.0
ForcedCircular YES
ThicknessSmoothing 0.6
Rmin 0.3
Rmax 3.0
Frame FIXED
EnergyNoise 1e-4
""", PLANET_FIXED),
    # an ensemble disk: isothermal with alpha viscosity and a Sigma slope away from
    # 1/2 (the initial viscous drift is not zero), a low-mass planet
    "iso_alpha": ("""AspectRatio 0.0788
Sigma0 6.3662e-4
AlphaViscosity 8.5e-4
SigmaSlope 1.2
ForcedCircular YES
ThicknessSmoothing 0.6
Rmin 0.4
Rmax 2.5
Frame FIXED
InnerBoundary WALL
""", "Earthlike 1.0 1.0267e-05 0.0 NO NO\n"),
    "corotating_rk5": ("""AspectRatio 0.05
Sigma0 8.84194128288308e-4
AlphaViscosity 1e-3
SigmaSlope 1.0
ForcedCircular NO
ThicknessSmoothing 0.3
Rmin 0.4
Rmax 4.0
Frame COROTATING
""", PLANET_MIGRATING),
    "selfgravity": ("""AspectRatio 0.05
Sigma0 8.84194128288308e-4
AlphaViscosity 1e-3
SigmaSlope 1.0
SelfGravity YES
ForcedCircular NO
ThicknessSmoothing 0.3
Rmin 0.4
Rmax 4.0
Frame FIXED
""", PLANET_MIGRATING),
}

FIELDS = ("dens", "vrad", "vtheta", "energy", "temperature")
RINGS = (1, 64)


def par_text(name, outdir, cfg_path):
    body, _ = CASES[name]
    return body + COMMON + f"PlanetConfig {cfg_path}\nOutputDir {outdir}/\nWriteEnergy YES\n"


def noise_env(text):
    env = dict(os.environ)
    for line in text.splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[0].upper() == "SIGMANOISE":
            env["FARGO_REF_SIGMA_NOISE"] = parts[1]
        if len(parts) >= 2 and parts[0].upper() == "ENERGYNOISE":
            env["FARGO_REF_ENERGY_NOISE"] = parts[1]
        if len(parts) >= 2 and parts[0].upper() == "NOISESEED":
            env["FARGO_REF_NOISE_SEED"] = parts[1]
    return env


def run_case(exe, name):
    with tempfile.TemporaryDirectory() as d:
        cfg = os.path.join(d, "planet.cfg")
        open(cfg, "w").write("# Name Distance Mass Accretion FeelsDisk FeelsOthers\n" + CASES[name][1])
        out = os.path.join(d, "out")
        os.makedirs(out)
        text = par_text(name, out, cfg)
        par = os.path.join(d, "run.par")
        open(par, "w").write(text)
        r = subprocess.run([exe, par], input="0\n", capture_output=True, text=True, env=noise_env(text),
                           cwd=d, timeout=3600)
        rec = {"par": np.array(text.replace(d, "@RUNDIR@")), "cfg": np.array(CASES[name][1]),
               "returncode": np.array(r.returncode), "machine": np.array(platform.machine())}
        if r.returncode != 0:
            rec["stderr"] = np.array((r.stdout + r.stderr)[-2000:])
            return rec
        nrad, nsec = 128, 384
        for k in (1, 2):
            for f in FIELDS:
                path = os.path.join(out, f, f"{f}{k}.dat")
                if not os.path.exists(path):
                    continue
                raw = open(path, "rb").read()
                a = np.frombuffer(raw, dtype=np.float64).reshape(nrad, nsec)
                rec[f"{f}{k}_sha256"] = np.array(hashlib.sha256(raw).hexdigest())
                rec[f"{f}{k}_ringsum"] = a.sum(axis=1)
                for i in RINGS:
                    rec[f"{f}{k}_ring{i}"] = a[i].copy()
        rows = open(os.path.join(out, "planet0.dat")).read().split("\n")
        rec["planet_rows"] = np.array([[float(x) for x in row.split("\t")] for row in rows if row.strip()])
        return rec


def main(names):
    from oracle.ref_emul import build_ref
    exe = build_ref.build()
    if exe is None:
        raise SystemExit("the reference sources are not available here")
    import concurrent.futures as cf
    names = names or list(CASES)
    with cf.ThreadPoolExecutor(max_workers=len(names)) as ex:
        for name, rec in zip(names, ex.map(lambda n: run_case(exe, n), names)):
            np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **rec)
            print(name, "returncode", int(rec["returncode"]), "keys", len(rec), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])

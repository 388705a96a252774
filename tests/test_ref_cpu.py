"""The CPU build of the reference (oracle/_ref/fargo_ref_cpu) against the golden
fixtures it made.

The fixtures of tests/golden/ were made with every block of every launch run in
order on one host thread and DeviceReduceKernel's blocks run as cooperative fibers.
The build now restates DeviceReduce's summation order without fibers
(oracle/ref_emul/reduce_wrap.cpp) and may run the blocks of a launch on several
host threads (FARGO_REF_THREADS).  Neither may change a bit: every dumped field
and planet row of the eight cases must be reproduced exactly, on one thread and on
four.  This build is bench.py's reference arm.
"""
import os
import platform
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
EXE = os.path.join(ROOT, "oracle", "_ref", "fargo_ref_cpu")
sys.path.insert(0, os.path.join(HERE, "golden"))

pytestmark = pytest.mark.skipif(not os.path.exists(EXE), reason="the CPU build of the reference is not built here")


@pytest.mark.parametrize("threads", ["1", "4"])
@pytest.mark.parametrize("name", ["iso", "open", "evanescent", "nonreflecting", "adiabatic_cooling",
                                  "corotating_rk5", "selfgravity", "iso_alpha"])
def test_reference_cpu_build_reproduces_fixture(name, threads, monkeypatch):
    import make_golden as mg
    rec_file = dict(np.load(os.path.join(HERE, "golden", f"ref_{name}.npz")))
    if str(rec_file["machine"]) != platform.machine():
        pytest.skip("fixtures were made on another machine type")
    monkeypatch.setenv("FARGO_REF_THREADS", threads)
    rec = mg.run_case(EXE, name)
    assert int(rec["returncode"]) == 0
    keys = [k for k in rec_file if k.endswith("_sha256")]
    assert keys
    for k in keys:
        assert str(rec[k]) == str(rec_file[k]), k
    assert np.array_equal(rec["planet_rows"], rec_file["planet_rows"])


def test_ensemble_disk_runs_as_the_reference_reads_its_par(tmp_path, monkeypatch):
    # an ensemble disk (config.c4_draws) written as .par keys and a planet-file mass
    # (bench.c4_overrides, as the reference's CUDA baseline of the ensemble runs it)
    # must be the disk the oracle builds from config.c4_disks: bitwise after two
    # shortened DTs of the reference's CPU build
    import bench
    from cudaprotoplanetarydisks_gb300.config import c4_disks, c4_draws
    from oracle.oracle import OracleDisk
    monkeypatch.setenv("FARGO_REF_THREADS", "4")
    k = 3  # a 128 x 384 disk
    d = c4_draws(k + 1)[k]
    out = str(tmp_path / "out")
    steps, _ = bench.run_reference_exe(EXE, "c1", 2, ninterm=1, outdir=out, overrides=bench.c4_overrides(d),
                                       planet_mass=d["q"], dt_divisor=20.0)
    assert len(steps) == 2
    params, planets = c4_disks(k + 1)[k]
    params.dt = params.dt / 20.0
    o = OracleDisk(params, planets)
    try:
        shape = (params.nrad, params.nsec)
        for n in (0, 1):
            if n:
                assert o.step_DT() == steps[0][0]
            for name in ("dens", "vrad", "vtheta"):
                ref = np.fromfile(os.path.join(out, name, f"{name}{n}.dat"), dtype=np.float64).reshape(shape)
                mine = o.field(name)[:-1]
                if platform.machine() == "x86_64":
                    assert np.array_equal(mine, ref), (name, n)
                else:  # other compilers contract other multiply-adds (the oracle pins allow 1e-12 there)
                    assert np.abs(mine - ref).max() <= 1e-12 * np.abs(ref).max(), (name, n)
    finally:
        o.close()

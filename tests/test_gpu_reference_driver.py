"""The reference's own host driver on this library (the drop-in binary).

cudaprotoplanetarydisks_gb300/shim/fargo_ref_driver_gb300 is the reference's
src/Main.cu, Interpret.cu, Psys.cu, Output.cu, Theo.cu, Init.cu and LowTasks.cu,
unchanged, linked through reference_shim.cu to libfargo_gb300.so.  Run on the
isothermal 128 x 384 disk for three DTs with a dump before each, its main() parses
the .par, reads the planets, writes the reference's dump files and planet file,
and steps through fargo_step_DT.  Its gasdens / gasvrad / gasvtheta dumps after one
and two DTs must be bitwise the fields of the same disk advanced through the C-ABI
(the same FP64 step on the same inputs), and its planet file must carry the same
orbit and clock.
"""
import os

import numpy as np
import pytest

import bench
import cudaprotoplanetarydisks_gb300 as fg

pytestmark = pytest.mark.gpu

EXE = os.path.join(bench.ROOT, "cudaprotoplanetarydisks_gb300", "shim", "fargo_ref_driver_gb300")


def test_reference_driver_on_the_library_matches_the_c_abi(tmp_path):
    if not os.path.exists(EXE):
        err = EXE + ".build_error"
        pytest.fail(open(err).read() if os.path.exists(err) else "the linked reference driver is missing")
    out = str(tmp_path / "out")
    bench.run_reference_exe(EXE, "c1", 3, ninterm=1, outdir=out)
    params, planets = fg.load_config("c1")
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    try:
        shape = (params.nrad, params.nsec)
        rows = [r.split() for r in open(os.path.join(out, "planet0.dat")).read().splitlines() if r.strip()]
        for k in (1, 2):
            disk.step_DT()
            for name in ("dens", "vrad", "vtheta"):
                dump = np.fromfile(os.path.join(out, name, f"{name}{k}.dat"), dtype=np.float64).reshape(shape)
                assert np.array_equal(dump, disk.field(name)[:-1]), (name, k)
            pl, sc = disk.planets()[0], disk.scalars()
            row = [float(x) for x in rows[k]]
            assert int(row[0]) == k
            assert (row[1], row[2], row[3], row[4]) == (pl.x, pl.y, pl.vx, pl.vy)
            assert row[7] == sc.physical_time
    finally:
        disk.close()

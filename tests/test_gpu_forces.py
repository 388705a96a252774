"""fargo_compute_force (ComputeForce) and fargo_update_log (UpdateLog) against
the CPU oracle; the driver's --torques option."""
import os
import subprocess

import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from oracle import force_ref

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CFG = os.path.join(ROOT, "cudaprotoplanetarydisks_gb300", "configs", "c1_planet.cfg")


def c1_disk(tmp_path, precision, nrad=64, nsec=192):
    par = os.path.join(ROOT, "cudaprotoplanetarydisks_gb300", "configs", "c1_isothermal.par")
    params = fg.read_par(par)
    params.nrad, params.nsec = nrad, nsec
    params.outputdir = (str(tmp_path) + "/").encode()
    planets = fg.read_planets(params, par)
    assert len(planets) == 1
    disk = fg.Disk(params, planets, precision)
    disk.run(1)
    return params, disk


def close(a, b, tol):
    scale = np.abs(b).max(axis=-1, keepdims=True)
    return np.all(np.abs(a - b) <= tol * scale)


@pytest.mark.parametrize("prec", [fg.FARGO_FP64, fg.FARGO_FP32_BULK])
def test_compute_force_matches_oracle(tmp_path, prec):
    params, disk = c1_disk(tmp_path, prec)
    _, rmed, _, surf = disk.mesh()
    dens = disk.field("dens")[:-1]
    p = disk.planets()[0]
    a = float(np.hypot(p.x, p.y))
    rh = force_ref.hill_radius(p.mass, a)
    for x, y, eps in ((p.x, p.y, 0.03), (0.2, -0.7, 0.01)):
        gf = disk.compute_force(x, y, eps, p.mass, a, rh)
        ref = force_ref.compute_force(dens, rmed, surf, x, y, eps, a, rh)
        assert close(gf, ref, 1e-12), np.abs(gf - ref).max()
    disk.close()


def test_update_log_rows(tmp_path):
    params, disk = c1_disk(tmp_path, fg.FARGO_FP64)
    disk.update_log(3)
    disk.update_log(4)
    _, rmed, _, surf = disk.mesh()
    dens = disk.field("dens")[:-1]
    p = disk.planets()[0]
    s = disk.scalars()
    r = float(np.hypot(p.x, p.y))
    eps = params.thicknesssmoothing * params.aspectratio * r ** (1.0 + params.flaringindex)
    gf = force_ref.compute_force(dens, rmed, surf, p.x, p.y, eps, r, force_ref.hill_radius(p.mass, r))
    rows = [line.split("\t") for line in (tmp_path / "tqwk0.dat").read_text().splitlines()]
    assert [row[0] for row in rows] == ["3", "4"] and all(len(row) == 10 for row in rows)
    got = np.array([float(v) for v in rows[0][1:]])
    ref = force_ref.torque_row(gf, p.x, p.y, p.vx, p.vy, s.physical_time)
    assert np.all(np.abs(got - ref) <= 1e-12 * np.abs(ref[:8]).max()), np.abs(got - ref).max()
    # no self-gravity: one file per Hill-cut level
    for level in range(fg.FORCE_LEVELS):
        level_rows = (tmp_path / f"tqwk0_{level}.dat").read_text().splitlines()
        assert len(level_rows) == 2 and len(level_rows[0].split("\t")) == 6
    disk.close()


def test_driver_torque_logs(tmp_path):
    exe = os.path.join(ROOT, "cudaprotoplanetarydisks_gb300", "fargo_gb300")
    par = tmp_path / "run.par"
    par.write_text(f"""AspectRatio 0.05\nSigma0 6.3662e-4\nViscosity 1e-5\nSigmaSlope 0.5
PlanetConfig {CFG}\nThicknessSmoothing 0.6\nNrad 32\nNsec 96\nRmin 0.4\nRmax 2.5
RadialSpacing LOGARITHM\nNtot 4\nNinterm 2\nDT 0.314159265359\nOutputDir {tmp_path}/\n""")
    r = subprocess.run([exe, "--torques", str(par)], input="0\n", capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    # one row before every DT, stamped with the last output's index (src/Main.cu:309-322)
    steps = [line.split("\t")[0] for line in (tmp_path / "tqwk0.dat").read_text().splitlines()]
    assert steps == ["0", "0", "0", "1", "1"]

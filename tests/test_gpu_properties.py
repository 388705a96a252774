"""Size-independent properties at the full workload sizes (256 x 768 with
self-gravity, 1024 x 3072 with the energy equation), failure reporting, and the
output files / driver executable."""
import os
import subprocess

import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from tests.helpers import disk_mass, small

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("cfg,prec,ndt,tol", [
    ("c2", fg.FARGO_FP64, 2, 1e-13),
    ("c2", fg.FARGO_FP32_BULK, 2, 1e-5),
    ("c3", fg.FARGO_FP32_BULK, 1, 1e-5),
    ("c3", fg.FARGO_FP64, 1, 1e-13),
])
def test_mass_conservation_full_size(cfg, prec, ndt, tol):
    # WALL boundaries: transport moves mass between cells only
    params, planets = fg.load_config(cfg)
    disk = fg.Disk(params, planets, prec)
    surf = disk.mesh()[3]
    m0 = disk_mass(disk.field("dens"), surf)
    nsub = disk.run(ndt)
    assert nsub > 0
    d = disk.field("dens")
    assert np.isfinite(d).all() and (d[:-1] > 0).all()
    m1 = disk_mass(d, surf)
    assert abs(m1 - m0) <= tol * m0, (m0, m1)
    s = disk.scalars()
    assert abs(s.physical_time - ndt * params.dt) < 1e-9
    disk.close()


def test_axisymmetry_preserved_full_size():
    params, planets = fg.load_config("c2", sigma_noise=0.0)
    planets[0].mass = 0.0
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    disk.run(1)
    for name in ("dens", "vtheta"):
        f = disk.field(name)[:-1]
        spread = (f.max(axis=1) - f.min(axis=1)).max()
        assert spread <= 1e-13 * np.abs(f).max(), (name, spread)
    disk.close()


def test_numeric_failure_is_reported_and_recoverable():
    # the failure is made on the host (a NaN written into the density); the device
    # flags it, the DT loop stops, the call returns FARGO_ERR_NUMERIC, and the
    # context keeps working once a valid state is loaded again
    params, planets = small("c1")
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    good = {k: disk.field(k) for k in ("dens", "vrad", "vtheta", "energy")}
    bad = good["dens"].copy()
    bad[10, 17] = np.nan
    disk.set_fields(dens=bad)
    with pytest.raises(fg.FargoError) as err:
        disk.step_DT()
    assert "status 4" in str(err.value)
    disk.set_fields(**good)
    assert disk.step_DT() > 0
    assert np.isfinite(disk.field("dens")).all()
    disk.close()


def test_invalid_parameters_rejected():
    params, planets = small("c2", nsec=190)  # 190 = 2 * 5 * 19: no radix-2/3 FFT plan
    with pytest.raises(fg.FargoError):
        fg.Disk(params, planets, fg.FARGO_FP64)


def test_output_files(tmp_path):
    params, planets = small("c3", outputdir=str(tmp_path) + "/", write_energy=1, write_qplus=1)
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    disk.write_dims()
    disk.step_DT()
    disk.write_outputs(1)
    n = params.nrad * params.nsec
    for name in ("dens", "vrad", "vtheta", "energy", "temperature", "qplus"):
        data = np.fromfile(tmp_path / name / f"{name}1.dat", dtype=np.float64)
        assert data.size == n
        assert np.array_equal(data, disk.field(name)[:-1].ravel())
    rows = (tmp_path / "planet0.dat").read_text().split("\n")
    assert rows[0].split("\t")[0] == "1" and len(rows[0].split("\t")) == 11
    assert len((tmp_path / "used_rad.dat").read_text().split()) == params.nrad + 1
    assert (tmp_path / "dims.dat").read_text().split()[-2:] == [str(params.nrad), str(params.nsec)]
    disk.close()


def test_driver_executable(tmp_path):
    exe = os.path.join(ROOT, "cudaprotoplanetarydisks_gb300", "fargo_gb300")
    cfg = os.path.join(ROOT, "cudaprotoplanetarydisks_gb300", "configs", "c1_planet.cfg")
    par = tmp_path / "run.par"
    par.write_text(f"""AspectRatio 0.05\nSigma0 6.3662e-4\nViscosity 1e-5\nSigmaSlope 0.5
PlanetConfig {cfg}\nForcedCircular YES\nThicknessSmoothing 0.6\nNrad 64\nNsec 192\nRmin 0.4\nRmax 2.5
RadialSpacing LOGARITHM\nNtot 2\nNinterm 1\nDT 0.314159265359\nOutputDir {tmp_path}/\nSigmaNoise 1e-4\n""")
    r = subprocess.run([exe, str(par)], input="0\n", capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    # NTOT+1 DT steps, outputs before steps 0, 1, 2 (src/Main.cu:309-325)
    for k in range(3):
        assert (tmp_path / "dens" / f"dens{k}.dat").stat().st_size == 64 * 192 * 8
    params = fg.read_par(str(par))
    planets = fg.read_planets(params, str(par))
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    disk.run(2)
    d2 = np.fromfile(tmp_path / "dens" / "dens2.dat", dtype=np.float64)
    assert np.array_equal(d2, disk.field("dens")[:-1].ravel())
    disk.close()


@pytest.mark.parametrize("fp32", [False, True])
def test_driver_restart_continues_the_run(tmp_path, fp32):
    """-s 1 from a copy of a run's outputs gives output 2 and the planet rows of
    the uninterrupted run, bitwise."""
    import shutil
    exe = os.path.join(ROOT, "cudaprotoplanetarydisks_gb300", "fargo_gb300")
    cfg = os.path.join(ROOT, "cudaprotoplanetarydisks_gb300", "configs", "c1_planet.cfg")

    def par(outdir):
        p = outdir / "run.par"
        p.write_text(f"""AspectRatio 0.05\nSigma0 6.3662e-4\nViscosity 1e-5\nSigmaSlope 0.5
PlanetConfig {cfg}\nForcedCircular NO\nThicknessSmoothing 0.6\nNrad 64\nNsec 192\nRmin 0.4\nRmax 2.5
RadialSpacing LOGARITHM\nNtot 4\nNinterm 2\nDT 0.314159265359\nOutputDir {outdir}/\nSigmaNoise 1e-4\n""")
        return str(p)

    extra = ["--fp32"] if fp32 else []
    a = tmp_path / "a"
    a.mkdir()
    r = subprocess.run([exe] + extra + [par(a)], input="0\n", capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    b = tmp_path / "b"
    shutil.copytree(a, b)
    for name in ("dens", "vrad", "vtheta"):
        (b / name / f"{name}2.dat").unlink()
    r = subprocess.run([exe, "-s", "1"] + extra + [par(b)], input="0\n", capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "restarting from output 1" in r.stdout
    for name in ("dens", "vrad", "vtheta"):
        x = np.fromfile(a / name / f"{name}2.dat", dtype=np.float64)
        y = np.fromfile(b / name / f"{name}2.dat", dtype=np.float64)
        assert np.array_equal(x, y), (name, float(np.abs(x - y).max()))
    assert (a / "planet0.dat").read_text() == (b / "planet0.dat").read_text()


def test_restart_with_missing_output_fails(tmp_path):
    params = fg.read_par(os.path.join(ROOT, "cudaprotoplanetarydisks_gb300", "configs", "c1_isothermal.par"))
    params.nrad, params.nsec = 32, 96
    params.outputdir = (str(tmp_path) + "/").encode()
    disk = fg.Disk(params, [], fg.FARGO_FP64)
    with pytest.raises(RuntimeError):
        disk.restart(3)
    disk.close()

"""The per-substep entry points of the C-ABI against the oracle's, each applied to
one identical state (the oracle's state after one DT, loaded into the GPU)."""
import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from oracle.oracle import OracleDisk
from tests.helpers import rel_linf, small

pytestmark = pytest.mark.gpu
TOL = 1e-9


def paired(cfg, **kw):
    params, planets = small(cfg, **kw)
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    ref = OracleDisk(params, planets)
    ref.step_DT()
    disk.step_DT()
    disk.set_fields(ref.field("dens"), ref.field("vrad"), ref.field("vtheta"), ref.field("energy"))
    return disk, ref


@pytest.mark.parametrize("cfg", ["c1", "c2", "c3"])
def test_condition_cfl(cfg):
    disk, ref = paired(cfg)
    for deltaT in (0.314159265359, 0.05, 1e-3):
        assert disk.condition_cfl(deltaT) == ref.condition_cfl(deltaT)


@pytest.mark.parametrize("cfg", ["c1", "c2"])
def test_potential(cfg):
    disk, ref = paired(cfg)
    disk.substep(fg.SUB_POTENTIAL, 0.01)
    ref.substep(fg.SUB_POTENTIAL, 0.01)
    assert rel_linf(disk.field("potential"), ref.field("potential")) < TOL


@pytest.mark.parametrize("cfg", ["c1", "c2", "c3"])
def test_source_step(cfg):
    disk, ref = paired(cfg)
    for d in (disk, ref):
        d.substep(fg.SUB_POTENTIAL, 0.01)
        d.substep(fg.SUB_SOURCE, 0.01)
    for name in ("vrad", "vtheta", "pressure"):
        assert rel_linf(disk.field(name), ref.field(name)) < TOL, name


def test_energy_step():
    disk, ref = paired("c3")
    for d in (disk, ref):
        d.substep(fg.SUB_ENERGY, 0.01)
    for name in ("energy", "qplus", "divergence"):
        assert rel_linf(disk.field(name), ref.field(name)) < TOL, name


@pytest.mark.parametrize("cfg", ["c1", "c3"])
def test_transport(cfg):
    disk, ref = paired(cfg)
    for d in (disk, ref):
        d.substep(fg.SUB_TRANSPORT, 0.02)
    names = ("dens", "vrad", "vtheta") + (("energy",) if cfg == "c3" else ())
    for name in names:
        assert rel_linf(disk.field(name), ref.field(name)) < TOL, name


@pytest.mark.parametrize("bc", ["open_inner", "evanescent", "non_reflecting"])
def test_boundaries(bc):
    disk, ref = paired("c3", **{bc: 1})
    for d in (disk, ref):
        d.substep(fg.SUB_BOUNDARY, 0.01)
    for name in ("dens", "vrad", "vtheta", "energy"):
        assert rel_linf(disk.field(name), ref.field(name)) < TOL, (bc, name)


def test_self_gravity_acceleration():
    disk, ref = paired("c2")
    for d in (disk, ref):
        d.substep(fg.SUB_POTENTIAL, 0.01)
        d.substep(fg.SUB_SOURCE, 0.01)
    for name in ("sg_accr", "sg_acct"):
        a, b = disk.field(name), ref.field(name)
        assert rel_linf(a, b) < TOL, name


def test_temperature_and_soundspeed():
    disk, ref = paired("c3")
    for d in (disk, ref):
        d.substep(fg.SUB_SOUNDSPEED, 0.0)
        d.substep(fg.SUB_TEMPERATURE, 0.0)
    assert rel_linf(disk.field("temperature"), ref.field("temperature")) < TOL
    assert rel_linf(disk.field("soundspeed"), ref.field("soundspeed")) < TOL


def test_substep_full_fixed_dt():
    params, planets = small("c2")
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    ref = OracleDisk(params, planets)
    for _ in range(3):
        disk.substep_full(0.01)
        ref.substep_full(0.01)
    for name in ("dens", "vrad", "vtheta"):
        assert rel_linf(disk.field(name), ref.field(name)) < TOL, name
    assert np.isclose(disk.scalars().physical_time, 0.03)

"""Parity of the CUDA step (FP64 mode) with the oracle on identical inputs.

Bar: the same number of CFL substeps per DT, every field within 1e-9 relative
(max |gpu - oracle| / max |oracle| over the dumped rings), planets within 1e-9.
The CUDA kernels use fused multiply-add and reciprocal multiplication where the
oracle divides, so agreement is to rounding (~1e-14 after a few DTs), not bitwise.
"""
import os

import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from oracle.oracle import OracleDisk
from tests.helpers import rel_l2, rel_linf, small

pytestmark = pytest.mark.gpu

TOL = 1e-9


def compare(disk, ref, fields, tol=TOL):
    worst = {}
    for name in fields:
        a, b = disk.field(name), ref.field(name)
        worst[name] = (rel_linf(a, b), rel_l2(a, b))
        assert worst[name][0] < tol, (name, worst[name])
    return worst


def compare_planets(disk, ref, tol=TOL):
    for pg, po in zip(disk.planets(), ref.planets()):
        for k in ("x", "y", "vx", "vy"):
            a, b = getattr(pg, k), getattr(po, k)
            assert abs(a - b) <= tol * max(1.0, abs(b)), (k, a, b)


def run_pair(params, planets, ndt, fields=("dens", "vrad", "vtheta")):
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    ref = OracleDisk(params, planets)
    try:
        compare(disk, ref, fields, tol=1e-15)  # identical initial state
        for _ in range(ndt):
            assert disk.step_DT() == ref.step_DT()
            compare(disk, ref, fields)
        compare_planets(disk, ref)
        s, so = disk.scalars(), ref.scalars()
        assert s.substeps == so.substeps
        assert abs(s.physical_time - so.physical_time) <= 1e-12 * max(1.0, so.physical_time)
        assert abs(s.omega_frame - so.omega_frame) <= 1e-9 * max(1.0, abs(so.omega_frame))
    finally:
        disk.close()
        ref.close()


def test_c1_full_length_matches_oracle():
    """The isothermal workload at full size over its stated length (200 hydro
    substeps): the same CFL decisions DT after DT and every field within the bar."""
    params, planets = fg.load_config("c1")
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    ref = OracleDisk(params, planets)
    try:
        while ref.scalars().substeps < 200:
            assert disk.step_DT() == ref.step_DT()
            compare(disk, ref, ("dens", "vrad", "vtheta"))
        compare_planets(disk, ref)
        assert disk.scalars().substeps == ref.scalars().substeps >= 200
    finally:
        disk.close()
        ref.close()


def with_planets(planets, **kw):
    for p in planets:
        for k, v in kw.items():
            setattr(p, k, v)
    return planets


CASES = {
    # the three workloads (the isothermal one at full size)
    "c1_isothermal_128x384": lambda: (fg.load_config("c1"), 3, ()),
    "c2_selfgravity_alpha_rk5": lambda: (small("c2"), 3, ()),
    # self-gravity at lengths with compile-time FFT plans (rings 384, columns 256)
    "c2_selfgravity_128x384": lambda: (small("c2", nrad=128, nsec=384), 2, ()),
    "c3_adiabatic_cooling": lambda: (small("c3"), 3, ("energy",)),
    "c3_adiabatic_no_cooling": lambda: (small("c3", cooling=0), 2, ("energy",)),
    # a ring wider than the register azimuthal kernel's CTA (2176 > 4 x 512 FP64
    # cells): several chunks of four cells per thread
    "wide_ring_register_chunks": lambda: (small("c1", nrad=24, nsec=2176), 2, ()),
    # boundaries
    "open_inner": lambda: (small("c1", open_inner=1), 2, ()),
    "evanescent": lambda: (small("c1", evanescent=1), 2, ()),
    "nonreflecting": lambda: (small("c1", non_reflecting=1), 2, ()),
    "nonreflecting_adiabatic": lambda: (small("c3", non_reflecting=1), 2, ("energy",)),
    "evanescent_selfgravity": lambda: (small("c2", evanescent=1), 2, ()),
    # frames and planets
    "corotating": lambda: (small("c2", corotating=1), 2, ()),
    "guiding_center": lambda: (small("c2", corotating=1, guiding_center=1), 2, ()),
    "roche_smoothing": lambda: (small("c1", thicknesssmoothing=0.0, rochesmoothing=0.5, roche_smoothing=1), 2, ()),
    "release_date_migration": lambda: (small("c2", releasedate=5.0, releaseradius=1.2), 2, ()),
    "no_indirect_term": lambda: (small("c2", indirect_term=0), 2, ()),
    # numerics switches
    "sloppy_cfl": lambda: (small("c1", sloppy_cfl=1), 2, ()),
    "standard_transport": lambda: (small("c1", fast_transport=0), 2, ()),
    "arithmetic_grid": lambda: (small("c1", log_grid=0), 2, ()),
    "imposed_drift_cavity": lambda: (small("c1", imposeddiskdrift=1e-4, cavityradius=0.8, cavityratio=3.0,
                                           cavitywidth=2.0), 2, ()),
    "transition_lambda": lambda: (small("c1", transitionradius=0.9, transitionratio=1.5, transitionwidth=2.0,
                                        lambdadoubling=1e-3), 2, ()),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_fp64_matches_oracle(case):
    (params, planets), ndt, extra = CASES[case]()
    run_pair(params, planets, ndt, ("dens", "vrad", "vtheta") + extra)


def test_two_planets_feeling_each_other():
    params, planets = small("c2")
    second = fg.FargoPlanet()
    second.x, second.y, second.mass = 2.2, 0.0, 2e-4
    second.vy = np.sqrt((1.0 + second.mass) / second.x)
    second.vx = -1e-10 * second.vy
    second.feel_disk, second.feel_others = 1, 1
    run_pair(params, planets + [second], 2)


def test_no_planet():
    # without a planet the reference adds no star potential either (the star term
    # sits inside the planet loop, src/Kernels.cu:1246): the potential is zero and
    # the unbound disk's evolution is chaotic, so one fixed substep is compared
    params, _ = small("c1")
    disk = fg.Disk(params, [], fg.FARGO_FP64)
    ref = OracleDisk(params, [])
    for d in (disk, ref):
        d.substep(fg.SUB_POTENTIAL, 1e-3)
    assert not disk.field("potential").any() and not ref.field("potential").any()
    for d in (disk, ref):
        d.substep_full(1e-3)
    compare(disk, ref, ("dens", "vrad", "vtheta"))
    disk.close()


def _disk_with_env(params, planets, prec, env):
    saved = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return fg.Disk(params, planets, prec)
    finally:
        for k, v in saved.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


@pytest.mark.parametrize("env", ["FARGO_NO_GRAPH", "FARGO_NO_PDL", "FARGO_ROTATE", "FARGO_NO_SG_AHEAD", "FARGO_NO_PAD",
                                 "FARGO_AZ_GLOBAL", "FARGO_PRIO"])
def test_code_paths_are_bitwise_identical(env):
    # the conditional-graph DT loop vs the host loop; programmatic dependent
    # launch vs plain launches; the rotated DT loop (each substep launches the
    # next one's CFL/force kernel and self-gravity transforms) vs the plain
    # one; the next substep's ring transforms launched after the azimuthal
    # transport vs at the substep start; two substeps per loop iteration (the
    # second one run with dt = 0 once the DT is done) vs one; the shared-memory
    # vs the global-memory ring
    # buffers of the barrier-per-phase azimuthal kernel; stream priorities (the
    # hydro chain above the self-gravity transforms) vs equal ones
    params, planets = small("c2")
    base = {"FARGO_AZ_GENERIC": "1"} if env == "FARGO_AZ_GLOBAL" else {}
    a = _disk_with_env(params, planets, fg.FARGO_FP64, base)
    b = _disk_with_env(params, planets, fg.FARGO_FP64, {**base, env: "1"})
    for _ in range(2):
        assert a.step_DT() == b.step_DT()
    for name in ("dens", "vrad", "vtheta"):
        assert np.array_equal(a.field(name), b.field(name))
    a.close()
    b.close()


@pytest.mark.parametrize("cfg", ["c1", "c2", "c3"])
def test_register_azimuthal_kernel_matches_barrier_kernel(cfg):
    # the register-blocked azimuthal transport (nsec % 4 == 0) runs the per-cell
    # arithmetic of the barrier-per-phase kernel; only the ring-mean summation
    # order differs, so the FP64 fields agree to a few ulps per substep
    params, planets = small(cfg)
    assert params.nsec % 4 == 0
    a = fg.Disk(params, planets, fg.FARGO_FP64)
    b = _disk_with_env(params, planets, fg.FARGO_FP64, {"FARGO_AZ_GENERIC": "1"})
    for _ in range(2):
        assert a.step_DT() == b.step_DT()
    names = ("dens", "vrad", "vtheta") + (("energy",) if params.adiabatic else ())
    for name in names:
        assert rel_linf(a.field(name), b.field(name)) < 1e-11, name
    a.close()
    b.close()


@pytest.mark.parametrize("prec,tol", [(fg.FARGO_FP64, 1e-12), (fg.FARGO_FP32_BULK, 1e-5)])
def test_compile_time_fft_plans_match_runtime_plans(prec, tol):
    # rings of 768 and columns of 512 (the 256x768 disk's lengths) with the
    # compile-time Stockham plans vs the run-time plans: the same butterflies and
    # twiddles, so the fields agree to rounding
    params, planets = small("c2", nrad=256, nsec=768)
    a = fg.Disk(params, planets, prec)
    b = _disk_with_env(params, planets, prec, {"FARGO_SG_GENERIC": "1"})
    assert a.step_DT() == b.step_DT()
    for name in ("dens", "vrad", "vtheta"):
        assert rel_linf(a.field(name), b.field(name)) < tol, name
    a.close()
    b.close()


@pytest.mark.parametrize("cfg,kw", [("c1", {}), ("c3", {}), ("c3", {"cooling": 0}), ("c2", {"corotating": 1}),
                                    ("c2", {"corotating": 1, "guiding_center": 1}), ("c1", {"sloppy_cfl": 1})])
def test_padded_substeps_leave_the_disk_unchanged(cfg, kw):
    # a loop body of two substeps runs the second one with dt = 0 when the DT
    # ended after the first: every field, the planets and the clocks must be
    # bitwise those of the one-substep loop, and the padded substeps must have run
    params, planets = small(cfg, **kw)
    a = fg.Disk(params, planets, fg.FARGO_FP64)
    b = _disk_with_env(params, planets, fg.FARGO_FP64, {"FARGO_NO_PAD": "1"})
    for _ in range(4):
        assert a.step_DT() == b.step_DT()
    names = ("dens", "vrad", "vtheta") + (("energy",) if params.adiabatic else ())
    for name in names:
        assert np.array_equal(a.field(name), b.field(name)), name
    for pa, pb in zip(a.planets(), b.planets()):
        assert (pa.x, pa.y, pa.vx, pa.vy) == (pb.x, pb.y, pb.vx, pb.vy)
    sa, sb = a.scalars(), b.scalars()
    assert (sa.physical_time, sa.omega_frame, sa.substeps, sa.last_dt) == \
           (sb.physical_time, sb.omega_frame, sb.substeps, sb.last_dt)
    assert sa.padded_substeps > 0 and sb.padded_substeps == 0
    a.close()
    b.close()

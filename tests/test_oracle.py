"""The oracle (CPU FP64 restatement of the reference step) checked on its own:
its FFT against numpy.fft (cuFFT is not under the reference tree), its
DeviceReduce order, and physical invariants the reference step has."""
import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from oracle import oracle as orc
from tests.helpers import disk_mass, lbp_ring, rest_state, sg_direct_sum, small


@pytest.mark.parametrize("shape", [(8, 6), (16, 12), (64, 48), (256, 384), (10, 7), (128, 66)])
@pytest.mark.parametrize("sign", [-1, 1])
def test_fft2d_matches_numpy(shape, sign):
    rng = np.random.default_rng(7)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    got = orc.fft2d(a, sign)
    want = np.fft.fft2(a) if sign < 0 else np.fft.ifft2(a) * a.size
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


def reduce_restated(x):
    """DeviceReduce (src/Kernels.cu:253-394) restated in numpy loops."""
    n = x.size
    p2 = 1
    while p2 < n:
        p2 <<= 1
    blocks = min((p2 + 31) // 32, 1024)
    grid = 64 * blocks
    parts = []
    for b in range(blocks):
        s = []
        for t in range(32):
            i = b * 64 + t
            acc = 0.0
            while i < n:
                acc += x[i]
                if i + 32 < n:
                    acc += x[i + 32]
                i += grid
            s.append(acc)
        off = 16
        while off:
            for t in range(off):
                s[t] = s[t] + s[t + off]
            off //= 2
        parts.append(s[0])
    tot = 0.0
    for v in parts:
        tot += v
    return tot


@pytest.mark.parametrize("n", [1, 31, 384, 1000, 49152])
def test_device_reduce_order(n):
    x = np.random.default_rng(n).standard_normal(n) * 1e3
    assert orc.device_reduce(x) == reduce_restated(x)
    assert abs(orc.device_reduce(x) - x.sum()) <= 1e-10 * np.abs(x).sum()


def test_mass_conserved_with_wall_boundaries():
    p, pl = small("c1")
    o = orc.OracleDisk(p, pl)
    surf = o.mesh()[3]
    m0 = disk_mass(o.field("dens"), surf)
    for _ in range(3):
        o.step_DT()
    m1 = disk_mass(o.field("dens"), surf)
    assert abs(m1 - m0) <= 1e-13 * m0


def test_open_boundary_semantics():
    # OpenBoundaryKernel (src/Kernels.cu:482-495): ring 0 copies ring 1 and the
    # radial velocity of ring 1 only allows inflow toward the star
    p, pl = small("c1", open_inner=1)
    o = orc.OracleDisk(p, pl)
    o.step_DT()
    o.substep(fg.SUB_BOUNDARY, 0.01)
    d, v = o.field("dens"), o.field("vrad")
    assert np.array_equal(d[0], d[1])
    assert (v[1] <= 0.0).all()
    assert np.isfinite(o.scalars().lost_mass)


def test_axisymmetric_disk_stays_axisymmetric():
    # no noise and a massless planet: every substep (including the integer FARGO
    # shift) maps an axisymmetric state to an axisymmetric state
    p, pl = small("c1", sigma_noise=0.0)
    pl[0].mass = 0.0
    o = orc.OracleDisk(p, pl)
    for _ in range(2):
        o.step_DT()
    for name in ("dens", "vrad", "vtheta"):
        f = o.field(name)[:-1]
        spread = (f.max(axis=1) - f.min(axis=1)).max()
        assert spread <= 1e-14 * max(np.abs(f).max(), 1e-300), (name, spread)


def test_results_do_not_depend_on_thread_count():
    p, pl = small("c2", nrad=32, nsec=96)
    outs = []
    for nt in (1, 3):
        orc.OracleDisk.set_threads(nt)
        o = orc.OracleDisk(p, pl)
        o.step_DT()
        outs.append([o.field(n) for n in ("dens", "vrad", "vtheta")])
    orc.OracleDisk.set_threads(8)
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_cfl_count_and_time():
    p, pl = small("c1")
    o = orc.OracleDisk(p, pl)
    n = o.step_DT()
    s = o.scalars()
    assert n >= 1 and s.substeps == n
    assert abs(s.physical_time - p.dt) <= 1e-12


def test_self_gravity_matches_a_direct_convolution():
    # the oracle's FFT self-gravity of the initial 16 x 32 self-gravitating disk
    # against the direct sum of its kernels
    params, planets = small("c2", nrad=16, nsec=32)
    o = orc.OracleDisk(params, planets)
    try:
        rinf, rmed, _, _ = o.mesh()
        accr, acct = sg_direct_sum(params, rinf, rmed, o.field("dens"))
        n = params.nrad
        er = float(np.abs(o.field("sg_accr")[:n] - accr).max() / np.abs(accr).max())
        et = float(np.abs(o.field("sg_acct")[:n] - acct).max() / np.abs(acct).max())
    finally:
        o.close()
    assert er < 1e-6 and et < 1e-6, (er, et)


def test_rest_state_stays_steady():
    ds, vr_max, axi, cs = rest_state(orc.OracleDisk)
    assert axi < 1e-12 and ds < 3e-3 and vr_max < 1e-2 * cs, (axi, ds, vr_max)


def test_viscous_ring_spreading_matches_lynden_bell_pringle():
    pytest.importorskip("scipy")
    err, dm, ndt, tau = lbp_ring(orc.OracleDisk)
    assert dm <= 1e-12 and err < 5e-3, (dm, err)

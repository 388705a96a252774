"""The disk-force oracle (oracle/force_ref.py) pinned by plain loops over the
cells on a small grid, for every Hill-cut level and an inner/outer split."""
import numpy as np

from oracle import force_ref


def test_compute_force_matches_direct_loops():
    rng = np.random.default_rng(4)
    nrad, nsec = 6, 16
    rmed = np.linspace(0.5, 1.8, nrad + 1)
    surf = rng.uniform(0.5, 1.5, nrad + 1) * 1e-2
    dens = rng.uniform(0.5, 1.5, (nrad, nsec)) * 1e-3
    x, y, eps, a = 0.9, 0.3, 0.04, 1.0
    rh = force_ref.hill_radius(1e-3, a)
    gf = force_ref.compute_force(dens, rmed, surf, x, y, eps, a, rh)
    assert gf.shape == (4, force_ref.LEVELS)
    for k in (0, 1, 5, force_ref.LEVELS - 1):
        ref = force_ref.direct_force(dens, rmed, surf, x, y, eps, a, rh, k)
        assert np.allclose(gf[:, k], ref, rtol=1e-12, atol=0.0), k
    # the cut only removes force: |level k| <= |level 0| cell by cell in sum of moduli
    assert np.all(np.abs(gf[:, -1]) <= np.abs(gf[:, 0]) + 1e-18)


def test_torque_row_layout():
    gf = np.arange(44, dtype=float).reshape(4, 11) + 1.0
    row = force_ref.torque_row(gf, 2.0, 0.0, 0.0, 1.0, 7.0)
    # torque x fy - y fx and power vx fx + vy fy of inner, outer, cut inner, cut outer
    assert row[0] == 2.0 * gf[2, 0] and row[3] == 2.0 * gf[3, -1]
    assert row[4] == gf[2, 0] and row[7] == gf[3, -1] and row[8] == 7.0

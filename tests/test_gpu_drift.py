"""FP32-bulk drift against FP64 over 100 planet orbits (2000 DTs), with controls.

The isothermal 128 x 384 disk with a planet on a fixed circular orbit runs 100
orbits four times: FP64, FP32-bulk, and two FP64 controls whose initial density
is perturbed by one unit in the last place (2^-52) and by one FP32 rounding
(2^-24).  Measured on GB300, density relative L2 after 100 orbits: 1-ulp control
3.7e-10, FP32-level control 8.6e-5, FP32-bulk 4.2e-2 to 1.3e-1 (two builds that
differ only in how one FP32 kernel was compiled: the drift depends on the
rounding pattern of the FP32 arithmetic, not on its size alone).  So the FP64
path is reproducible far below the 1e-9 parity bar, the flow amplifies a single
FP32-sized perturbation only to ~1e-4, and the FP32-bulk drift is the FP32
arithmetic's, accumulated over every substep.  The bounds hold those
measurements with a margin; the 1e-5 target for 100 orbits is not met by
FP32-bulk storage.
"""
import pytest

from cudaprotoplanetarydisks_gb300.drift import drift

pytestmark = pytest.mark.gpu


def test_fp32_drift_over_100_orbits_against_fp64_controls():
    r = drift("c1", 100, every=10, control=True)
    rows = r["by_orbit"]
    assert r["dts"] == 2000
    # FP64 against itself from a one-ulp perturbation: reproducible
    assert max(row["control_dens"]["rel_l2"] for row in rows) < 1e-8
    # FP64 from an FP32-sized perturbation: the flow's own amplification stays small
    assert max(row["control32_dens"]["rel_l2"] for row in rows) < 1e-3
    # FP32-bulk against FP64: bounded, and far above what a single FP32 rounding
    # of the initial state grows to
    assert max(row["dens"]["rel_l2"] for row in rows) < 0.5
    assert r["final_dens_rel_l2"] > 10 * r["final_control32_dens_rel_l2"]
    print([(row["orbits"], row["dens"]["rel_l2"], row["control32_dens"]["rel_l2"], row["control_dens"]["rel_l2"])
           for row in rows])

"""FP32-bulk drift against FP64 over 100 planet orbits (2000 DTs), with a control.

The isothermal 128 x 384 disk with a planet on a fixed circular orbit runs 100
orbits three times: FP64, FP32-bulk, and FP64 from a density perturbed by one
unit in the last place.  Measured on GB300: the control stays within 3.3e-10 of
the FP64 run (the flow does not amplify an ulp-level perturbation over 100
orbits, so the FP64 path is reproducible to far better than the 1e-9 parity bar),
while the FP32-bulk density drifts to 8.6e-4 (10 orbits) and 4.3e-2 (100 orbits)
relative L2: the drift is the FP32 arithmetic's, not the flow's.  The bounds
below hold those measurements with a margin; the 1e-5 target for 100 orbits is
not met by FP32-bulk storage.
"""
import pytest

from cudaprotoplanetarydisks_gb300.drift import drift

pytestmark = pytest.mark.gpu


def test_fp32_drift_over_100_orbits_is_bounded_and_fp64_is_reproducible():
    r = drift("c1", 100, every=10, control=True)
    rows = {row["orbits"]: row for row in r["by_orbit"]}
    assert r["dts"] == 2000
    # FP64 against itself from a one-ulp perturbation: reproducible
    assert max(row["control_dens"]["rel_l2"] for row in r["by_orbit"]) < 1e-8
    # FP32-bulk against FP64: the measured drift, bounded
    assert rows[10]["dens"]["rel_l2"] < 3e-3
    assert rows[100]["dens"]["rel_l2"] < 0.1
    assert r["final_dens_rel_l2"] > 100 * r["final_control_dens_rel_l2"]
    print({k: (v["dens"]["rel_l2"], v["control_dens"]["rel_l2"]) for k, v in rows.items()})

"""FP32-bulk mode: error of every field against the FP64 oracle stays within a
stated bound after a few DTs (relative L2 over the dumped rings)."""
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from oracle.oracle import OracleDisk
from tests.helpers import rel_l2, rel_linf, small

pytestmark = pytest.mark.gpu

# relative L2 bound per field after 3 DTs (float32 has ~6e-8 unit roundoff; the
# planet wake amplifies it; the radial velocity is small in magnitude, so its
# relative error is the largest)
BOUND = {"dens": 1e-4, "vtheta": 1e-5, "vrad": 2e-3, "energy": 1e-4}


@pytest.mark.parametrize("cfg,kw", [("c1", {}), ("c2", {"nrad": 64, "nsec": 192}), ("c3", {"nrad": 64, "nsec": 192})])
def test_fp32_bulk_error_vs_fp64_oracle(cfg, kw):
    params, planets = fg.load_config(cfg, **kw)
    disk = fg.Disk(params, planets, fg.FARGO_FP32_BULK)
    ref = OracleDisk(params, planets)
    for _ in range(3):
        assert disk.step_DT() == ref.step_DT()
    names = ("dens", "vrad", "vtheta") + (("energy",) if params.adiabatic else ())
    for name in names:
        e2 = rel_l2(disk.field(name), ref.field(name))
        einf = rel_linf(disk.field(name), ref.field(name))
        print(f"{cfg} {name}: rel L2 {e2:.2e}  rel Linf {einf:.2e}")
        assert e2 < BOUND[name], (name, e2)
    disk.close()

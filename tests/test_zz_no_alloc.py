"""fargo_condition_cfl_noalloc: the CFL integer for callers that cannot call
cudaMalloc (their device memory belongs to another allocator, or their loop must
not take cudaMalloc's implicit synchronisation).  It reads buffers the caller
already owns and keeps its partial results in a fixed array inside the library.

The test calls it through the C-ABI on device buffers owned by torch, twice in a
row, and checks each result against fargo_condition_cfl on the same disk state and
against the oracle's ConditionCFL (the reference's arithmetic, which this entry
point follows) on the oracle's copy of the same run.
This file is collected last so that a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from oracle.oracle import OracleDisk
from tests.helpers import small

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("cfg", ["c1", "c3"])
def test_noalloc_cfl_matches_context_cfl(cfg):
    import torch
    params, planets = small(cfg)
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    ref = OracleDisk(params, planets)
    assert disk.step_DT() == ref.step_DT()  # a non-trivial state, the same on both
    rinf, rmed, rsup, _ = disk.mesh()
    bufs = {n: dev(disk.field(n)) for n in ("vrad", "vtheta", "soundspeed")}
    mesh = [dev(rinf), dev(rmed), dev(rsup)]
    out = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    lib = fg._capi.load()
    stream = torch.cuda.current_stream().cuda_stream
    p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    for deltaT in (params.dt, 0.05):  # two calls in a row share the fixed scratch
        rc = lib.fargo_condition_cfl_noalloc(p(bufs["vrad"]), p(bufs["vtheta"]), p(bufs["soundspeed"]),
                                             p(mesh[0]), p(mesh[1]), p(mesh[2]), params.nrad, params.nsec,
                                             params.fast_transport, deltaT, ctypes.c_void_p(stream), p(out))
        assert rc == fg._capi.FARGO_OK
        torch.cuda.synchronize()
        got = int(out.item())
        assert got == disk.condition_cfl(deltaT)
        assert got == ref.condition_cfl(deltaT)
    disk.close()
    ref.close()


def test_noalloc_rejects_oversized_grid():
    import torch
    lib = fg._capi.load()
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = ctypes.c_void_p(x.data_ptr())
    rc = lib.fargo_condition_cfl_noalloc(p, p, p, p, p, p, 16385, 8, 1, 0.1, None, ctypes.c_void_p(out.data_ptr()))
    assert rc == fg._capi.FARGO_ERR_INVALID
    # rings wider than the shared-memory staging are rejected the same way (before any launch)
    rc = lib.fargo_condition_cfl_noalloc(p, p, p, p, p, p, 8, 16388, 1, 0.1, None, ctypes.c_void_p(out.data_ptr()))
    assert rc == fg._capi.FARGO_ERR_INVALID

"""The reference's own CUDA build on the GB300 against this code's FP64 mode.

oracle/_ref/fargoGPU_sm103a is the reference's src/*.cu compiled by nvcc for
sm_103a with two source-compat fixes (oracle/ref_cuda/build_ref_cuda.py).  It runs
the configurations whose kernels were read for out-of-bounds access (WALL
boundaries, no self-gravity): the isothermal 128 x 384 disk
(configs/c1_isothermal.par) and the adiabatic disk with cooling and alpha viscosity
(configs/c3_adiabatic.par) at 128 x 384, and one disk of the batched ensemble
(isothermal with alpha viscosity, 128 x 384), for three DTs with a dump before each.
The same disk advanced by this code in FP64 must take the same number of hydro
substeps in every DT and match the reference's gasdens / gasvrad / gasvtheta (and
gasenergy) dumps after one and two DTs within 1e-9 relative.
"""
import os

import numpy as np
import pytest

import bench
import cudaprotoplanetarydisks_gb300 as fg
from tests.helpers import rel_l2, rel_linf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg,size", [("c1", None), ("c3", (128, 384)), ("c4", 3)])
def test_reference_cuda_build_matches_fp64_path(tmp_path, cfg, size):
    if not os.path.exists(bench.REF_CUDA_EXE):
        err = bench.REF_CUDA_EXE + ".build_error"
        pytest.fail(open(err).read() if os.path.exists(err) else "the reference's CUDA build is missing")
    out = str(tmp_path / "out")
    if cfg == "c4":
        # disk `size` of the batched ensemble (isothermal, alpha viscosity, its own
        # planet mass), as bench.reference_cuda_c4 runs it
        from cudaprotoplanetarydisks_gb300.config import c4_draws
        d = c4_draws(size + 1)[size]
        over = bench.c4_overrides(d)
        steps, cells = bench.run_reference_exe(bench.REF_CUDA_EXE, "c1", 3, ninterm=1, outdir=out, overrides=over,
                                               planet_mass=d["q"])
        params, planets = fg.c4_disks(size + 1)[size]
    else:
        over = {"NRAD": size[0], "NSEC": size[1], "WRITEENERGY": "YES"} if size else None
        steps, cells = bench.run_reference_exe(bench.REF_CUDA_EXE, cfg, 3, ninterm=1, outdir=out, overrides=over)
        params, planets = fg.load_config(cfg, **({"nrad": size[0], "nsec": size[1]} if size else {}))
    assert len(steps) == 3
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    names = ("dens", "vrad", "vtheta") + (("energy",) if params.adiabatic else ())
    try:
        shape = (params.nrad, params.nsec)
        for k in (1, 2):
            assert disk.step_DT() == steps[k - 1][0], (k, steps[k - 1])
            for name in names:
                ref = np.fromfile(os.path.join(out, name, f"{name}{k}.dat"), dtype=np.float64).reshape(shape)
                mine = disk.field(name)[:-1]
                full_ref = np.vstack([ref, np.zeros((1, params.nsec))])
                full_mine = np.vstack([mine, np.zeros((1, params.nsec))])
                err = rel_linf(full_mine, full_ref)
                assert err < 1e-9, (name, k, err, rel_l2(full_mine, full_ref))
    finally:
        disk.close()

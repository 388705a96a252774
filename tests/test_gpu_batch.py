"""The batched ensemble (fargo_batch_*): disks of different sizes and parameters
advanced side by side give, disk by disk, bitwise the results of the same disks
run alone; advance(t_end) brings every disk to t_end with its own DT count."""
import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg

pytestmark = pytest.mark.gpu


def small_ensemble(n=4):
    # the seeded ensemble workload at reduced sizes (Nsec = 3 Nrad)
    return fg.c4_disks(n, seed=7, nrad_choices=(32, 48, 64))


@pytest.mark.parametrize("prec", [fg.FARGO_FP64, fg.FARGO_FP32_BULK])
def test_batched_disks_match_solo_runs(prec):
    disks = small_ensemble()
    assert len({p.nrad for p, _ in disks}) > 1
    batch = fg.Batch(disks, prec)
    batch.run_async(2)
    batch.sync()
    for k, (params, planets) in enumerate(disks):
        solo = fg.Disk(params, planets, prec)
        solo.run(2)
        b = batch.disk(k)
        for name in ("dens", "vrad", "vtheta"):
            assert np.array_equal(b.field(name), solo.field(name)), (k, name)
        assert b.scalars().substeps == solo.scalars().substeps
        pb, ps = b.planets()[0], solo.planets()[0]
        assert (pb.x, pb.y) == (ps.x, ps.y)
        solo.close()
    batch.close()


def test_advance_reaches_t_end_on_every_disk():
    disks = small_ensemble(3)
    disks[1][0].dt = 0.5 * disks[1][0].dt  # a disk with its own DT
    batch = fg.Batch(disks, fg.FARGO_FP32_BULK)
    t_end = 3 * disks[0][0].dt
    nsub = batch.advance(t_end)
    assert nsub == batch.substeps() > 0
    for k in range(len(batch)):
        t = batch.disk(k).scalars().physical_time
        assert abs(t - t_end) <= 1e-9 * t_end, (k, t, t_end)
    # a second call with the same t_end does nothing
    assert batch.advance(t_end) == 0
    batch.close()


def test_batch_variant_is_bitwise_the_default():
    disks = small_ensemble(3)
    v = fg.default_variant()
    v.pad, v.priority, v.pdl = 0, 1, 0
    a = fg.Batch(disks, fg.FARGO_FP32_BULK)
    b = fg.Batch(disks, fg.FARGO_FP32_BULK, variant=v)
    for x in (a, b):
        x.run_async(2)
        x.sync()
    for k in range(len(disks)):
        for name in ("dens", "vrad", "vtheta"):
            assert np.array_equal(a.disk(k).field(name), b.disk(k).field(name)), (k, name)
    a.close()
    b.close()


def test_autotune_keeps_a_variant_at_least_as_fast():
    disks = small_ensemble(4)
    v, best, default = fg.autotune(disks, fg.FARGO_FP32_BULK, ndt=1)
    assert best >= default > 0
    assert set(v.as_dict()) == {"graph", "pdl", "pad", "sg_ahead", "rotate", "az_generic", "priority",
                                "cell_block", "rad_tma", "az_chunks", "rad_col"}
    assert v.priority in (0, 1, 2) and v.pad in (0, 1) and v.pdl in (0, 1)
    assert v.cell_block in (0, 1, 2, 3) and v.rad_tma in (0, 1) and v.az_chunks in (1, 2)


@pytest.mark.parametrize("cell_block,rad_tma,az_chunks", [(1, 0, 1), (2, 1, 1), (3, 0, 1)])
@pytest.mark.parametrize("precision", [fg.FARGO_FP32_BULK, fg.FARGO_FP64])
def test_tile_shapes_are_bitwise_the_default(cell_block, rad_tma, az_chunks, precision):
    # the autotuner's tile and launch shapes change which thread forms a cell, never
    # its arithmetic: fields bitwise equal to the default shapes
    disks = small_ensemble(3)
    v = fg.default_variant()
    v.cell_block, v.rad_tma, v.az_chunks = cell_block, rad_tma, az_chunks
    a = fg.Batch(disks, precision)
    b = fg.Batch(disks, precision, variant=v)
    for x in (a, b):
        x.run_async(2)
        x.sync()
    for k in range(len(disks)):
        for name in ("dens", "vrad", "vtheta"):
            assert np.array_equal(a.disk(k).field(name), b.disk(k).field(name)), (k, name, cell_block)
    a.close()
    b.close()


@pytest.mark.parametrize("by_width", [True, False])
@pytest.mark.parametrize("precision", [fg.FARGO_FP32_BULK, fg.FARGO_FP64])
def test_fused_ensemble_is_bitwise_the_disks_alone(precision, by_width):
    # one launch per substep kernel for the whole ensemble, masked subcycling: every
    # disk still takes its own substeps and ends bitwise where it ends alone
    # widths that take both forms of the CFL kernel (four cells per thread at 288
    # and 384 sectors, the streamed form at 96)
    disks = fg.c4_disks(5, seed=7, nrad_choices=(32, 96, 128))
    assert len({p.nsec for p, _ in disks}) > 1
    b = fg.Batch(disks, precision).fuse(by_width=by_width)
    per_substep, per_dt = b.fused_launches()
    lanes = b.fused_lanes()
    assert lanes == (len({p.nsec for p, _ in disks}) if by_width else 1)
    assert per_substep <= 15 * lanes + 1 and per_dt <= 2
    b.run_async(2)
    b.sync()
    for k, (p, pl) in enumerate(disks):
        d = fg.Disk(p, pl, precision)
        d.run(2)
        assert d.scalars().substeps == b.disk(k).scalars().substeps
        for name in ("dens", "vrad", "vtheta"):
            x, y = d.field(name), b.disk(k).field(name)
            assert np.array_equal(x, y), (k, name, float(np.abs(x - y).max() / np.abs(x).max()))
        pa, pb = d.planets()[0], b.disk(k).planets()[0]
        assert (pa.x, pa.y, pa.vx, pa.vy) == (pb.x, pb.y, pb.vx, pb.vy)
        d.close()
    b.close()


def test_fused_ensemble_adiabatic_and_corotating_disks():
    # the energy equation (sound speed at the DT start, heating and cooling) and a
    # corotating frame (frame correction before the hydro) ride in the same launches
    base = small_ensemble(2)
    disks = []
    for k, (p, pl) in enumerate(base):
        p3, pl3 = fg.load_config("c3", nrad=p.nrad, nsec=p.nsec)
        disks.append((p3, pl3))
        q = fg.FargoParams.from_buffer_copy(p)
        q.corotating = 1
        disks.append((q, pl))
    b = fg.Batch(disks, fg.FARGO_FP64).fuse()
    b.run_async(2)
    b.sync()
    for k, (p, pl) in enumerate(disks):
        d = fg.Disk(p, pl, fg.FARGO_FP64)
        d.run(2)
        for name in ("dens", "vrad", "vtheta", "energy"):
            assert np.array_equal(d.field(name), b.disk(k).field(name)), (k, name)
        d.close()
    b.close()


def test_fuse_rejects_self_gravity():
    p, pl = fg.load_config("c2", nrad=32, nsec=96)
    b = fg.Batch([(p, pl)], fg.FARGO_FP64)
    with pytest.raises(fg.FargoError, match="self-gravity"):
        b.fuse()
    b.close()


def test_two_azimuthal_chunks_per_thread_agree_to_rounding():
    # az_chunks = 2 sums the ring mean of v_theta in another order: FP64 fields agree
    # to rounding with the default after two DTs
    disks = small_ensemble(3)
    v = fg.default_variant()
    v.az_chunks = 2
    a = fg.Batch(disks, fg.FARGO_FP64)
    b = fg.Batch(disks, fg.FARGO_FP64, variant=v)
    for x in (a, b):
        x.run_async(2)
        x.sync()
    for k in range(len(disks)):
        assert a.disk(k).scalars().substeps == b.disk(k).scalars().substeps
        for name in ("dens", "vrad", "vtheta"):
            x, y = a.disk(k).field(name), b.disk(k).field(name)
            assert np.abs(x - y).max() <= 1e-11 * np.abs(x).max(), (k, name)
    a.close()
    b.close()


def test_fused_kernel_times_cover_every_group():
    disks = fg.c4_disks(6, seed=11, nrad_choices=(32, 64))
    b = fg.Batch(disks, fg.FARGO_FP32_BULK).fuse()
    times = b.fused_kernel_times(reps=2)
    per_substep, _ = b.fused_launches()
    assert len(times) == per_substep - 1  # every group but the loop condition
    assert all(ms > 0.0 for _, ms in times)
    names = {name for name, _ in times}
    assert {"kb_cfl_forces", "kb_azimuthal4", "kb_end"} <= names and ("kb_radial_col" in names or "kb_radial" in names)
    b.close()

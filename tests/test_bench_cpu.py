"""bench.py's host-side helpers, without a GPU: algorithmic bytes per launch, the
DRAM traffic read from the committed ncu summaries, the clock record parsed from
nvidia-smi's CSV, and the process environment of a single-GPU run."""
import os
import tempfile

import bench
import cudaprotoplanetarydisks_gb300 as fg


def test_algorithmic_bytes_per_launch():
    p, _ = fg.load_config("c2")
    g = p.nrad * p.nsec
    # isothermal azimuthal sweep: 6 quantities and v_theta in, 5 out
    assert bench.kernel_bytes("k_transport_azimuthal", p, 4) == 11 * g * 4
    p3, _ = fg.load_config("c3")
    g3 = p3.nrad * p3.nsec
    assert bench.kernel_bytes("k_transport_azimuthal", p3, 4) == 13 * g3 * 4
    assert bench.kernel_bytes("k_cfl_forces", p, 8) == 4 * g * 8
    assert bench.kernel_bytes("no_such_kernel", p, 4) == 0


def test_traffic_from_committed_profiles():
    assert bench.ncu_traffic("k_cfl_forces", "c2") == 2.53e6
    assert abs(bench.ncu_traffic("k_transport_azimuthal", "wide") - 377.29e6) < 1.0
    assert bench.ncu_traffic("k_cfl_forces", "no_such_config") is None
    assert bench.ncu_traffic("no_such_kernel", "c2") is None


class _Done:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_record_parsing():
    lines = ["0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
             "0, 2040, 2070, 1350.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
             "0, 2070, 2070, 1000.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
             "garbage line"]
    fd, path = tempfile.mkstemp(suffix=".csv")
    with os.fdopen(fd, "w") as f:
        f.write("\n".join(lines) + "\n")
    s = bench.ClockSampler(0)
    s.proc, s.path = _Done(), path
    rec = s.stop()
    assert rec == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 3, "reasons": ["sw_power_cap"]}
    assert not os.path.exists(path)
    assert bench.ClockSampler(0).stop()["reasons"] == ["nvidia-smi unavailable"]


def test_single_gpu_environment(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_env() == (1, 0, 0)


def test_fp64_profile_columns():
    # profiles/kernels_c3_fp64.md: FP64-pipe warp instructions per launch, DRAM MB
    n = bench.ncu_fp64_instructions("k_transport_azimuthal", "c3")
    assert n is not None and n > 3145728 * 100  # hundreds of FP64 instructions per cell
    assert bench.ncu_fp64_instructions("no_such_kernel", "c3") is None
    t = bench.ncu_traffic("k_transport_radial_tma", "c3", "fp64")
    assert t is not None and 1e8 < t < 1e9
    # the FP32 summary; the timer's generic azimuthal name finds the register form
    t = bench.ncu_traffic("k_transport_azimuthal", "c3", "fp32")
    assert t is not None and 1e7 < t < 1e9


def test_step_algorithmic_bytes():
    p, _ = fg.load_config("c3")
    assert bench.step_alg_bytes(p, 8) == 64 and bench.step_alg_bytes(p, 4) == 32
    p2, _ = fg.load_config("c2")
    assert bench.step_alg_bytes(p2, 8) == 48 + 128


def test_reference_arm_never_loads_the_product(tmp_path):
    # the reference arm runs the reference's own code (its CPU build) and must not
    # map libfargo_gb300.so: run it in a fresh process on the small isothermal disk
    import json
    import subprocess
    import sys
    if not os.path.exists(bench.REF_EXE):
        import pytest
        pytest.skip("the CPU build of the reference is not built here")
    code = ("import sys, json, bench; sys.argv = ['bench.py', '--impl', 'reference', '--config', 'c1', "
            "'--steps', '2', '--warmup', '1']; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print(json.dumps({'product_imported': 'cudaprotoplanetarydisks_gb300' in sys.modules, "
            "'lib_mapped': 'libfargo_gb300' in maps}))")
    r = subprocess.run([sys.executable, "-c", code], cwd=bench.ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    line, probe = lines[0], lines[1]
    assert line["impl"] == "reference" and line["cpu_baseline"]["kind"] == "reference"
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert not probe["product_imported"] and not probe["lib_mapped"]

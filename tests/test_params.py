"""The .par / .cfg interface (ReadVariables src/Interpret.cu:100-212,
InitPlanetarySystem src/Psys.cu:168-217), checked on the host."""
import math
import os

import pytest

import cudaprotoplanetarydisks_gb300 as fg
from cudaprotoplanetarydisks_gb300 import config


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_defaults_match_param_cuh():
    p = config.default_params()
    assert (p.nrad, p.nsec, p.ntot, p.ninterm) == (64, 64, 1501, 10)
    assert p.dt == 1.0 and p.sigma0 == 173.0 and p.aspectratio == 0.05
    assert p.masstaper == 1e-7 and p.adiabaticindex == 1.4 and p.coolingtime0 == 6.28
    assert p.fast_transport == 1 and p.indirect_term == 1 and p.is_disk == 1
    assert p.log_grid == 0 and p.cavityratio == 1.0 and p.transitionratio == 1.0


def test_case_folding_comments_and_flags(tmp_path):
    par = write(tmp_path, "a.par", """
# a comment line
aspectratio\t0.07   trailing words are ignored
SIGMA0 :  2e-3
Nrad 100
nSeC 300
RadialSpacing LOGARITHM
InnerBoundary EVANESCENT
Frame GUIDING-CENTER
Transport STANDARD
Adiabatic YES
AdiabaticIndex 1.66
Cooling YES
IndirectTerm NO
ThicknessSmoothing 0.6
OutputDir out/x/
UnknownKey 42
""")
    p = config.read_par(par)
    assert p.aspectratio == 0.07 and p.sigma0 == 2e-3 and (p.nrad, p.nsec) == (100, 300)
    assert p.log_grid == 1 and p.evanescent == 1 and p.open_inner == 0
    assert p.corotating == 1 and p.guiding_center == 1 and p.fast_transport == 0
    assert p.adiabatic == 1 and p.write_temperature == 1 and p.adiabaticindex == 1.66 and p.cooling == 1
    assert p.indirect_term == 0
    assert p.outputdir == b"out/x/"


def test_string_values_are_exact_words(tmp_path):
    # only LOGARITHM selects the log grid (src/Interpret.cu:136); "L" or "A" is arithmetic
    p = config.read_par(write(tmp_path, "b.par", "RadialSpacing L\nThicknessSmoothing 0.6\n"))
    assert p.log_grid == 0


def test_writedivv_cannot_be_enabled(tmp_path):
    # src/Interpret.cu:74 assigns a number to the string
    p = config.read_par(write(tmp_path, "c.par", "WriteDivV YES\nThicknessSmoothing 0.6\n"))
    assert p.write_divv == 0


def test_adiabatic_index_one_falls_back_to_isothermal(tmp_path):
    p = config.read_par(write(tmp_path, "d.par", "Adiabatic YES\nAdiabaticIndex 1.0\nThicknessSmoothing 0.6\n"))
    assert p.adiabatic == 0


@pytest.mark.parametrize("text", [
    "Viscosity 1e-5\nAlphaViscosity 1e-3\nThicknessSmoothing 0.6\n",
    "ThicknessSmoothing 0.6\nRocheSmoothing 0.5\n",
    "Nrad 10\n",
])
def test_conflicts_the_reference_stops_on(tmp_path, text):
    with pytest.raises(ValueError):
        config.read_par(write(tmp_path, "e.par", text))


def test_missing_file():
    with pytest.raises(FileNotFoundError):
        config.read_par("/nonexistent/file.par")


def test_alpha_and_roche_flags(tmp_path):
    p = config.read_par(write(tmp_path, "f.par", "AlphaViscosity 1e-3\nRocheSmoothing 0.5\n"))
    assert p.viscosity_alpha == 1 and p.roche_smoothing == 1


def test_switches():
    p = config.default_params()
    lib = fg._capi.load()
    import ctypes
    assert lib.fargo_params_apply_switches(b"-cb", ctypes.byref(p)) == 0
    assert p.sloppy_cfl == 1 and p.centrifugal_balance == 1
    assert lib.fargo_params_apply_switches(b"-x", ctypes.byref(p)) == fg._capi.FARGO_ERR_INVALID


def test_planet_table(tmp_path):
    cfg = write(tmp_path, "p.cfg", """# Name Distance Mass Accretion FeelsDisk FeelsOthers
Jupiter   1.0  0.001  0.0  NO  NO
Saturn    2.0  3e-4   0.5  YES yes
# comment
  indented lines are not planets
""")
    par = write(tmp_path, "p.par", f"PlanetConfig {cfg}\nThicknessSmoothing 0.6\nEccentricity 0.1\n")
    p = config.read_par(par)
    pl = config.read_planets(p, par)
    assert len(pl) == 2
    assert pl[0].feel_disk == 0 and pl[0].feel_others == 0 and pl[1].feel_disk == 1 and pl[1].feel_others == 1
    assert pl[1].acc == 0.5 and pl[1].mass == 3e-4
    e = 0.1
    assert pl[0].x == 1.0 * (1.0 + e) and pl[0].y == 0.0
    vy = math.sqrt(1.0 * (1.0 + 0.001) / 1.0) * math.sqrt((1.0 - e) / (1.0 + e))
    assert pl[0].vy == vy and pl[0].vx == -1e-10 * vy


@pytest.mark.parametrize("name", ["c1", "c2", "c3", "wide"])
def test_shipped_workloads_parse(name):
    p, pl = fg.load_config(name)
    assert p.log_grid == 1 and len(pl) == 1
    if name == "c2":
        assert p.self_gravity == 1 and p.viscosity_alpha == 1 and (p.nrad, p.nsec) == (256, 768)
        assert abs(p.sigma0 * 2 * math.pi * 3.6 - 0.02) < 1e-12
    if name == "c3":
        assert p.adiabatic == 1 and p.cooling == 1 and (p.nrad, p.nsec) == (1024, 3072)
    if name == "wide":
        # the reference's in/template4.par setup
        assert p.adiabatic == 1 and p.cooling == 0 and (p.nrad, p.nsec) == (2048, 4096)
        assert p.non_reflecting == 1 and p.corotating == 1 and p.guiding_center == 1


def test_ensemble_draws_are_seeded():
    a = fg.c4_disks(8, seed=3)
    b = fg.c4_disks(8, seed=3)
    c = fg.c4_disks(8, seed=4)
    key = lambda d: [(p.nrad, p.nsec, p.alphaviscosity, p.aspectratio, p.sigmaslope, pl[0].mass) for p, pl in d]  # noqa: E731
    assert key(a) == key(b) != key(c)
    for p, pl in a:
        assert p.nsec == 3 * p.nrad and p.nrad in fg.config.C4_NRAD and len(pl) == 1
        assert 1e-5 <= pl[0].mass <= 3e-3 and 0.03 <= p.aspectratio <= 0.08

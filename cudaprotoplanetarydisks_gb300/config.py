"""The reference's .par / .cfg parameter interface, through the C-ABI parser.

read_par mirrors ReadVariables (src/Interpret.cu:100-212); read_planets mirrors
InitPlanetarySystem (src/Psys.cu:168-217).  The workloads of the benchmark and
of the parity tests are shipped as .par/.cfg files in configs/.
"""
import ctypes
import os

from . import _capi

CONFIG_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "configs")

NAMED = {
    "c1": "c1_isothermal.par",
    "c2": "c2_selfgravity.par",
    "c3": "c3_adiabatic.par",
    "wide": "wide_template4.par",
}


def default_params():
    p = _capi.FargoParams()
    _capi.load().fargo_params_default(ctypes.byref(p))
    return p


def read_par(path, switches=None):
    """Parse a .par file; switches is an optional CLI switch string such as "-c"."""
    lib = _capi.load()
    p = default_params()
    rc = lib.fargo_params_read(os.fsencode(path), ctypes.byref(p))
    if rc == _capi.FARGO_ERR_IO:
        raise FileNotFoundError(path)
    if rc != _capi.FARGO_OK:
        raise ValueError(f"{path}: conflicting parameters (status {rc})")
    if switches:
        rc = lib.fargo_params_apply_switches(switches.encode(), ctypes.byref(p))
        if rc != _capi.FARGO_OK:
            raise ValueError(f"bad switches {switches!r}")
    return p


def resolve_planet_config(params, par_path=None):
    """PlanetConfig is relative to the working directory in the reference; fall back
    to the directory of the .par file."""
    name = params.planetconfig.decode()
    if os.path.exists(name):
        return name
    if par_path is not None:
        cand = os.path.join(os.path.dirname(os.path.abspath(par_path)), name)
        if os.path.exists(cand):
            return cand
    raise FileNotFoundError(name)


def read_planets(params, par_path=None, cap=64):
    lib = _capi.load()
    path = resolve_planet_config(params, par_path)
    arr = (_capi.FargoPlanet * cap)()
    nb = ctypes.c_int(0)
    rc = lib.fargo_planets_read(os.fsencode(path), ctypes.byref(params), arr, cap, ctypes.byref(nb))
    if rc != _capi.FARGO_OK:
        raise ValueError(f"{path}: cannot read planets (status {rc})")
    return [arr[k] for k in range(nb.value)]


def load_config(name_or_path, **overrides):
    """(params, planets) of a named workload (c1, c2, c3, wide) or of a .par path.
    Keyword overrides set FargoParams members (e.g. nrad=64, nsec=192)."""
    path = name_or_path
    if name_or_path in NAMED:
        path = os.path.join(CONFIG_DIR, NAMED[name_or_path])
    params = read_par(path)
    planets = read_planets(params, path)
    for k, v in overrides.items():
        if isinstance(v, str):
            v = v.encode()
        setattr(params, k, v)
    # the switches the .par reader derives from these values (fargo_params_read's
    # last step, after src/Interpret.cu's checks)
    if "alphaviscosity" in overrides or "viscosity" in overrides:
        if params.alphaviscosity != 0.0 and params.viscosity != 0.0:
            raise ValueError("VISCOSITY and ALPHAVISCOSITY cannot both be set")
        params.viscosity_alpha = 1 if params.alphaviscosity != 0.0 else 0
    if "rochesmoothing" in overrides or "thicknesssmoothing" in overrides:
        if params.thicknesssmoothing != 0.0 and params.rochesmoothing != 0.0:
            raise ValueError("THICKNESSSMOOTHING and ROCHESMOOTHING cannot both be set")
        params.roche_smoothing = 1 if params.rochesmoothing != 0.0 else 0
    return params, planets


# the batched-ensemble workload: sizes and the seeded per-disk parameter draws
C4_NRAD = (128, 192, 256, 384, 512)


def c4_draws(n=64, seed=2024, nrad_choices=C4_NRAD):
    """The seeded per-disk draws of the ensemble workload, one dict per disk:
    nrad uniform in nrad_choices (nsec = 3 nrad); planet mass ratio q log-uniform in
    [1e-5, 3e-3]; alpha viscosity log-uniform in [1e-4, 1e-2]; aspect ratio h
    uniform in [0.03, 0.08]; Sigma slope uniform in [0, 1.5]; the disk's noise seed."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n):
        nrad = int(rng.choice(nrad_choices))
        q = float(10 ** rng.uniform(np.log10(1e-5), np.log10(3e-3)))
        alpha = float(10 ** rng.uniform(-4.0, -2.0))
        h = float(rng.uniform(0.03, 0.08))
        slope = float(rng.uniform(0.0, 1.5))
        out.append({"nrad": nrad, "nsec": 3 * nrad, "q": q, "alpha": alpha, "h": h, "slope": slope,
                    "noise_seed": seed * 1000 + k + 1})
    return out


def c4_disks(n=64, seed=2024, nrad_choices=C4_NRAD, sigma_noise=1e-4):
    """(params, planets) of n seeded disks: the isothermal c1 setup (log grid on
    [0.4, 2.5], one planet on a fixed circular orbit at r = 1, FARGO transport)
    with the per-disk draws of c4_draws, no uniform viscosity, Sigma0 = 6.3662e-4
    and density noise of relative amplitude sigma_noise seeded per disk."""
    out = []
    for d in c4_draws(n, seed, nrad_choices):
        params, planets = load_config("c1", nrad=d["nrad"], nsec=d["nsec"], viscosity=0.0, alphaviscosity=d["alpha"],
                                      aspectratio=d["h"], sigmaslope=d["slope"], sigma0=6.3662e-4,
                                      noise_seed=d["noise_seed"], sigma_noise=sigma_noise)
        set_planet_mass(params, planets[0], d["q"])
        out.append((params, planets))
    return out


def set_planet_mass(params, planet, mass):
    """A planet of the planet file read with another mass: the mass and the initial
    velocity that InitPlanetarySystem derives from it (src/Psys.cu: vy =
    sqrt((1 + m) / d) sqrt((1 - e) / (1 + e)), vx = -1e-10 vy, d the file's
    distance, here x / (1 + e), exact for the circular orbits of the workloads)."""
    import math
    e = params.eccentricity
    dist = planet.x / (1.0 + e)
    planet.mass = mass
    planet.vy = math.sqrt(1.0 * (1.0 + mass) / dist) * math.sqrt((1.0 - e) / (1.0 + e))
    planet.vx = -0.0000000001 * planet.vy

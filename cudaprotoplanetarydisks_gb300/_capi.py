"""ctypes view of include/fargo_gb300.h (the C-ABI of libfargo_gb300.so)."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfargo_gb300.so")

FARGO_OK = 0
FARGO_ERR_INVALID = 1
FARGO_ERR_CUDA = 2
FARGO_ERR_IO = 3
FARGO_ERR_NUMERIC = 4
FARGO_ERR_STATE = 5

FARGO_FP64 = 0
FARGO_FP32_BULK = 1
FORCE_LEVELS = 11  # FARGO_FORCE_LEVELS: the reference's dimfxy

SUB_BOUNDARY = 1
SUB_SOURCE = 2
SUB_ENERGY = 3
SUB_TRANSPORT = 4
SUB_TEMPERATURE = 5
SUB_SOUNDSPEED = 6
SUB_POTENTIAL = 7

FIELDS = {
    "dens": 0, "vrad": 1, "vtheta": 2, "energy": 3, "temperature": 4,
    "pressure": 5, "soundspeed": 6, "potential": 7, "qplus": 8,
    "divergence": 9, "sg_accr": 10, "sg_acct": 11,
}

_D = ctypes.c_double
_I = ctypes.c_int


class FargoParams(ctypes.Structure):
    _fields_ = [
        ("nrad", _I), ("nsec", _I), ("rmin", _D), ("rmax", _D), ("log_grid", _I),
        ("dt", _D), ("ntot", _I), ("ninterm", _I),
        ("sigma0", _D), ("sigmaslope", _D), ("aspectratio", _D), ("flaringindex", _D),
        ("viscosity", _D), ("alphaviscosity", _D), ("imposeddiskdrift", _D), ("eccentricity", _D),
        ("cavityradius", _D), ("cavityratio", _D), ("cavitywidth", _D),
        ("transitionradius", _D), ("transitionratio", _D), ("transitionwidth", _D),
        ("lambdadoubling", _D), ("adiabaticindex", _D), ("coolingtime0", _D),
        ("thicknesssmoothing", _D), ("rochesmoothing", _D), ("masstaper", _D),
        ("releaseradius", _D), ("releasedate", _D), ("omegaframe", _D),
        ("fast_transport", _I), ("open_inner", _I), ("non_reflecting", _I), ("evanescent", _I),
        ("is_disk", _I), ("corotating", _I), ("guiding_center", _I), ("indirect_term", _I),
        ("exclude_hill", _I), ("self_gravity", _I), ("sg_zero_mode", _I),
        ("adiabatic", _I), ("cooling", _I), ("cic_planet", _I), ("forced_circular", _I),
        ("viscosity_alpha", _I), ("roche_smoothing", _I), ("advect_label", _I),
        ("outer_source_mass", _I),
        ("write_density", _I), ("write_velocity", _I), ("write_energy", _I),
        ("write_temperature", _I), ("write_divv", _I), ("write_qplus", _I),
        ("sloppy_cfl", _I), ("centrifugal_balance", _I), ("scaling_factor", _D),
        ("outputdir", ctypes.c_char * 512), ("planetconfig", ctypes.c_char * 512),
        ("sigma_noise", _D), ("energy_noise", _D), ("noise_seed", ctypes.c_ulonglong),
    ]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = v.decode() if isinstance(v, bytes) else v
        return out


class FargoPlanet(ctypes.Structure):
    _fields_ = [("x", _D), ("y", _D), ("vx", _D), ("vy", _D), ("mass", _D), ("acc", _D),
                ("feel_disk", _I), ("feel_others", _I)]


class FargoVariant(ctypes.Structure):
    """fargo_variant: the execution variant of a context (bitwise-equal results)."""
    _fields_ = [("graph", ctypes.c_int), ("pdl", ctypes.c_int), ("pad", ctypes.c_int), ("sg_ahead", ctypes.c_int),
                ("rotate", ctypes.c_int), ("az_generic", ctypes.c_int), ("priority", ctypes.c_int),
                ("cell_block", ctypes.c_int), ("rad_tma", ctypes.c_int), ("az_chunks", ctypes.c_int),
                ("rad_col", ctypes.c_int)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class FargoScalars(ctypes.Structure):
    _fields_ = [("physical_time", _D), ("omega_frame", _D), ("lost_mass", _D),
                ("last_dt", _D), ("substeps", ctypes.c_longlong), ("last_cfl", _I), ("nb", _I),
                ("launches_per_substep", _I), ("launches_per_dt", _I), ("padded_substeps", ctypes.c_longlong)]


_DP = ctypes.POINTER(_D)
_P = ctypes.c_void_p

# (name, restype, argtypes) for every entry point declared in include/fargo_gb300.h
SIGNATURES = [
    ("fargo_params_default", None, [ctypes.POINTER(FargoParams)]),
    ("fargo_params_read", _I, [ctypes.c_char_p, ctypes.POINTER(FargoParams)]),
    ("fargo_params_apply_switches", _I, [ctypes.c_char_p, ctypes.POINTER(FargoParams)]),
    ("fargo_planets_read", _I, [ctypes.c_char_p, ctypes.POINTER(FargoParams),
                                ctypes.POINTER(FargoPlanet), _I, ctypes.POINTER(_I)]),
    ("fargo_ctx_create", _I, [ctypes.POINTER(FargoParams), ctypes.POINTER(FargoPlanet), _I, _I,
                              _P, ctypes.POINTER(_P)]),
    ("fargo_ctx_destroy", None, [_P]),
    ("fargo_last_error", ctypes.c_char_p, [_P]),
    ("fargo_get_fields", _I, [_P, _DP, _DP, _DP, _DP, _DP]),
    ("fargo_set_fields", _I, [_P, _DP, _DP, _DP, _DP]),
    ("fargo_get_field", _I, [_P, _I, _DP]),
    ("fargo_get_field_device", _I, [_P, _I, _P]),
    ("fargo_get_planets", _I, [_P, ctypes.POINTER(FargoPlanet), _I, ctypes.POINTER(_I)]),
    ("fargo_get_scalars", _I, [_P, ctypes.POINTER(FargoScalars)]),
    ("fargo_get_mesh", _I, [_P, _DP, _DP, _DP, _DP]),
    ("fargo_step_DT", _I, [_P, ctypes.POINTER(_I)]),
    ("fargo_run", _I, [_P, _I, ctypes.POINTER(ctypes.c_longlong)]),
    ("fargo_run_async", _I, [_P, _I]),
    ("fargo_sync", _I, [_P]),
    ("fargo_substep_full", _I, [_P, _D]),
    ("fargo_substep", _I, [_P, _I, _D]),
    ("fargo_condition_cfl", _I, [_P, _D, ctypes.POINTER(_I)]),
    ("fargo_write_outputs", _I, [_P, _I]),
    ("fargo_write_dims", _I, [_P]),
    ("fargo_restart", _I, [_P, _I]),
    ("fargo_compute_force", _I, [_P, _D, _D, _D, _D, _D, _D, ctypes.POINTER(_D)]),
    ("fargo_update_log", _I, [_P, _I]),
    ("fargo_time_substep_kernels", _I, [_P, _I, _DP, _I, ctypes.POINTER(_I)]),
    ("fargo_substep_kernel_name", ctypes.c_char_p, [_P, _I]),
    ("fargo_fp64_pipe_peak", _I, [ctypes.POINTER(_D)]),
    ("fargo_div_selftest", _I, [ctypes.POINTER(_D), ctypes.POINTER(_D), _I, ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    ("fargo_tc_selftest", _I, [_P, _P, _I, _I, _I, _P]),
    ("fargo_condition_cfl_noalloc", _I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _D, _P, _P]),
    ("fargo_batch_create", _I, [_I, ctypes.POINTER(FargoParams), ctypes.POINTER(FargoPlanet), ctypes.POINTER(_I),
                                _I, ctypes.POINTER(_P)]),
    ("fargo_batch_create_variant", _I, [_I, ctypes.POINTER(FargoParams), ctypes.POINTER(FargoPlanet),
                                        ctypes.POINTER(_I), _I, ctypes.POINTER(FargoVariant), ctypes.POINTER(_P)]),
    ("fargo_batch_autotune", _I, [_I, ctypes.POINTER(FargoParams), ctypes.POINTER(FargoPlanet), ctypes.POINTER(_I),
                                  _I, _I, ctypes.POINTER(FargoVariant), ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    ("fargo_variant_default", None, [ctypes.POINTER(FargoVariant)]),
    ("fargo_ctx_create_variant", _I, [ctypes.POINTER(FargoParams), ctypes.POINTER(FargoPlanet), _I, _I, _P,
                                      ctypes.POINTER(FargoVariant), ctypes.POINTER(_P)]),
    ("fargo_batch_destroy", None, [_P]),
    ("fargo_batch_size", _I, [_P]),
    ("fargo_batch_disk", _P, [_P, _I]),
    ("fargo_batch_run_async", _I, [_P, _I]),
    ("fargo_batch_sync", _I, [_P]),
    ("fargo_batch_fuse", _I, [_P]),
    ("fargo_batch_last_error", ctypes.c_char_p, [_P]),
    ("fargo_batch_fused_launches", _I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("fargo_batch_fuse_by_width", _I, [_P, _I]),
    ("fargo_batch_fused_lanes", _I, [_P, ctypes.POINTER(_I)]),
    ("fargo_batch_fused_time_kernels", _I, [_P, _I, ctypes.POINTER(_D), _I, ctypes.POINTER(_I)]),
    ("fargo_batch_fused_kernel_name", ctypes.c_char_p, [_P, _I]),
    ("fargo_batch_advance", _I, [_P, _D, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(_I)]),
    ("fargo_mlp_create", _I, [_I, ctypes.POINTER(_P)]),
    ("fargo_mlp_destroy", None, [_P]),
    ("fargo_mlp_set_params", _I, [_P, ctypes.POINTER(ctypes.c_float)]),
    ("fargo_mlp_get_params", _I, [_P, ctypes.POINTER(ctypes.c_float)]),
    ("fargo_mlp_get_grad", _I, [_P, ctypes.POINTER(ctypes.c_float)]),
    ("fargo_mlp_forward", _I, [_P, _P, _I, _P, _I, _P]),
    ("fargo_mlp_set_tensor_path", _I, [_P, _I]),
    ("fargo_mlp_status", _I, [_P]),
    ("fargo_mlp_backward", _I, [_P, _P, _I, _P, _P]),
    ("fargo_mlp_adam", _I, [_P, ctypes.c_float, _P]),
    ("fargo_learned_features", _I, [_I, _P, _P, _P, _P, _I, _I, _D, ctypes.POINTER(ctypes.c_float), _P, _P]),
    ("fargo_learned_divergence", _I, [_P, _P, _I, _I, ctypes.c_float, _P, _P]),
    ("fargo_learned_ring_center", _I, [_P, _I, _I, _P]),
    ("fargo_learned_divergence_limited", _I, [_P, _P, ctypes.c_float, ctypes.c_float, _P]),
    ("fargo_learned_loss", _I, [_P, _P, _P, _I, _I, ctypes.c_float, ctypes.c_float, _P, _P, _P, _P, _P, _P]),
    ("fargo_learned_restrict", _I, [_P, _P, _I]),
    ("fargo_learned_apply", _I, [_P, _P, ctypes.POINTER(_I), ctypes.POINTER(_D)]),
    ("fargo_learned_features_ctx", _I, [_P, ctypes.POINTER(ctypes.c_float), _P]),
    ("fargo_learned_density", _I, [_P, _P]),
]

_lib = None


def load(path=None):
    """Load libfargo_gb300.so; raise (never fall back) when it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(p)
    lib.missing_symbols = []
    for name, res, args in SIGNATURES:
        try:
            fn = getattr(lib, name)
        except AttributeError:
            lib.missing_symbols.append(name)
            continue
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib

"""C-ABI checks that need no GPU: the library loads, exports every entry point of
include/fargo_gb300.h, and the ctypes layout matches the C layout."""
import ctypes
import os
import re
import subprocess
import tempfile

from cudaprotoplanetarydisks_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fargo_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fargo_[a-z_A-Z0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = _capi.load()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.missing_symbols == []


def test_ctypes_signatures_cover_header():
    assert sorted(n for n, _, _ in _capi.SIGNATURES) == declared_functions()


def test_struct_layout_matches_c():
    fields = [f for f, _ in _capi.FargoParams._fields_]
    prog = ["#include <stdio.h>", "#include <stddef.h>", '#include "fargo_gb300.h"', "int main(void){",
            'printf("%zu %zu %zu\\n", sizeof(fargo_params), sizeof(fargo_planet), sizeof(fargo_scalars));']
    for f in fields:
        prog.append(f'printf("%zu\\n", offsetof(fargo_params, {f}));')
    prog.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write("\n".join(prog))
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    sizes = [int(x) for x in out[:3]]
    assert sizes == [ctypes.sizeof(_capi.FargoParams), ctypes.sizeof(_capi.FargoPlanet),
                     ctypes.sizeof(_capi.FargoScalars)]
    offs = [int(x) for x in out[3:]]
    assert offs == [getattr(_capi.FargoParams, f).offset for f in fields]


def test_invalid_create_is_rejected_without_gpu_work():
    lib = _capi.load()
    p = _capi.FargoParams()
    lib.fargo_params_default(ctypes.byref(p))
    p.nrad = 2  # too small: rejected before any device call
    h = ctypes.c_void_p()
    assert lib.fargo_ctx_create(ctypes.byref(p), None, 0, 0, None, ctypes.byref(h)) == _capi.FARGO_ERR_INVALID
    p.nrad = 64
    assert lib.fargo_ctx_create(ctypes.byref(p), None, 0, 7, None, ctypes.byref(h)) == _capi.FARGO_ERR_INVALID
    assert lib.fargo_ctx_create(ctypes.byref(p), None, -1, 0, None, ctypes.byref(h)) == _capi.FARGO_ERR_INVALID
    assert lib.fargo_last_error(None) == b"no context"


def test_variant_layout_and_default_switches(monkeypatch):
    prog = ["#include <stdio.h>", '#include "fargo_gb300.h"',
            'int main(void){printf("%zu\\n", sizeof(fargo_variant)); return 0;}']
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "v.c")
        open(c, "w").write("\n".join(prog))
        exe = os.path.join(d, "v")
        subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        size = int(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)
    assert size == ctypes.sizeof(_capi.FargoVariant)
    lib = _capi.load()
    for name in ("FARGO_NO_GRAPH", "FARGO_NO_PDL", "FARGO_NO_PAD", "FARGO_NO_SG_AHEAD", "FARGO_ROTATE",
                 "FARGO_AZ_GENERIC", "FARGO_PRIO", "FARGO_CELL_BLOCK", "FARGO_NO_TMA", "FARGO_AZ_CHUNKS2", "FARGO_RAD_COL"):
        monkeypatch.delenv(name, raising=False)
    v = _capi.FargoVariant()
    lib.fargo_variant_default(ctypes.byref(v))
    assert v.as_dict() == {"graph": 1, "pdl": 1, "pad": 1, "sg_ahead": 1, "rotate": 0, "az_generic": 0,
                           "priority": 0, "cell_block": 0, "rad_tma": 1, "az_chunks": 1, "rad_col": -1}
    monkeypatch.setenv("FARGO_NO_PAD", "1")
    monkeypatch.setenv("FARGO_ROTATE", "1")
    monkeypatch.setenv("FARGO_PRIO", "2")
    lib.fargo_variant_default(ctypes.byref(v))
    assert (v.pad, v.rotate, v.priority, v.graph) == (0, 1, 2, 1)
    # an unknown priority mode is rejected before any device call
    p = _capi.FargoParams()
    lib.fargo_params_default(ctypes.byref(p))
    p.nrad = 64
    v.priority = 5
    h = ctypes.c_void_p()
    assert lib.fargo_ctx_create_variant(ctypes.byref(p), None, 0, 0, None, ctypes.byref(v),
                                        ctypes.byref(h)) == _capi.FARGO_ERR_INVALID
    # so are unknown tile shapes
    lib.fargo_variant_default(ctypes.byref(v))
    for field, bad in (("cell_block", 4), ("az_chunks", 3), ("az_chunks", 0), ("rad_col", 2)):
        w = _capi.FargoVariant.from_buffer_copy(v)
        setattr(w, field, bad)
        assert lib.fargo_ctx_create_variant(ctypes.byref(p), None, 0, 0, None, ctypes.byref(w),
                                            ctypes.byref(h)) == _capi.FARGO_ERR_INVALID

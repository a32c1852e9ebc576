"""The C-ABI library loads and exports every entry point its headers declare.
No compute call is made here (no GPU is needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(lbm_\w+)\s*\(", text)
    return sorted(set(names))


def test_headers_declare_the_api():
    names = declared_functions()
    for required in ("lbm_gpu_create", "lbm_gpu_step", "lbm_gpu_residual", "lbm_gpu_get_populations", "lbm_gpu_create_box"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from lbm_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from lbm_gb300 import build
        build.build()
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    lib.lbm_gpu_abi_version.restype = ctypes.c_int
    assert lib.lbm_gpu_abi_version() == 1


def test_invalid_arguments_are_rejected_without_a_gpu():
    from lbm_gb300 import _lib
    lib = _lib.load()
    assert lib.lbm_gpu_create(None, None, None, None) == -1
    assert lib.lbm_gpu_step(None, 1) == -1
    assert lib.lbm_gpu_create_box(None, None, None, None) == -1


def test_grid_and_particle_entry_points_reject_invalid_arguments_without_a_gpu():
    import ctypes as C

    from lbm_gb300 import _lib, gridgen
    from lbm_gb300.lpt import _lpt_lib

    lib = gridgen._grid_lib()
    h = C.c_void_p()
    assert lib.lbm_grid_create(0, 5, None, 0, None, C.byref(h)) == -1           # no dimension
    assert lib.lbm_grid_create(2, 5, None, 0, None, C.byref(h)) == -1           # no geometry and no box
    descs, _ = gridgen.geometry_objects({"b": {"type": "box", "A": [0, 0, 0], "B": [1, 1, 1]}}, 3)
    # 2^33 positions: more than the device build takes; refused before any CUDA call
    assert lib.lbm_grid_create_device(3, 11, C.cast(descs, C.c_void_p), 1, None, 0, C.byref(h)) == -2
    bad = gridgen.GeomDesc()
    bad.kind = 7
    assert lib.lbm_grid_create(2, 3, C.byref(bad), 1, None, C.byref(h)) == -2   # unknown object kind
    assert lib.lbm_grid_align(None, 0) == -1
    assert lib.lbm_grid_ncells(None) == 0
    lp = _lpt_lib()
    assert lp.lbm_lpt_create(None, C.byref(h)) == -1
    assert lp.lbm_lpt_step(None, 1) == -1
    assert lp.lbm_lpt_set_particles(None, 0, None) == -1
    assert lp.lbm_lpt_count(None) == 0

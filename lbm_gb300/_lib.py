"""ctypes binding of the C ABI in include/lbm_gpu.h and include/lbm_gpu_box.h.

The CUDA library is the only implementation of the step: if it cannot be
loaded the import of a solver raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblbm_gpu.so")

LBM_OK = 0
STATUS = {0: "LBM_OK", -1: "LBM_ERR_INVALID", -2: "LBM_ERR_UNSUPPORTED", -3: "LBM_ERR_TABLE", -4: "LBM_ERR_CUDA",
          -5: "LBM_ERR_DIVERGED", -6: "LBM_ERR_TIMEOUT", -7: "LBM_ERR_NOMEM"}


class LBMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class TableDesc(C.Structure):
    _fields_ = [("lattice", C.c_int32), ("equation", C.c_int32), ("ncells", C.c_int64), ("nnghbr", C.c_int32),
                ("device", C.c_int32), ("omega", C.c_double), ("relax_time", C.c_double), ("dt", C.c_double),
                ("poisson_k", C.c_double), ("bbox", C.c_double * 6), ("cell_length", C.c_double)]


class BndDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("has_vec", C.c_int32), ("has_pressure", C.c_int32), ("reserved", C.c_int32),
                ("ncells", C.c_int64), ("cells", C.c_void_p), ("normals", C.c_void_p), ("values", C.c_void_p),
                ("vec", C.c_double * 3), ("scalar", C.c_double), ("nconn", C.c_int64), ("conn_cells", C.c_void_p),
                ("conn_normals", C.c_void_p)]


class BoxDesc(C.Structure):
    _fields_ = [("lattice", C.c_int32), ("equation", C.c_int32), ("storage", C.c_int32), ("device", C.c_int32),
                ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("face", C.c_int32 * 6), ("omega", C.c_double),
                ("wall_velocity", (C.c_double * 3) * 6), ("body_force", C.c_double * 3), ("inlet_density", C.c_double),
                ("inlet_velocity", C.c_double * 3), ("init_density", C.c_double), ("init_velocity", C.c_double * 3),
                ("kappa_sq", C.c_double), ("pb_nonlinear", C.c_int32), ("no_shift", C.c_int32)]


class BatchDesc(C.Structure):
    _fields_ = [("lattice", C.c_int32), ("storage", C.c_int32), ("device", C.c_int32), ("ndomains", C.c_int32),
                ("lid_velocity", C.c_double)]


_lib = None
_lock = threading.Lock()

# name -> (restype, argtypes)
_SIGS = {
    "lbm_gpu_abi_version": (C.c_int, []),
    "lbm_gpu_create": (C.c_int, [C.POINTER(TableDesc), C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "lbm_gpu_add_boundary": (C.c_int, [C.c_void_p, C.POINTER(BndDesc)]),
    "lbm_gpu_set_forcing": (C.c_int, [C.c_void_p, C.c_double, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]),
    "lbm_gpu_initial_condition": (C.c_int, [C.c_void_p]),
    "lbm_gpu_step": (C.c_int, [C.c_void_p, C.c_int64]),
    "lbm_gpu_residual": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_gpu_update_moments": (C.c_int, [C.c_void_p]),
    "lbm_gpu_get_vars": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_gpu_set_vars": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_gpu_get_varsold": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_gpu_get_populations": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_gpu_set_populations": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_gpu_reduce_mass_momentum": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_gpu_synchronize": (C.c_int, [C.c_void_p]),
    "lbm_gpu_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "lbm_gpu_last_error": (C.c_char_p, [C.c_void_p]),
    "lbm_gpu_destroy": (None, [C.c_void_p]),
    "lbm_gpu_create_box": (C.c_int, [C.POINTER(BoxDesc), C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "lbm_gpu_box_moments": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "lbm_gpu_box_probe": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "lbm_gpu_box_autotune": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "lbm_gpu_box_select_kernel": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "lbm_gpu_box_kernels": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "lbm_gpu_box_test_wait": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32]),
    "lbm_gpu_box_set_slice_omega": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "lbm_gpu_box_set_slice_kappa": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "lbm_gpu_box_storage_bytes": (C.c_int, [C.c_int32]),
    "lbm_gpu_create_batch": (C.c_int, [C.POINTER(BatchDesc), C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "lbm_gpu_batch_residuals": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_gpu_batch_run": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_double, C.c_void_p]),
    "lbm_gpu_batch_get_domain": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "lbm_gpu_batch_status": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lbm_gpu_batch_profile_steps": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                              C.POINTER(C.c_int64)]),
    "lbm_gpu_batch_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "lbm_gpu_residual_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p]),
    "lbm_gpu_box_profile_steps": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                            C.POINTER(C.c_int64)]),
    "lbm_gpu_box_time_steps": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double)]),
}


def load(path: str = LIB_PATH):
    """Load the CUDA library.  Raises if it was not built (``__graft_entry__.build``
    or ``python lbm_gb300/build.py``)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise RuntimeError(f"CUDA library not built: {path} (run python lbm_gb300/build.py)")
            lib = C.CDLL(path)
            for name, (res, args) in _SIGS.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(rc: int, ctx=None, what: str = ""):
    if rc != LBM_OK:
        msg = ""
        if ctx:
            raw = load().lbm_gpu_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise LBMError(rc, f"{what}: {msg}")

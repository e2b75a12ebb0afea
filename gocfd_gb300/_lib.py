"""ctypes binding of libgcfd (include/gcfd.h).

The library is built in-tree (``gocfd_gb300/libgcfd.so``).  There is no CPU
fallback: if the shared library is missing or was built for another machine,
``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

GCFD_OK = 0
ERRORS = {
    -1: "GCFD_ERR_ARG",
    -2: "GCFD_ERR_SHAPE",
    -3: "GCFD_ERR_CUDA",
    -4: "GCFD_ERR_NAN",
    -5: "GCFD_ERR_TIMEOUT",
    -6: "GCFD_ERR_OOM",
    -7: "GCFD_ERR_UNSUPPORTED",
}

# Every symbol declared in include/gcfd.h.
EXPORTS = [
    "gcfd_create", "gcfd_destroy", "gcfd_last_error", "gcfd_dims", "gcfd_set_state",
    "gcfd_get_state", "gcfd_set_state_device", "gcfd_get_state_device", "gcfd_set_time",
    "gcfd_get_time", "gcfd_rhs", "gcfd_step", "gcfd_enqueue_steps", "gcfd_get_stream", "gcfd_set_option",
    "gcfd_get_option", "gcfd_profile_step",
    "gcfd_host_operator", "gcfd_read_mesh", "gcfd_free_mesh", "gcfd_residual_norms_static", "gcfd_functional", "gcfd_rhs_vjp",
    "gcfd_record_steps", "gcfd_step_vjp", "gcfd_sample_points", "gcfd_wall_points", "gcfd_device_fma_peaks",
    "gcfd_host_graph_element", "gcfd_graph_mesh", "gcfd_graph_fields",
]


class GcfdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Mesh(C.Structure):
    _fields_ = [
        ("nverts", C.c_int32), ("vx", C.POINTER(C.c_double)), ("vy", C.POINTER(C.c_double)),
        ("K", C.c_int32), ("etov", C.POINTER(C.c_int32)),
        ("nbc", C.c_int32), ("bc_v1", C.POINTER(C.c_int32)), ("bc_v2", C.POINTER(C.c_int32)),
        ("bc_flag", C.POINTER(C.c_int32)),
    ]


class Params(C.Structure):
    _fields_ = [
        ("N", C.c_int32), ("cfl", C.c_double), ("final_time", C.c_double), ("minf", C.c_double),
        ("gamma", C.c_double), ("alpha", C.c_double), ("kappa", C.c_double),
        ("max_iterations", C.c_int32), ("flux_type", C.c_int32), ("init_type", C.c_int32),
        ("limiter", C.c_int32), ("local_time_stepping", C.c_int32), ("precision", C.c_int32),
        ("vortex_x0", C.c_double), ("vortex_y0", C.c_double), ("device", C.c_int32),
    ]


_lib = None
_lock = threading.Lock()
PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int32)


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libgcfd.so (building it first when absent); raise if impossible."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"libgcfd.so not built at {path}")
            _build.build()
        lib = C.CDLL(path)
        for name in EXPORTS:
            getattr(lib, name)  # raises AttributeError when a symbol is missing
        lib.gcfd_create.argtypes = [C.POINTER(Mesh), C.POINTER(Params), C.POINTER(C.c_void_p)]
        lib.gcfd_destroy.argtypes = [C.c_void_p]
        lib.gcfd_last_error.argtypes = [C.c_void_p]
        lib.gcfd_last_error.restype = C.c_char_p
        lib.gcfd_dims.argtypes = [C.c_void_p, PI, PI, PI, PI, PI]
        lib.gcfd_set_state.argtypes = [C.c_void_p, C.c_int32, PI, C.POINTER(PD)]
        lib.gcfd_get_state.argtypes = [C.c_void_p, C.c_int32, PI, C.POINTER(PD)]
        lib.gcfd_set_state_device.argtypes = [C.c_void_p, C.c_void_p]
        lib.gcfd_get_state_device.argtypes = [C.c_void_p, C.c_void_p]
        lib.gcfd_set_time.argtypes = [C.c_void_p, C.c_double]
        lib.gcfd_get_time.argtypes = [C.c_void_p, PD, PI]
        lib.gcfd_rhs.argtypes = [C.c_void_p, C.c_double, C.c_int32, PI, C.POINTER(PD), C.POINTER(PD)]
        lib.gcfd_step.argtypes = [C.c_void_p, C.c_int32, PD, PD, PD, PD, PD]
        lib.gcfd_enqueue_steps.argtypes = [C.c_void_p, C.c_int32]
        lib.gcfd_get_stream.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        lib.gcfd_set_option.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        lib.gcfd_get_option.argtypes = [C.c_void_p, C.c_int32, PI]
        lib.gcfd_profile_step.argtypes = [C.c_void_p, PD, PI]
        lib.gcfd_host_operator.argtypes = [C.c_int32, C.c_int32, PD, PI, PI]
        lib.gcfd_read_mesh.argtypes = [C.c_char_p, C.POINTER(Mesh)]
        lib.gcfd_free_mesh.argtypes = [C.POINTER(Mesh)]
        lib.gcfd_free_mesh.restype = None
        lib.gcfd_residual_norms_static.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, PD, PD, PD]
        lib.gcfd_functional.argtypes = [C.c_void_p, C.c_int32, PD, C.c_int32, PI, C.POINTER(PD), PD]
        lib.gcfd_rhs_vjp.argtypes = [C.c_void_p, C.c_double, C.c_int32, PI, C.POINTER(PD), C.POINTER(PD),
                                     C.POINTER(PD), PD, PD]
        lib.gcfd_record_steps.argtypes = [C.c_void_p, C.c_int32, C.c_int32, PD, PD]
        lib.gcfd_step_vjp.argtypes = [C.c_void_p, C.c_int32, PI, C.POINTER(PD), C.c_double, C.POINTER(PD), PD, PD]
        lib.gcfd_sample_points.argtypes = [C.c_void_p, C.c_int32, PD, PD, PD, PI]
        lib.gcfd_wall_points.argtypes = [C.c_void_p, PI, PD, PD, PD, PD]
        lib.gcfd_device_fma_peaks.argtypes = [C.c_int32, PD, PD]
        lib.gcfd_host_graph_element.argtypes = [C.c_int32, PI, PI, PD, PI]
        lib.gcfd_graph_mesh.argtypes = [C.c_void_p, PI, PI, C.POINTER(C.c_float), C.POINTER(C.c_int64)]
        lib.gcfd_graph_fields.argtypes = [C.c_void_p, C.c_int32, PI, C.POINTER(C.c_float)]
        _lib = lib
        return lib


def check(lib, ctx, rc: int):
    if rc != GCFD_OK:
        msg = lib.gcfd_last_error(ctx)
        raise GcfdError(rc, msg.decode() if msg else "")


def graph_element(N: int):
    """The reference element's graph points (len_element x 2 (r, s)) and
    sub-triangles (ntri x 3, local indices) of the solution output (no GPU)."""
    lib = load()
    L, nt = C.c_int32(), C.c_int32()
    check(lib, None, lib.gcfd_host_graph_element(int(N), C.byref(L), C.byref(nt), None, None))
    rs = np.zeros((L.value, 2))
    tris = np.zeros((nt.value, 3), dtype=np.int32)
    check(lib, None, lib.gcfd_host_graph_element(int(N), None, None, rs.ctypes.data_as(PD), tris.ctypes.data_as(PI)))
    return rs, tris


def read_mesh(path: str):
    """A Gambit (.neu) or SU2 (.su2) mesh read by the library's C++ reader:
    (VX, VY, EToV (K x 3, 0-based), bc_edges [(v1, v2, flag)]).  No GPU needed."""
    lib = load()
    m = Mesh()
    check(lib, None, lib.gcfd_read_mesh(os.fsencode(path), C.byref(m)))
    try:
        vx = np.ctypeslib.as_array(m.vx, shape=(m.nverts,)).copy()
        vy = np.ctypeslib.as_array(m.vy, shape=(m.nverts,)).copy()
        etov = np.ctypeslib.as_array(m.etov, shape=(m.K * 3,)).reshape(m.K, 3).copy()
        bc = [(int(m.bc_v1[i]), int(m.bc_v2[i]), int(m.bc_flag[i])) for i in range(m.nbc)]
    finally:
        lib.gcfd_free_mesh(C.byref(m))
    return vx, vy, etov, bc


def host_operator(N: int, which: int) -> np.ndarray:
    """FP64 operator matrix built by the library's host code (no GPU needed)."""
    lib = load()
    rows, cols = C.c_int32(), C.c_int32()
    check(lib, None, lib.gcfd_host_operator(N, which, None, C.byref(rows), C.byref(cols)))
    out = np.zeros((rows.value, cols.value), dtype=np.float64)
    check(lib, None, lib.gcfd_host_operator(N, which, out.ctypes.data_as(PD), C.byref(rows), C.byref(cols)))
    return out


def device_fma_peaks(device: int = 0):
    """(FP64, FP32) SIMT FMA rates of the device in TFLOP/s (gcfd_device_fma_peaks)."""
    lib = load()
    f64, f32 = C.c_double(), C.c_double()
    check(lib, None, lib.gcfd_device_fma_peaks(int(device), C.byref(f64), C.byref(f32)))
    return f64.value, f32.value

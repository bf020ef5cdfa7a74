"""ctypes front end of oracle/_ref (the reference's own sources compiled against the host SYCL
subset, see oracle/build_ref.py) — TEST INFRASTRUCTURE, development container only."""
from __future__ import annotations

import ctypes

import numpy as np

from . import build_ref

ALGORITHMS = {"nptl": 0, "lptl": 1, "npol": 2, "nsol": 3}
LAYOUTS = {"collision": 0, "stream": 1, "bundle": 2}
_LIBS: dict = {}


def load(precision: str = "f64") -> ctypes.CDLL:
    if precision in _LIBS:
        return _LIBS[precision]
    if not build_ref.build():
        raise RuntimeError("reference tree not available")
    lib = ctypes.CDLL(build_ref.lib_path(precision))
    lib.refo_create.restype = ctypes.c_void_p
    lib.refo_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_char_p, ctypes.c_uint,
                                ctypes.c_uint, ctypes.c_uint] + [ctypes.c_double] * 7 + [ctypes.c_uint]
    lib.refo_run.argtypes = [ctypes.c_void_p]
    lib.refo_destroy.argtypes = [ctypes.c_void_p]
    lib.refo_results.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    lib.refo_domain.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    _LIBS[precision] = lib
    return lib


def run(algorithm, data_layout, work_group_size, scenario, w, h, steps, inlet_density=1.05, relaxation_time=0.6,
        outlet_density=1.0, inlet_velocity=(0.0, 0.0), outlet_velocity=(0.0, 0.0), precision="f64", rand_seed=1):
    """Runs the reference's algorithm class for `steps` steps; returns rho, jx, jy, |j| and its Domain."""
    lib = load(precision)
    h_ = lib.refo_create(ALGORITHMS[algorithm], LAYOUTS[data_layout], work_group_size, scenario.encode(), w, h,
                         steps, inlet_velocity[0], inlet_velocity[1], inlet_density, outlet_velocity[0],
                         outlet_velocity[1], outlet_density, relaxation_time, rand_seed)
    if not h_:
        raise ValueError("reference rejected the configuration")
    try:
        lib.refo_run(h_)
        out = {}
        for i, k in enumerate(("rho", "jx", "jy", "jabs")):
            a = np.empty(w * h)
            lib.refo_results(h_, i, a.ctypes.data)
            out[k] = a
        dom = (ctypes.c_uint * 7)()
        lib.refo_domain(h_, dom)
        out["domain"] = list(dom)
        return out
    finally:
        lib.refo_destroy(h_)

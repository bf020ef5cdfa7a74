"""ctypes front end of the CPU oracle (``oracle/plbm_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` as the checker.  The product library never loads it.

``Oracle`` mirrors how the reference's tests drive a simulation
(tests/smoke_test.cpp:46-70: build properties, run N steps, read rho/jx/jy/|j|).
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ALGORITHMS = {"nptl": 0, "lptl": 1, "npol": 2, "nsol": 3}
LAYOUTS = {"collision": 0, "stream": 1, "bundle": 2}
SCENARIOS = {"Hagen-Poiseuille": 0, "walls": 1, "circle": 2, "square": 3, "wing": 4,
             "skyscraper": 5, "porous": 6, "plate": 7, "custom": 100}


# "f64": the reference's double arithmetic, every operation rounded (-ffp-contract=off);
# "f32": its USE_FLOAT build; "f64_contracted": the same double code with the compiler free to fuse
# multiply-adds, a legal compilation of the reference that rounds differently (used only to measure
# how strongly a configuration amplifies rounding differences).
_LIBS_BY_PRECISION = {"f64": "libplbm_oracle.so", "f32": "libplbm_oracle_f32.so",
                      "f64_contracted": "libplbm_oracle_contracted.so"}


def lib_path(precision: str = "f64") -> str:
    return os.path.join(HERE, _LIBS_BY_PRECISION[precision])


def build(force: bool = False) -> None:
    """Compiles the oracle variants (see _LIBS_BY_PRECISION)."""
    src = os.path.join(HERE, "plbm_oracle.c")
    fma = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
    for prec, extra in (("f64", ["-ffp-contract=off"]), ("f32", ["-ffp-contract=off", "-DPLBMO_FLOAT"]),
                        ("f64_contracted", ["-ffp-contract=fast", *fma])):
        out = lib_path(prec)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            continue
        cmd = ["gcc", "-O2", "-std=c11", "-fno-fast-math", "-fopenmp",
               "-fPIC", "-shared", *extra, "-o", out + ".tmp", src, "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(out + ".tmp", out)


class Domain(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint) for n in (
        "total_node_count", "horizontal_nodes", "vertical_nodes", "subdomain_vertical_nodes",
        "subdomain_horizontal_nodes", "subdomain_count_vertical", "subdomain_count_horizontal")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


_LIBS: dict = {}


def load(precision: str = "f64") -> ctypes.CDLL:
    if precision in _LIBS:
        return _LIBS[precision]
    build()
    lib = ctypes.CDLL(lib_path(precision))
    lib.plbmo_create.restype = ctypes.c_void_p
    lib.plbmo_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_int, ctypes.c_uint,
                                 ctypes.c_uint] + [ctypes.c_double] * 7 + [ctypes.c_int, ctypes.c_void_p]
    lib.plbmo_destroy.argtypes = [ctypes.c_void_p]
    lib.plbmo_run.argtypes = [ctypes.c_void_p, ctypes.c_uint]
    lib.plbmo_results.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    lib.plbmo_flags.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.plbmo_lattice.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    lib.plbmo_lattice.restype = ctypes.c_size_t
    lib.plbmo_get_domain.argtypes = [ctypes.c_void_p, ctypes.POINTER(Domain)]
    lib.plbmo_domain_for.argtypes = [ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                     ctypes.POINTER(Domain)]
    lib.plbmo_rand_reset.argtypes = [ctypes.c_uint]
    lib.plbmo_rand.restype = ctypes.c_int
    lib.plbmo_threads.restype = ctypes.c_int
    _LIBS[precision] = lib
    return lib


def domain_for(algorithm: str, work_group_size: int, inner_w: int, inner_h: int) -> dict | None:
    d = Domain()
    rc = load().plbmo_domain_for(ALGORITHMS[algorithm], work_group_size, inner_w + 2, inner_h + 2,
                                 ctypes.byref(d))
    return None if rc != 0 else d.as_dict()


class Oracle:
    """One simulation of the restated reference path."""

    def __init__(self, algorithm="nptl", data_layout="stream", work_group_size=1024,
                 scenario="Hagen-Poiseuille", horizontal_nodes=400, vertical_nodes=100,
                 inlet_velocity=(0.0, 0.0), inlet_density=1.2, outlet_velocity=(0.0, 0.0),
                 outlet_density=1.0, relaxation_time=0.6, nan_protection=True, mask=None,
                 precision="f64"):
        self.lib = load(precision)
        self.w, self.h = int(horizontal_nodes), int(vertical_nodes)
        self._mask = None
        sc = SCENARIOS[scenario] if mask is None else SCENARIOS["custom"]
        if mask is not None:
            self._mask = np.ascontiguousarray(mask, dtype=np.int8).reshape(self.h, self.w)
        self.h_ = self.lib.plbmo_create(
            ALGORITHMS[algorithm], LAYOUTS[data_layout], int(work_group_size), sc, self.w, self.h,
            float(inlet_velocity[0]), float(inlet_velocity[1]), float(inlet_density),
            float(outlet_velocity[0]), float(outlet_velocity[1]), float(outlet_density),
            float(relaxation_time), int(bool(nan_protection)),
            None if self._mask is None else self._mask.ctypes.data)
        if not self.h_:
            raise ValueError("illegal oracle configuration")
        self.steps = 0

    def __del__(self):
        h = getattr(self, "h_", None)
        if h:
            self.lib.plbmo_destroy(h)
            self.h_ = None

    def run(self, steps: int) -> "Oracle":
        self.lib.plbmo_run(self.h_, int(steps))
        self.steps += int(steps)
        return self

    def result(self, which: int) -> np.ndarray:
        out = np.empty(self.w * self.h, dtype=np.float64)
        self.lib.plbmo_results(self.h_, which, out.ctypes.data)
        return out

    def results(self) -> dict:
        return {k: self.result(i) for i, k in enumerate(("rho", "jx", "jy", "jabs"))}

    def domain(self) -> dict:
        d = Domain()
        self.lib.plbmo_get_domain(self.h_, ctypes.byref(d))
        return d.as_dict()

    def flags(self) -> np.ndarray:
        out = np.empty(self.domain()["total_node_count"], dtype=np.int8)
        self.lib.plbmo_flags(self.h_, out.ctypes.data)
        return out

    def lattice(self, which: int = 0) -> np.ndarray:
        out = np.empty(9 * self.domain()["total_node_count"], dtype=np.float64)
        n = self.lib.plbmo_lattice(self.h_, which, out.ctypes.data)
        return out[:n]


def threads() -> int:
    return int(load().plbmo_threads())

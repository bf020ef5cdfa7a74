"""portlbm_gb300 — PortLBM's per-timestep D2Q9 BGK update on one GB300 (sm_103a).

Python mirror of the reference's public API (SC-SGS/PortLBM):

* ``Properties``            core::Properties (include/lbm/core/properties.hpp:30-166): the
                            constructor takes INNER extents and stores inner + 2, like
                            src/lbm/core/simulation.cpp:21-58; ``validate()`` raises
                            ``PropertyArgumentException`` with the reference's messages.
* ``create_handler``        lbm::create_handler (include/lbm/portlbm_factory.hpp:59,73), from a
                            ``Properties`` or a settings.json path.
* ``AlgorithmHandler``      execution::AlgorithmHandler (include/lbm/execution/
                            algorithm_handler.hpp:40-156): initialize/start/pause/
                            block_until_finished/is_finished and the result getters.

Everything runs in ``libplbm.so`` (hand-written CUDA + C++ host code) through the C ABI of
``include/plbm_c.h``; there is no CPU fallback.  If the library is missing or no GPU is
present, creating a handler raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

__all__ = [
    "Properties", "create_handler", "AlgorithmHandler", "Exception", "PropertyArgumentException",
    "WaitException", "CudaException", "ParseException", "NoDeviceException", "PRECISIONS",
    "properties_to_json", "json_to_properties", "library_path", "load_library", "compute_domain", "make_flags",
    "porous_disks", "Batch", "write_npy", "benchmark_work_group_sizes", "run_benchmark",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
PRECISIONS = {"f64_strict": 0, "f64_fast": 1, "f32_ref": 2, "f32": 3, "f16s": 4, "bf16s": 5, "f64_q60": 6,
              "f16c": 7}
BYTES_PER_VALUE = {0: 8, 1: 8, 2: 4, 3: 4, 4: 2, 5: 2, 6: 8}


class Exception(RuntimeError):  # noqa: A001 - mirrors lbm::exceptions::Exception
    """lbm::exceptions::Exception (include/lbm/exceptions/exceptions.hpp:31)."""


class PropertyArgumentException(Exception):
    """lbm::exceptions::json::PropertyArgumentException (exceptions.hpp:70)."""


class WaitException(Exception):
    """lbm::exceptions::algorithm::WaitException (exceptions.hpp:150)."""


class CudaException(Exception):
    """A CUDA runtime error inside libplbm."""


class ParseException(Exception):
    """settings.json could not be read or parsed (nlohmann::json errors in the reference)."""


class NoDeviceException(CudaException):
    """No CUDA device is visible."""


_CODES = {-1: PropertyArgumentException, -2: Exception, -3: WaitException, -4: CudaException,
          -5: ParseException, -6: ParseException, -7: Exception, -8: Exception, -9: NoDeviceException}


class _CProps(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_char_p), ("data_layout", ctypes.c_char_p), ("debug_mode", ctypes.c_int),
                ("work_group_size", ctypes.c_uint), ("time_steps", ctypes.c_uint),
                ("frame_update_interval", ctypes.c_uint), ("scenario", ctypes.c_char_p),
                ("vertical_nodes", ctypes.c_uint), ("horizontal_nodes", ctypes.c_uint),
                ("inlet_velocity_x", ctypes.c_double), ("inlet_velocity_y", ctypes.c_double),
                ("inlet_density", ctypes.c_double), ("outlet_velocity_x", ctypes.c_double),
                ("outlet_velocity_y", ctypes.c_double), ("outlet_density", ctypes.c_double),
                ("relaxation_time", ctypes.c_double)]


class _COpts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("nan_protection", ctypes.c_int), ("use_graph", ctypes.c_int),
                ("device", ctypes.c_int), ("mask", ctypes.c_void_p), ("gather", ctypes.c_int)]


# PLBM_GATHER_*: the gather of obstacle-adjacent nodes in the f32/f16s/bf16s nptl/lptl steps
GATHER = {"auto": 0, "open": 1, "porous": 2}


def library_path() -> str:
    """libplbm.so, or the bounds-checked build libplbm_checked.so when PLBM_CHECKED=1."""
    name = "libplbm_checked.so" if os.environ.get("PLBM_CHECKED") == "1" else "libplbm.so"
    return os.path.join(_HERE, name)


_LIB = None

# Exported symbols of include/plbm_c.h with their argument types.
_SIGS = {
    "plbm_default_options": (None, [ctypes.POINTER(_COpts)]),
    "plbm_validate": (ctypes.c_int, [ctypes.POINTER(_CProps)]),
    "plbm_create": (ctypes.c_int, [ctypes.POINTER(_CProps), ctypes.POINTER(_COpts), ctypes.POINTER(ctypes.c_void_p)]),
    "plbm_create_from_json": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_COpts), ctypes.POINTER(ctypes.c_void_p)]),
    "plbm_destroy": (None, [ctypes.c_void_p]),
    "plbm_initialize": (ctypes.c_int, [ctypes.c_void_p]),
    "plbm_start": (ctypes.c_int, [ctypes.c_void_p]),
    "plbm_pause": (ctypes.c_int, [ctypes.c_void_p]),
    "plbm_block_until_finished": (ctypes.c_int, [ctypes.c_void_p]),
    "plbm_is_finished": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "plbm_get_results": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)),
                                        ctypes.POINTER(ctypes.c_size_t)]),
    "plbm_get_extents": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_uint)]),
    "plbm_get_domain": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)]),
    "plbm_get_progress": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "plbm_get_last_frametime": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "plbm_get_current_iteration": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)]),
    "plbm_get_properties": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_CProps)]),
    "plbm_properties_to_json": (ctypes.c_int, [ctypes.POINTER(_CProps), ctypes.c_char_p]),
    "plbm_json_to_properties": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(_CProps)]),
    "plbm_run_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint, ctypes.POINTER(ctypes.c_double)]),
    "plbm_sync_results": (ctypes.c_int, [ctypes.c_void_p]),
    "plbm_gather_form": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "plbm_launches_per_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)]),
    "plbm_bytes_per_node": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "plbm_mass_momentum": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "plbm_compute_domain": (ctypes.c_int, [ctypes.POINTER(_CProps), ctypes.POINTER(ctypes.c_uint)]),
    "plbm_make_flags": (ctypes.c_int, [ctypes.POINTER(_CProps), ctypes.c_void_p]),
    "plbm_set_frame_export": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_uint]),
    "plbm_write_npy": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint]),
    "plbm_benchmark_run": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_COpts),
                                          ctypes.c_uint, ctypes.c_double]),
    "plbm_benchmark_work_group_sizes": (ctypes.c_int, [ctypes.c_uint, ctypes.POINTER(ctypes.c_uint), ctypes.c_uint,
                                                       ctypes.POINTER(ctypes.c_uint)]),
    "plbm_set_equilibrium": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "plbm_set_precision": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "plbm_run_to_residual": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_uint, ctypes.c_uint,
                                            ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_double)]),
    "plbm_porous_disks": (ctypes.c_int, [ctypes.c_uint, ctypes.c_uint, ctypes.c_uint64, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_void_p]),
    "plbm_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "plbm_version": (ctypes.c_char_p, []),
}


def load_library() -> ctypes.CDLL:
    """Loads the in-tree libplbm.so; raises if it has not been built (no fallback path)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m portlbm_gb300.build`")
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _check(rc: int, handle=None) -> None:
    if rc == 0:
        return
    lib = load_library()
    msg = lib.plbm_last_error(handle).decode(errors="replace")
    raise _CODES.get(rc, Exception)(msg)


class Properties:
    """core::Properties; ``vertical_nodes``/``horizontal_nodes`` are passed as inner extents and
    stored with the two ghost layers added (src/lbm/core/simulation.cpp:45-48)."""

    def __init__(self, algorithm: str, data_layout: str, debug_mode: bool, work_group_size: int,
                 time_steps: int, frame_update_interval: int, scenario: str, vertical_nodes: int,
                 horizontal_nodes: int, inlet_velocity_x: float, inlet_velocity_y: float,
                 inlet_density: float, outlet_velocity_x: float, outlet_velocity_y: float,
                 outlet_density: float, relaxation_time: float):
        self.algorithm = algorithm
        self.data_layout = data_layout
        self.debug_mode = bool(debug_mode)
        self.work_group_size = int(work_group_size)
        self.time_steps = int(time_steps)
        self.frame_update_interval = int(frame_update_interval)
        self.scenario = scenario
        self.vertical_nodes = int(vertical_nodes) + 2
        self.horizontal_nodes = int(horizontal_nodes) + 2
        self.total_unexpanded_node_count = self.vertical_nodes * self.horizontal_nodes
        self.domain_node_count = int(vertical_nodes) * int(horizontal_nodes)
        self.inlet_velocity_x = float(inlet_velocity_x)
        self.inlet_velocity_y = float(inlet_velocity_y)
        self.inlet_density = float(inlet_density)
        self.outlet_velocity_x = float(outlet_velocity_x)
        self.outlet_velocity_y = float(outlet_velocity_y)
        self.outlet_density = float(outlet_density)
        self.relaxation_time = float(relaxation_time)
        self.settings_path = ""

    def _c(self) -> _CProps:
        self._keep = [s.encode() for s in (self.algorithm, self.data_layout, self.scenario)]
        return _CProps(self._keep[0], self._keep[1], int(self.debug_mode), self.work_group_size, self.time_steps,
                       self.frame_update_interval, self._keep[2], self.vertical_nodes - 2,
                       self.horizontal_nodes - 2, self.inlet_velocity_x, self.inlet_velocity_y,
                       self.inlet_density, self.outlet_velocity_x, self.outlet_velocity_y, self.outlet_density,
                       self.relaxation_time)

    @classmethod
    def _from_c(cls, c: _CProps, path: str = "") -> "Properties":
        p = cls(c.algorithm.decode(), c.data_layout.decode(), bool(c.debug_mode), c.work_group_size, c.time_steps,
                c.frame_update_interval, c.scenario.decode(), c.vertical_nodes, c.horizontal_nodes,
                c.inlet_velocity_x, c.inlet_velocity_y, c.inlet_density, c.outlet_velocity_x, c.outlet_velocity_y,
                c.outlet_density, c.relaxation_time)
        p.settings_path = path
        return p

    def validate(self) -> None:
        """Properties::validate (src/lbm/core/simulation.cpp:60-125)."""
        c = self._c()
        _check(load_library().plbm_validate(ctypes.byref(c)))

    def to_string(self) -> str:
        """Properties::to_string (src/lbm/core/simulation.cpp:137-175)."""
        return ("Algorithmic properties: \n"
                f"\tAlgorithm: {self.algorithm} \n\tData layout: {self.data_layout} \n"
                f"\tWork group size: {self.work_group_size} \n\tDebug mode: {str(self.debug_mode).lower()} \n"
                f"\tTime steps: {self.time_steps} \n\tFrame update interval: {self.frame_update_interval} \n"
                "Domain properties: \n"
                f"\tScenario: {self.scenario}\n\tVertical nodes: {self.vertical_nodes} \n"
                f"\tHorizontal nodes: {self.horizontal_nodes} \n\tNode count: {self.total_unexpanded_node_count} \n"
                "Physical: \n"
                f"\tInlet velocity: ({self.inlet_velocity_x:.6f}, {self.inlet_velocity_y:.6f})\n"
                f"\tInlet density: {self.inlet_density:.6f}\n"
                f"\tOutlet velocity: ({self.outlet_velocity_x:.6f}, {self.outlet_velocity_y:.6f})\n"
                f"\tOutlet density: {self.outlet_density:.6f}\n"
                f"\tRelaxation time: {self.relaxation_time:.6f}\n\n")


_DOMAIN_KEYS = ("total_node_count", "horizontal_nodes", "vertical_nodes", "subdomain_vertical_nodes",
                "subdomain_horizontal_nodes", "subdomain_count_vertical", "subdomain_count_horizontal")


def compute_domain(props: Properties) -> dict:
    """core::Domain(properties) (src/lbm/core/simulation.cpp:194-382), computed on the host."""
    c = props._c()
    arr = (ctypes.c_uint * 7)()
    _check(load_library().plbm_compute_domain(ctypes.byref(c), arr))
    return dict(zip(_DOMAIN_KEYS, list(arr)))


def make_flags(props: Properties) -> np.ndarray:
    """Inner (H, W) phase flags of the scenario (0 fluid, 1 solid), as setup_domain builds them."""
    c = props._c()
    out = np.empty((props.vertical_nodes - 2, props.horizontal_nodes - 2), dtype=np.int8)
    _check(load_library().plbm_make_flags(ctypes.byref(c), out.ctypes.data))
    return out


def porous_disks(w: int, h: int, seed: int, porosity: float, rmin: float = 3.0, rmax: float = 12.0) -> np.ndarray:
    """Seeded porous channel: walls on the first/last inner row plus non-overlapping disks with radius
    uniform in [rmin, rmax] until the interior's fluid fraction reaches `porosity`; (H, W) int8."""
    out = np.empty((h, w), dtype=np.int8)
    n = load_library().plbm_porous_disks(w, h, seed, porosity, rmin, rmax, out.ctypes.data)
    if n < 0:
        _check(n)
    return out


def properties_to_json(props: Properties, path: str) -> None:
    """file_interaction::properties_to_json (src/lbm/file_interaction/file_interaction.cpp:11-37),
    writing the inner node counts."""
    c = props._c()
    _check(load_library().plbm_properties_to_json(ctypes.byref(c), path.encode()))


def json_to_properties(path: str, offset: int = 0) -> Properties:
    """file_interaction::json_to_properties (file_interaction.cpp:39-69)."""
    c = _CProps()
    _check(load_library().plbm_json_to_properties(path.encode(), int(offset), ctypes.byref(c)))
    return Properties._from_c(c, path)


class AlgorithmHandler:
    """execution::AlgorithmHandler backed by a libplbm handle."""

    def __init__(self, handle: int):
        self._lib = load_library()
        self._h = ctypes.c_void_p(handle)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.plbm_destroy(h)
            self._h = None

    def close(self) -> None:
        self.__del__()

    def _call(self, name: str, *args):
        _check(getattr(self._lib, name)(self._h, *args), self._h)

    # -- life cycle (algorithm_handler.hpp:55-88) --
    def initialize(self) -> None:
        self._call("plbm_initialize")

    def start(self) -> None:
        self._call("plbm_start")

    def pause(self) -> None:
        self._call("plbm_pause")

    def block_until_finished(self) -> None:
        self._call("plbm_block_until_finished")

    def is_finished(self) -> bool:
        v = ctypes.c_int()
        self._call("plbm_is_finished", ctypes.byref(v))
        return bool(v.value)

    # -- results (algorithm_handler.hpp:90-121) --
    def _result(self, which: int, copy: bool = True) -> np.ndarray:
        ptr = ctypes.POINTER(ctypes.c_double)()
        n = ctypes.c_size_t()
        self._call("plbm_get_results", which, ctypes.byref(ptr), ctypes.byref(n))
        arr = np.ctypeslib.as_array(ptr, shape=(n.value,))
        return arr.copy() if copy else arr

    def get_densities(self, copy: bool = True) -> np.ndarray:
        return self._result(0, copy)

    def get_x_velocities(self, copy: bool = True) -> np.ndarray:
        return self._result(1, copy)

    def get_y_velocities(self, copy: bool = True) -> np.ndarray:
        return self._result(2, copy)

    def get_absolute_velocities(self, copy: bool = True) -> np.ndarray:
        return self._result(3, copy)

    # -- extents and status (algorithm_handler.hpp:123-151) --
    def get_horizontal_nodes(self) -> int:
        h, v = ctypes.c_uint(), ctypes.c_uint()
        self._call("plbm_get_extents", ctypes.byref(h), ctypes.byref(v))
        return h.value

    def get_vertical_nodes(self) -> int:
        h, v = ctypes.c_uint(), ctypes.c_uint()
        self._call("plbm_get_extents", ctypes.byref(h), ctypes.byref(v))
        return v.value

    def get_properties(self) -> Properties:
        c = _CProps()
        self._call("plbm_get_properties", ctypes.byref(c))
        return Properties._from_c(c)

    def get_inlet_density(self) -> float:
        return self.get_properties().inlet_density

    def get_outlet_density(self) -> float:
        return self.get_properties().outlet_density

    def get_domain(self) -> dict:
        arr = (ctypes.c_uint * 7)()
        self._call("plbm_get_domain", arr)
        keys = ("total_node_count", "horizontal_nodes", "vertical_nodes", "subdomain_vertical_nodes",
                "subdomain_horizontal_nodes", "subdomain_count_vertical", "subdomain_count_horizontal")
        return dict(zip(keys, list(arr)))

    def get_progress(self) -> float:
        v = ctypes.c_double()
        self._call("plbm_get_progress", ctypes.byref(v))
        return v.value

    def get_last_frametime(self) -> float:
        v = ctypes.c_double()
        self._call("plbm_get_last_frametime", ctypes.byref(v))
        return v.value

    def get_current_iteration(self) -> int:
        v = ctypes.c_uint()
        self._call("plbm_get_current_iteration", ctypes.byref(v))
        return v.value

    # -- measurement hooks (no counterpart in the reference) --
    def run_steps(self, n: int) -> float:
        """Runs n steps synchronously with device-resident data; returns device ms per step."""
        ms = ctypes.c_double()
        self._call("plbm_run_steps", int(n), ctypes.byref(ms))
        return ms.value

    def sync_results(self) -> None:
        self._call("plbm_sync_results")

    FIELDS = ("rho", "jx", "jy", "jabs")

    def set_frame_export(self, directory, fields=FIELDS) -> None:
        """Headless frames: from the next start() on, every frame step and the last step write the
        chosen results as <directory>/frame_<iteration>_<field>.npy (float64, H x W).  None turns
        it off.  (Stands in for the reference's GUI, include/lbm/gui/lbm_gui.hpp.)"""
        bits = 0
        for f in fields or ():
            bits |= 1 << self.FIELDS.index(f)
        self._call("plbm_set_frame_export", None if directory is None else str(directory).encode(),
                   bits if directory is not None else 0)

    def set_equilibrium(self, rho, jx, jy) -> None:
        """Replaces the state by the equilibrium populations of the inner fields (W*H each, row-major;
        solid entries ignored); nptl/lptl only, before stepping or after an even number of steps."""
        h, v = ctypes.c_uint(), ctypes.c_uint()
        self._call("plbm_get_extents", ctypes.byref(h), ctypes.byref(v))
        n = (h.value - 2) * (v.value - 2)
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in (rho, jx, jy)]
        if any(a.size != n for a in arrs):
            raise ValueError(f"fields must hold {n} inner values each")
        self._call("plbm_set_equilibrium", *(a.ctypes.data for a in arrs))

    def mass_momentum(self) -> tuple:
        out = (ctypes.c_double * 3)()
        self._call("plbm_mass_momentum", out)
        return tuple(out)

    def run_to_residual(self, target: float = 1e-6, k: int = 100, max_steps: int = 1_000_000) -> tuple:
        """Steps in chunks of k until ||j^n - j^(n-k)|| / (k ||j^n||) < target; returns (steps, residual)."""
        steps, r = ctypes.c_uint(), ctypes.c_double()
        self._call("plbm_run_to_residual", float(target), int(k), int(max_steps), ctypes.byref(steps), ctypes.byref(r))
        return steps.value, r.value

    def set_precision(self, precision: str) -> None:
        """Re-encodes the state in another shifted storage form ("f32", "f16s", "bf16s", "f16c") and
        continues in it (plbm_set_precision)."""
        self._call("plbm_set_precision", PRECISIONS[precision])

    def run_to_residual_escalating(self, target: float = 1e-6, k: int = 100, max_steps: int = 1_000_000,
                                   chunk: int = 1000, stall: float = 0.95, then: str = "f32") -> tuple:
        """Steps a 16-bit form towards the residual target; when a chunk of `chunk` steps no longer
        lowers the residual below `stall` times its previous value (the form's rounding floor), the
        state is re-encoded in `then` (FP32) and the run continues there.  Returns (steps, residual,
        steps before the switch, or None when the target was met without one)."""
        total, prev, switched = 0, None, None
        while total < max_steps:
            n, r = self.run_to_residual(target, k, min(chunk, max_steps - total))
            total += n
            if r < target:
                return total, r, switched
            if switched is None and prev is not None and r > stall * prev:
                self.set_precision(then)
                switched = total
            prev = r
        return total, prev, switched

    def bytes_per_node(self) -> float:
        v = ctypes.c_double()
        self._call("plbm_bytes_per_node", ctypes.byref(v))
        return v.value

    def gather_form(self) -> str:
        """The gather the step runs: "open" or "porous"."""
        v = ctypes.c_int()
        self._call("plbm_gather_form", ctypes.byref(v))
        return {1: "open", 2: "porous"}[v.value]

    def launches_per_step(self) -> int:
        v = ctypes.c_uint()
        self._call("plbm_launches_per_step", ctypes.byref(v))
        return v.value


class _CBatchDomain(ctypes.Structure):
    _fields_ = [("inner_w", ctypes.c_uint), ("inner_h", ctypes.c_uint), ("relaxation_time", ctypes.c_double),
                ("inlet_density", ctypes.c_double), ("outlet_density", ctypes.c_double), ("mask", ctypes.c_void_p)]


BATCH_MODES = {"persistent": 0, "persistent_graph": 1, "per_domain": 2}
BATCH_TILE_VEC = 0x10000   # PLBM_BATCH_TILE_VEC: vectorised rows of the 2-byte batches (set_tile's tile_h)


class Batch:
    """Many independent channels advanced together (plbm_batch_* in include/plbm_c.h)."""

    def __init__(self, domains, precision: str = "f32"):
        """domains: iterable of dicts {mask: (H, W) int8, relaxation_time, inlet_density, outlet_density}."""
        lib = load_library()
        self._lib = lib
        for name, res, args in (
                ("plbm_batch_create", ctypes.c_int, [ctypes.c_uint, ctypes.POINTER(_CBatchDomain), ctypes.c_int,
                                                     ctypes.POINTER(ctypes.c_void_p)]),
                ("plbm_batch_destroy", None, [ctypes.c_void_p]),
                ("plbm_batch_set_tile", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
                ("plbm_batch_autotune", ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint] + [ctypes.POINTER(ctypes.c_int)] * 3),
                ("plbm_batch_run", ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint, ctypes.c_int,
                                                  ctypes.POINTER(ctypes.c_double)]),
                ("plbm_batch_results", ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint, ctypes.c_int, ctypes.c_void_p]),
                ("plbm_batch_info", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_ulonglong),
                                                   ctypes.POINTER(ctypes.c_uint)]),
                ("plbm_batch_last_error", ctypes.c_char_p, [])):
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        self._masks = [np.ascontiguousarray(d["mask"], dtype=np.int8) for d in domains]
        arr = (_CBatchDomain * len(self._masks))()
        self.shapes = []
        for i, (d, m) in enumerate(zip(domains, self._masks)):
            arr[i] = _CBatchDomain(m.shape[1], m.shape[0], d["relaxation_time"], d["inlet_density"],
                                   d.get("outlet_density", 1.0), m.ctypes.data)
            self.shapes.append(m.shape)
        h = ctypes.c_void_p()
        rc = lib.plbm_batch_create(len(self._masks), arr, PRECISIONS[precision], ctypes.byref(h))
        if rc != 0:
            raise _CODES.get(rc, Exception)(lib.plbm_batch_last_error().decode())
        self._h = h

    def _ok(self, rc):
        if rc != 0:
            raise _CODES.get(rc, Exception)(self._lib.plbm_batch_last_error().decode())

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.plbm_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def set_tile(self, tile_w: int, tile_h: int, blocks_per_sm: int = 8):
        """tile_h = threads_y + 256 * rows per thread (+ BATCH_TILE_VEC for vectorised rows)."""
        self._ok(self._lib.plbm_batch_set_tile(self._h, tile_w, tile_h, blocks_per_sm))

    def autotune(self, steps: int = 4) -> tuple:
        w, h, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._ok(self._lib.plbm_batch_autotune(self._h, steps, ctypes.byref(w), ctypes.byref(h), ctypes.byref(b)))
        return w.value, h.value, b.value

    def run(self, steps: int, mode: str = "persistent_graph") -> float:
        ms = ctypes.c_double()
        self._ok(self._lib.plbm_batch_run(self._h, steps, BATCH_MODES[mode], ctypes.byref(ms)))
        return ms.value

    def result(self, domain: int, which: int) -> np.ndarray:
        h, w = self.shapes[domain]
        out = np.empty(h * w, dtype=np.float64)
        self._ok(self._lib.plbm_batch_results(self._h, domain, which, out.ctypes.data))
        return out

    def info(self) -> tuple:
        n, t = ctypes.c_ulonglong(), ctypes.c_uint()
        self._ok(self._lib.plbm_batch_info(self._h, ctypes.byref(n), ctypes.byref(t)))
        return n.value, t.value


def write_npy(path, array) -> None:
    """A 2-D float64 array as .npy through the library's own writer (the frame-export format)."""
    a = np.ascontiguousarray(array, dtype=np.float64)
    if a.ndim != 2:
        raise ValueError("write_npy takes a 2-D array")
    _check(load_library().plbm_write_npy(str(path).encode(), a.ctypes.data, a.shape[0], a.shape[1]))


def benchmark_work_group_sizes(max_work_group_size: int = 1024) -> list:
    """The work-group sizes the benchmark sweep tests (Benchmark::get_work_group_sizes)."""
    lib = load_library()
    n = ctypes.c_uint()
    lib.plbm_benchmark_work_group_sizes(max_work_group_size, None, 0, ctypes.byref(n))
    out = (ctypes.c_uint * n.value)()
    lib.plbm_benchmark_work_group_sizes(max_work_group_size, out, n.value, ctypes.byref(n))
    return list(out)


def run_benchmark(settings_path, benchmark_path=None, output_root=None, precision: str = "f64_strict",
                  phases=(0, 1, 2), hbm_gbs: float = 0.0, device: int = 0) -> None:
    """The reference's benchmark driver (src/lbm/benchmark/benchmark.cpp) on this library; see
    plbm_benchmark_run in include/plbm_c.h.  Output under <output_root>/benchmarks/phase<N>/."""
    lib = load_library()
    opts = _COpts()
    lib.plbm_default_options(ctypes.byref(opts))
    opts.precision = PRECISIONS[precision]
    opts.device = int(device)
    mask = 0
    for ph in phases:
        mask |= 1 << int(ph)
    rc = lib.plbm_benchmark_run(str(settings_path).encode(),
                                None if benchmark_path is None else str(benchmark_path).encode(),
                                None if output_root is None else str(output_root).encode(),
                                ctypes.byref(opts), mask, float(hbm_gbs))
    if rc != 0:
        raise _CODES.get(rc, Exception)(f"benchmark failed ({rc})")


def create_handler(source, precision: str = "f64_strict", mask=None, nan_protection: bool = True,
                   use_graph: bool = True, device: int = 0, gather: str = "auto") -> AlgorithmHandler:
    """lbm::create_handler from a ``Properties`` or a settings.json path.

    ``precision`` picks the arithmetic form ("f64_strict" is the drop-in); ``mask`` is an optional
    (H, W) array of 0 (fluid) / 1 (solid) replacing walls and scenario geometry; ``gather``
    ("auto", "open", "porous") picks how the f32/f16s/bf16s steps gather obstacle-adjacent nodes
    (same results; "auto" decides from the geometry).
    """
    lib = load_library()
    opts = _COpts()
    lib.plbm_default_options(ctypes.byref(opts))
    opts.gather = GATHER[gather]
    opts.precision = PRECISIONS[precision]
    opts.nan_protection = int(bool(nan_protection))
    opts.use_graph = int(bool(use_graph))
    opts.device = int(device)
    keep = None
    if mask is not None:
        keep = np.ascontiguousarray(mask, dtype=np.int8)
        opts.mask = keep.ctypes.data
    out = ctypes.c_void_p()
    if isinstance(source, Properties):
        c = source._c()
        rc = lib.plbm_create(ctypes.byref(c), ctypes.byref(opts), ctypes.byref(out))
    else:
        if precision == "f64_strict":
            opts.precision = 0
        rc = lib.plbm_create_from_json(str(source).encode(), ctypes.byref(opts), ctypes.byref(out))
    _check(rc)
    del keep
    return AlgorithmHandler(out.value)

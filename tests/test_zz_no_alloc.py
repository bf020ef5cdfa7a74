"""plbm_nptl_steps_noalloc — the entry point for callers that cannot let the library allocate.

Some callers own all device memory through their own allocator or arena, or run where the device
synchronisation of cudaMalloc/cudaFree is not acceptable; they pass every buffer themselves and the
step's only other state sits in a fixed __device__ array inside the library.  This test allocates
the caller's buffers with torch, calls the entry point through the C ABI twice in a row (a run and
its continuation) and checks each result against the regular handler path
(plbm_create + plbm_run_steps) with the tolerance the FP64 drop-in tests use: exact equality.
It passes alone in a fresh process and after the other tests (no state is assumed).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class NoallocArgs(ctypes.Structure):
    _fields_ = [("lattice0", ctypes.c_void_p), ("lattice1", ctypes.c_void_p), ("flags", ctypes.c_void_p),
                ("results", ctypes.c_void_p), ("inner_w", ctypes.c_uint), ("inner_h", ctypes.c_uint),
                ("relaxation_time", ctypes.c_double), ("inlet_density", ctypes.c_double),
                ("inlet_velocity_x", ctypes.c_double), ("inlet_velocity_y", ctypes.c_double),
                ("outlet_density", ctypes.c_double), ("outlet_velocity_x", ctypes.c_double),
                ("outlet_velocity_y", ctypes.c_double), ("first_step", ctypes.c_uint), ("steps", ctypes.c_uint),
                ("nan_protection", ctypes.c_int), ("stream", ctypes.c_void_p)]


def _mask(w, h):
    yy, xx = np.mgrid[0:h, 0:w]
    m = ((xx - w // 4) ** 2 + (yy - h // 2) ** 2 <= (h // 8) ** 2).astype(np.int8)
    m[0, :] = 1
    m[-1, :] = 1
    return m


def _lib(plbm):
    lib = plbm.load_library()
    lib.plbm_nptl_steps_noalloc.restype = ctypes.c_int
    lib.plbm_nptl_steps_noalloc.argtypes = [ctypes.POINTER(NoallocArgs)]
    lib.plbm_noalloc_last_error.restype = ctypes.c_char_p
    return lib


def test_noalloc_matches_handler_on_two_calls(plbm):
    import torch

    w, h, n = 70, 40, 150
    mask = _mask(w, h)
    props = plbm.Properties("nptl", "stream", False, 64, 2 * n, 2 * n, "Hagen-Poiseuille", h, w, 0.0, 0.0, 1.05,
                            0.0, 0.0, 1.0, 0.6)
    hd = plbm.create_handler(props, precision="f64_strict", mask=mask)
    ref = []
    for _ in range(2):
        hd.run_steps(n)
        hd.sync_results()
        ref.append(np.stack([hd.get_densities(), hd.get_x_velocities(), hd.get_y_velocities(),
                             hd.get_absolute_velocities()]))
    hd.close()

    lib = _lib(plbm)
    pitch = (w + 31) // 32 * 32
    dev = torch.device("cuda:0")
    lat0 = torch.empty(9 * pitch * h, dtype=torch.float64, device=dev)
    lat1 = torch.empty(9 * pitch * h, dtype=torch.float64, device=dev)
    flags = torch.from_numpy(mask.reshape(-1).copy()).to(dev)
    res = torch.empty(4 * w * h, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    args = NoallocArgs(lat0.data_ptr(), lat1.data_ptr(), flags.data_ptr(), res.data_ptr(), w, h, 0.6, 1.05, 0.0,
                       0.0, 1.0, 0.0, 0.0, 0, n, 1, None)
    for call in range(2):
        args.first_step = call * n
        rc = lib.plbm_nptl_steps_noalloc(ctypes.byref(args))
        assert rc == 0, lib.plbm_noalloc_last_error()
        torch.cuda.synchronize()
        got = res.cpu().numpy().reshape(4, -1)
        assert float(np.max(np.abs(got - ref[call]))) == 0.0


def test_noalloc_rejects_domains_beyond_its_scratch(plbm):
    lib = _lib(plbm)
    dummy = ctypes.c_void_p(1)
    args = NoallocArgs(dummy, dummy, dummy, dummy, 64, 65537, 0.6, 1.05, 0.0, 0.0, 1.0, 0.0, 0.0, 0, 1, 1, None)
    rc = lib.plbm_nptl_steps_noalloc(ctypes.byref(args))
    assert rc == -7
    assert b"PLBM_NOALLOC_MAX_ROWS" in lib.plbm_noalloc_last_error()

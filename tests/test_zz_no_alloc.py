"""plbm_nptl_steps_noalloc — the entry point for callers that cannot let the library allocate.

Some callers own all device memory through their own allocator or arena, or run where the device
synchronisation of cudaMalloc/cudaFree is not acceptable; they pass every buffer themselves and the
step's only other state sits in a fixed __device__ array inside the library.  This test allocates
the caller's buffers with torch, calls the entry point through the C ABI twice in a row (a run and
its continuation, once starting the second call on an odd step) and checks each result against
the regular handler path (plbm_create + plbm_run_steps) with the tolerance the FP64 drop-in tests
use: exact equality; further calls leave the device's free memory unchanged.
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


def _handler_results(plbm, mask, w, h, splits):
    props = plbm.Properties("nptl", "stream", False, 64, sum(splits), sum(splits), "Hagen-Poiseuille", h, w, 0.0, 0.0,
                            1.05, 0.0, 0.0, 1.0, 0.6)
    hd = plbm.create_handler(props, precision="f64_strict", mask=mask)
    ref = []
    for n in splits:
        hd.run_steps(n)
        hd.sync_results()
        ref.append(np.stack([hd.get_densities(), hd.get_x_velocities(), hd.get_y_velocities(),
                             hd.get_absolute_velocities()]))
    hd.close()
    return ref


def _buffers(mask, w, h):
    import torch
    pitch = (w + 31) // 32 * 32
    dev = torch.device("cuda:0")
    lat0 = torch.empty(9 * pitch * h, dtype=torch.float64, device=dev)
    lat1 = torch.empty(9 * pitch * h, dtype=torch.float64, device=dev)
    flags = torch.from_numpy(np.ascontiguousarray(mask).reshape(-1).copy()).to(dev)
    res = torch.empty(4 * w * h, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    return lat0, lat1, flags, res


@pytest.mark.parametrize("splits", [(150, 150), (75, 225)])
def test_noalloc_matches_handler_on_two_calls(plbm, splits):
    """Two calls in a row, the second continuing the first; (75, 225) starts the second call on an
    odd step, so it reads lattice1 and the jy scratch of the other parity."""
    import torch

    w, h = 70, 40
    mask = _mask(w, h)
    ref = _handler_results(plbm, mask, w, h, splits)
    lib = _lib(plbm)
    lat0, lat1, flags, res = _buffers(mask, w, h)
    args = NoallocArgs(lat0.data_ptr(), lat1.data_ptr(), flags.data_ptr(), res.data_ptr(), w, h, 0.6, 1.05, 0.0,
                       0.0, 1.0, 0.0, 0.0, 0, 0, 1, None)
    done = 0
    for call, n in enumerate(splits):
        args.first_step = done
        args.steps = n
        rc = lib.plbm_nptl_steps_noalloc(ctypes.byref(args))
        assert rc == 0, lib.plbm_noalloc_last_error()
        torch.cuda.synchronize()
        done += n
        got = res.cpu().numpy().reshape(4, -1)
        assert float(np.max(np.abs(got - ref[call]))) == 0.0


def test_noalloc_allocates_no_device_memory(plbm):
    """After a first call (which may load the library's device code and its fixed array), further
    calls leave the device's free memory unchanged; torch's caching allocator is not touched in
    between."""
    import torch

    w, h = 96, 48
    mask = _mask(w, h)
    lib = _lib(plbm)
    lat0, lat1, flags, res = _buffers(mask, w, h)
    args = NoallocArgs(lat0.data_ptr(), lat1.data_ptr(), flags.data_ptr(), res.data_ptr(), w, h, 0.7, 1.05, 0.0,
                       0.0, 1.0, 0.0, 0.0, 0, 20, 1, None)
    assert lib.plbm_nptl_steps_noalloc(ctypes.byref(args)) == 0, lib.plbm_noalloc_last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for k in range(1, 6):
        args.first_step = 20 * k
        assert lib.plbm_nptl_steps_noalloc(ctypes.byref(args)) == 0, lib.plbm_noalloc_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_treats_every_nonzero_flag_as_solid(plbm):
    """Flags are not checked; a value other than 0 or 1 acts as solid for the node and as a
    bounce-back source for its neighbours, exactly like 1."""
    import torch

    w, h = 64, 32
    mask = _mask(w, h)
    other = mask.copy()
    other[other == 1] = np.int8(-3)
    out = []
    lib = _lib(plbm)
    for m in (mask, other):
        lat0, lat1, flags, res = _buffers(m, w, h)
        args = NoallocArgs(lat0.data_ptr(), lat1.data_ptr(), flags.data_ptr(), res.data_ptr(), w, h, 0.6, 1.05, 0.0,
                           0.0, 1.0, 0.0, 0.0, 0, 120, 1, None)
        assert lib.plbm_nptl_steps_noalloc(ctypes.byref(args)) == 0, lib.plbm_noalloc_last_error()
        torch.cuda.synchronize()
        out.append(res.cpu().numpy())
    assert np.array_equal(out[0], out[1])


def test_noalloc_rejects_domains_beyond_its_scratch(plbm):
    lib = _lib(plbm)
    dummy = ctypes.c_void_p(1)
    args = NoallocArgs(dummy, dummy, dummy, dummy, 64, 65537, 0.6, 1.05, 0.0, 0.0, 1.0, 0.0, 0.0, 0, 1, 1, None)
    rc = lib.plbm_nptl_steps_noalloc(ctypes.byref(args))
    assert rc == -7
    assert b"PLBM_NOALLOC_MAX_ROWS" in lib.plbm_noalloc_last_error()
    args.inner_h = 64
    args.inner_w = (1 << 30) + 1
    assert lib.plbm_nptl_steps_noalloc(ctypes.byref(args)) == -7
    assert b"inner_w" in lib.plbm_noalloc_last_error()

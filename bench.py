"""Benchmark of PortLBM's per-timestep D2Q9 BGK update on GB300 (one JSON line on stdout).

Workload: the FP64 drop-in at 8192 x 8192 inner nodes — channel with bounce-back walls, a circle
obstacle of radius H/8 centred at (W/4, H/2), inlet density 1.2 / outlet 1.0, tau 0.6, nptl
algorithm, stream layout.  A "step" is one lattice-Boltzmann timestep over the whole domain.

* ``value``      MLUPS (W*H inner nodes x steps / s) of K device-resident steps, timed with CUDA
                 events on the solver's stream, of the FP64-accuracy form f64_q60 (populations in
                 64-bit fixed point, BGK update on the integer pipe; agrees with the reference to
                 <= 1e-12, see tests/test_gpu_parity.py).  ``err_vs_oracle`` restates that error
                 live: max |GPU - oracle| of rho, jx, jy after 2000 steps of the 400x100 channel.
* ``e2e``        the same metric through the public API with host buffers: create_handler from
                 host properties + host mask (H2D), K steps, results read back (D2H), all timed.
* ``roofline``   HBM roofline of the step kernel: 144 algorithmic bytes per node update (9 loads +
                 9 stores of 8 B) / CUDA-event time per launch, against MEASURED_PEAKS.json.
* ``cpu_baseline`` the CPU oracle (restated reference, OpenMP over all host cores) on a bounded
                 sample of the same workload.
* ``--impl reference`` times the CPU oracle as the reference arm (the reference's own SYCL build
                 needs AdaptiveCpp/LLVM, absent here and on the GPU host).

Multi-GPU: the path does not shard (no halo exchange is implemented); N ranks run N independent
replicas ("scaling": "weak") and `value` sums them.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W_DEFAULT, H_DEFAULT = 8192, 8192
VARIANT_STEPS = 200          # device-resident steps per storage form in `variants`
ERR_HEADLINE_STEPS = 50      # steps of the headline channel compared with the CPU oracle
BYTES_PER_NODE = {"f64_strict": 144.0, "f64_fast": 144.0, "f64_q60": 144.0, "f32_ref": 72.0, "f32": 72.0,
                  "f16s": 36.0, "bf16s": 36.0, "f16c": 36.0}


def circle_channel_mask(w: int, h: int) -> np.ndarray:
    """Walls on the first/last inner row and a disk of radius floor(H/8) at (floor(W/4), floor(H/2))
    (inner coordinates, 0-based)."""
    yy, xx = np.mgrid[0:h, 0:w]
    r = h // 8
    m = ((xx - w // 4) ** 2 + (yy - h // 2) ** 2 <= r * r).astype(np.int8)
    m[0, :] = 1
    m[h - 1, :] = 1
    return m


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d.get("bf16_tflops", 1900.0)),
                "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


class NvmlClocks:
    """Read-only NVML queries through ctypes (the driver's libnvidia-ml): SM clock, its maximum and
    the active clock event (throttle) reasons of one GPU.  None of the available() checks fail loudly:
    without the library the caller falls back to nvidia-smi."""

    # nvmlClocksEventReasons bits, in the order of ClockSampler's reason names
    REASON_BITS = (0x8, 0x40, 0x20, 0x4)   # hw_slowdown, hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap

    def __init__(self, index: int):
        import ctypes
        self.ct = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit")
        self.dev = ctypes.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(self.dev)) != 0:
            raise OSError("nvmlDeviceGetHandleByIndex")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        v = ctypes.c_uint()
        self.max_mhz = float(v.value) if self.lib.nvmlDeviceGetMaxClockInfo(self.dev, 1, ctypes.byref(v)) == 0 else 0.0

    def sample(self):
        """(SM MHz, maximum SM MHz, reason bits) now; NVML_CLOCK_SM is 1."""
        ct = self.ct
        v, r = ct.c_uint(), ct.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.dev, 1, ct.byref(v)) != 0:
            return None
        if self.reasons_fn(self.dev, ct.byref(r)) != 0:
            r.value = 0
        return float(v.value), self.max_mhz, r.value

    def close(self):
        self.lib.nvmlShutdown()


class ClockSampler:
    """Samples the SM clock and the throttle reasons while running: through NVML every millisecond
    where the library loads (a timed window of 20 steps is ~30 ms), else with nvidia-smi every
    `interval_ms`; summary() keeps the samples whose timestamp falls inside the timed steps'
    wall-clock window."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0, interval_ms: int = 20):
        self.index = index
        self.interval_ms = interval_ms
        self.proc = None
        self.lines: list[str] = []
        self.nvml_samples: list[tuple] = []
        self._nvml = None
        self._stop = threading.Event()
        self._t = None
        self.period_s = 0.001

    def _poll_nvml(self):
        while not self._stop.is_set():
            x = self._nvml.sample()
            if x is not None:
                self.nvml_samples.append((time.time(),) + x)
            time.sleep(self.period_s)

    def relax(self, period_s: float = 0.05):
        """Samples every `period_s` from now on (NVML queries every millisecond next to a run that
        synchronises with the driver from its own thread slowed the end-to-end run by ~25 %)."""
        self.period_s = period_s

    def __enter__(self):
        try:
            self._nvml = NvmlClocks(self.index)
            self._t = threading.Thread(target=self._poll_nvml, daemon=True)
            self._t.start()
            return self
        except Exception:
            self._nvml = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        self._stop.set()
        if self._nvml is not None:
            if self._t:
                self._t.join(timeout=2)
            self._nvml.close()
            self._nvml = None
            return
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self._t:
            self._t.join(timeout=2)

    def _samples(self):
        import datetime
        for t, clk, cmax, bits in self.nvml_samples:
            yield t, clk, cmax, ["Active" if bits & b else "Not Active" for b in NvmlClocks.REASON_BITS]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                t = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                yield t, float(parts[1]), float(parts[2]), parts[5:9]
            except ValueError:
                continue

    def summary(self, window=None) -> dict:
        """window: (t0, t1) in time.time() seconds; samples outside it (set-up, warm-up) are dropped.
        With no sample inside a short window, the samples within 0.3 s of it are used."""
        samples = list(self._samples())
        if window:
            t0, t1 = window
            inside = [x for x in samples if t0 <= x[0] <= t1]
            samples = inside or [x for x in samples if t0 - 0.3 <= x[0] <= t1 + 0.3]
        sm, smax, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for _, clk, cmax, flags in samples:
            sm.append(clk)
            smax = max(smax, cmax)
            for name, v in zip(names, flags):
                if v.lower() == "active":
                    reasons.add(name)
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
               "reasons": sorted(reasons), "samples": len(sm)}
        if window:
            out["window_s"] = round(window[1] - window[0], 3)
        return out


def make_props(plbm, alg, lay, w, h, steps, fui=None, wg=1024):
    return plbm.Properties(alg, lay, False, wg, steps, fui or steps, "Hagen-Poiseuille", h, w, 0.0, 0.0, 1.2, 0.0,
                           0.0, 1.0, 0.6)


def device_run(plbm, precision, alg, lay, w, h, mask, steps, warmup, tau=None, window=None):
    """K device-resident steps; returns (ms_per_step, handler).  `window` (a list) receives the
    wall-clock bounds of the timed steps (run_steps synchronises before it returns)."""
    props = make_props(plbm, alg, lay, w, h, steps + warmup + 10)
    if tau is not None:
        props.relaxation_time = float(tau)
    hd = plbm.create_handler(props, precision=precision, mask=mask)
    hd.run_steps(warmup)
    t0 = time.time()
    ms = hd.run_steps(steps)
    if window is not None:
        window[:] = [t0, time.time()]
    return ms, hd


def e2e_run(plbm, precision, alg, lay, w, h, mask, steps):
    """Public API, host buffers in and out: create (H2D mask), K steps, results D2H."""
    import torch
    pinned = torch.from_numpy(mask.reshape(-1)).pin_memory().numpy()
    t0 = time.perf_counter()
    hd = plbm.create_handler(make_props(plbm, alg, lay, w, h, steps), precision=precision, mask=pinned.reshape(h, w))
    hd.start()
    hd.block_until_finished()
    outs = [hd.get_densities(copy=False), hd.get_x_velocities(copy=False), hd.get_y_velocities(copy=False),
            hd.get_absolute_velocities(copy=False)]
    checksum = float(sum(float(o[:: max(1, o.size // 4096)].sum()) for o in outs))
    t1 = time.perf_counter()
    hd.close()
    return (t1 - t0) * 1e3, checksum


def cpu_oracle_sample(w, h, steps, mask, threads=None):
    """Times the CPU oracle (all OpenMP threads) on `steps` timesteps of the same workload."""
    from oracle import plbm_oracle
    plbm_oracle.build()
    o = plbm_oracle.Oracle("nptl", "stream", 1024, "Hagen-Poiseuille", w, h, inlet_density=1.2,
                           relaxation_time=0.6, mask=mask)
    o.run(1)
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    return w * h * steps / dt / 1e6, plbm_oracle.threads(), dt


def err_vs_oracle(plbm, precision, steps=2000, w=400, h=100, mask=None, alg="nptl", lay="stream", tau=0.6):
    """max |GPU - oracle| over rho, jx, jy after `steps` steps: by default the 400x100
    Hagen-Poiseuille channel; with `mask`, that channel (e.g. the headline circle channel)."""
    from oracle import plbm_oracle
    plbm_oracle.build()
    props = plbm.Properties(alg, lay, False, 1024, steps, steps, "Hagen-Poiseuille", h, w, 0.0, 0.0, 1.2,
                            0.0, 0.0, 1.0, tau)
    hd = plbm.create_handler(props, precision=precision, mask=mask)
    hd.start()
    hd.block_until_finished()
    got = [hd.get_densities(), hd.get_x_velocities(), hd.get_y_velocities()]
    hd.close()
    o = plbm_oracle.Oracle(alg, "stream", 1024, "Hagen-Poiseuille", w, h, inlet_density=1.2, relaxation_time=tau,
                           mask=mask)
    o.run(steps)
    err = 0.0
    for i, a in enumerate(got):
        err = max(err, float(np.max(np.abs(a - o.result(i)))))
    return err


def parity_drift(plbm, w=2000, h=500, checkpoints=(1000, 2000, 5000, 10000), taus=(0.55, 0.6, 1.0),
                 precisions=("f64_q60", "f64_fast")):
    """Growth of the FP64-accuracy forms' error against the oracle with the number of steps on the
    2000x500 circle channel (nptl, stream): max |GPU - oracle| over rho, jx, jy at each checkpoint,
    GPU handlers and the oracle advanced side by side."""
    from oracle import plbm_oracle
    plbm_oracle.build()
    mask = circle_channel_mask(w, h)
    out = {"domain": f"{w}x{h} circle channel, nptl+stream, rho 1.2/1.0", "rows": []}
    for tau in taus:
        o = plbm_oracle.Oracle("nptl", "stream", 1024, "Hagen-Poiseuille", w, h, inlet_density=1.2,
                               relaxation_time=tau, mask=mask)
        props = plbm.Properties("nptl", "stream", False, 1024, 10 ** 8, 10 ** 8, "Hagen-Poiseuille", h, w, 0.0, 0.0,
                                1.2, 0.0, 0.0, 1.0, tau)
        hds = {p: plbm.create_handler(props, precision=p, mask=mask) for p in precisions}
        done = 0
        for c in checkpoints:
            o.run(c - done)
            ref = [o.result(i) for i in range(3)]
            row = {"tau": tau, "steps": c,
                   "oracle_max_abs_j": float(max(np.nanmax(np.abs(ref[1])), np.nanmax(np.abs(ref[2]))))}
            for p, hd in list(hds.items()):
                try:
                    hd.run_steps(c - done)
                    hd.sync_results()
                except plbm.Exception as e:   # an unstable run leaves the form's range: recorded, not fatal
                    row[p] = f"stopped: {e}"
                    hd.close()
                    del hds[p]
                    continue
                got = [hd.get_densities(), hd.get_x_velocities(), hd.get_y_velocities()]
                row[p] = max(float(np.max(np.abs(a - b))) for a, b in zip(got, ref))
            done = c
            out["rows"].append(row)
        for hd in hds.values():
            hd.close()
    return out


# DRAM read + write bytes of one step launch, from ncu captures of the 4096^2 circle channel
# (profiles/), per inner node; geometry scales with the domain, so traffic is proportional.
TRAFFIC_PER_NODE = {"nptl_stream_f64_q60": 2.293e9 / (4096 * 4096), "nptl_stream_f64_fast": 2.283e9 / (4096 * 4096),
                    "nptl_stream_f32": 1.1375e9 / (4096 * 4096), "nptl_stream_f16s": 0.5923e9 / (4096 * 4096)}


def precision_study(plbm, w=1024, h=256, seed=12345, porosity=0.7, target=1e-6, max_steps=100000,
                    ref_target=1e-9, ref_cap=400000, big=(8192, 8192), big_steps=2000, big_cap=None, small=True,
                    forms=("f64_strict", "f64_fast", "f32", "f16s", "f16c", "bf16s")):
    """Each storage form against the FP64 steady state on a seeded porous channel (disks r in [3, 12],
    tau 0.6, rho 1.01 / 1.0).  The reference steady state is f64_q60 (FP64 accuracy, <= 1e-12 from
    the drop-in) run to residual `ref_target`; every form reports its steps and time to residual
    `target` (None where rounding keeps it above), then runs on towards `ref_target` (at most
    `max_steps` steps in all) and reports its final residual and the relative L2 error of its
    momentum field and relative total-mass difference against that reference.  (A run stopped at
    residual 1e-6 is still ~2e-3 from its steady state, so comparing there would charge the
    transient to the form.)  Then the same errors on the 8192^2 porous channel against f64_q60,
    after `big_steps` steps or, with `big_cap`, run to `target` with at most `big_cap` steps."""
    mask = plbm.porous_disks(w, h, seed, porosity)
    fluid = mask.reshape(-1) == 0

    def run(prec, mk, ww, hh, to_residual=True, steps=0, cap=max_steps, tgt=target):
        props = plbm.Properties("nptl", "stream", False, 1024, 10 ** 9, 10 ** 9, "Hagen-Poiseuille", hh, ww, 0.0,
                                0.0, 1.01, 0.0, 0.0, 1.0, 0.6)
        hd = plbm.create_handler(props, precision=prec, mask=mk)
        t0 = time.perf_counter()
        if to_residual:
            n, r = hd.run_to_residual(tgt, 100, cap)
        else:
            hd.run_steps(steps)
            hd.sync_results()
            n, r = steps, None
        dt = time.perf_counter() - t0
        out = (hd.get_densities(), hd.get_x_velocities(), hd.get_y_velocities())
        hd.close()
        return n, r, dt, out

    def run_to_steady(prec, mk, ww, hh):
        """Steps and time to residual `target`, then on to `ref_target` (the form's steady state, or
        its rounding plateau) within `max_steps` in all; the fields are those of the end."""
        props = plbm.Properties("nptl", "stream", False, 1024, 10 ** 9, 10 ** 9, "Hagen-Poiseuille", hh, ww, 0.0,
                                0.0, 1.01, 0.0, 0.0, 1.0, 0.6)
        hd = plbm.create_handler(props, precision=prec, mask=mk)
        t0 = time.perf_counter()
        n1, r1 = hd.run_to_residual(target, 100, max_steps)
        dt = time.perf_counter() - t0
        n2, r2 = hd.run_to_residual(ref_target, 100, max_steps - n1) if n1 < max_steps else (0, r1)
        out = (hd.get_densities(), hd.get_x_velocities(), hd.get_y_velocities())
        hd.close()
        reached = r1 < target
        return {"steps_to_target": n1 if reached else None, "seconds_to_target": round(dt, 3) if reached else None,
                "steps": n1 + n2, "residual": r2}, out

    def errs(a, b, fl):
        ja = np.concatenate([a[1][fl], a[2][fl]])
        jb = np.concatenate([b[1][fl], b[2][fl]])
        return (float(np.linalg.norm(ja - jb) / np.linalg.norm(jb)),
                float((a[0][fl].sum() - b[0][fl].sum()) / b[0][fl].sum()))

    study = {"target_residual": target}
    if small:
        nref, rref, tref, ref = run("f64_q60", mask, w, h, cap=ref_cap, tgt=ref_target)
        study.update({"domain": f"{w}x{h} porous (seed {seed}, porosity {porosity})",
                      "reference": {"precision": "f64_q60", "steps": nref, "residual": rref,
                                    "seconds": round(tref, 3)}})
        for prec in forms:
            rec, out = run_to_steady(prec, mask, w, h)
            l2, dm = errs(out, ref, fluid)
            study[prec] = dict(rec, rel_l2_j_vs_f64=l2, mass_rel_diff_vs_f64=dm)
        # the 16-bit forms finished in FP32: stepped in 16 bits until a 1000-step chunk no longer
        # lowers the residual (the form's rounding floor), re-encoded in FP32 (plbm_set_precision),
        # on to the target; then on towards ref_target for the comparison
        rec, _ = run_to_steady("f64_q60", mask, w, h)
        study["f64_q60_to_target"] = {"steps": rec["steps_to_target"], "seconds": rec["seconds_to_target"]}
        for prec in [f for f in forms if f in ("f16s", "f16c", "bf16s")]:
            props = plbm.Properties("nptl", "stream", False, 1024, 10 ** 9, 10 ** 9, "Hagen-Poiseuille", h, w, 0.0,
                                    0.0, 1.01, 0.0, 0.0, 1.0, 0.6)
            hd = plbm.create_handler(props, precision=prec, mask=mask)
            t0 = time.perf_counter()
            n1, r1, switched = hd.run_to_residual_escalating(target, 100, max_steps)
            dt = time.perf_counter() - t0
            n2, r2 = hd.run_to_residual(ref_target, 100, max_steps - n1) if n1 < max_steps else (0, r1)
            out = (hd.get_densities(), hd.get_x_velocities(), hd.get_y_velocities())
            hd.close()
            l2, dm = errs(out, ref, fluid)
            reached = r1 < target
            study[prec + "_then_f32"] = {"steps_to_target": n1 if reached else None,
                                         "seconds_to_target": round(dt, 3) if reached else None,
                                         "switched_at_step": switched, "steps": n1 + n2, "residual": r2,
                                         "rel_l2_j_vs_f64": l2, "mass_rel_diff_vs_f64": dm}
    bw, bh = big
    bmask = plbm.porous_disks(bw, bh, seed, porosity)
    bfl = bmask.reshape(-1) == 0
    conv = big_cap is not None
    nref, rref, tref, bref = run("f64_q60", bmask, bw, bh, conv, big_steps, big_cap or 0)
    study["large"] = {"domain": f"{bw}x{bh} porous (seed {seed}, porosity {porosity}), against f64_q60",
                      "f64_q60": {"steps": nref, "residual": rref, "seconds": round(tref, 1)}}
    if not conv:
        study["large"]["domain"] += f", {big_steps} steps"
    for prec in ("f32", "f16s", "f16c", "bf16s"):
        n, r, dt, out = run(prec, bmask, bw, bh, conv, big_steps, big_cap or 0)
        l2, dm = errs(out, bref, bfl)
        study["large"][prec] = {"steps": n, "residual": r, "seconds": round(dt, 1), "rel_l2_j": l2,
                                "mass_rel_diff": dm}
    return study


def batch_domains(plbm, n=256, seed=2024):
    """256 independent porous channels: W, H uniform in 64..1024, disks r in [3, 12] at porosity
    uniform in [0.6, 0.8], tau uniform in [0.55, 1.0], inlet density uniform in [1.001, 1.05]."""
    rng = np.random.default_rng(seed)
    doms = []
    for i in range(n):
        w, h = int(rng.integers(64, 1025)), int(rng.integers(64, 1025))
        doms.append({"mask": plbm.porous_disks(w, h, seed * 1000 + i, float(rng.uniform(0.6, 0.8))),
                     "relaxation_time": float(rng.uniform(0.55, 1.0)),
                     "inlet_density": float(rng.uniform(1.001, 1.05)), "outlet_density": 1.0})
    return doms


def parse_batch_tile(text, plbm):
    """"W,TY,ROWS,BLOCKS[,vec]" -> Batch.set_tile's (tile_w, tile_h, blocks_per_sm)."""
    parts = text.split(",")
    w, ty, rows, blocks = (int(v) for v in parts[:4])
    vec = len(parts) > 4 and parts[4] == "vec"
    return w, ty + 256 * rows + (plbm.BATCH_TILE_VEC if vec else 0), blocks


def batch_study(plbm, steps=100, precisions=("f32", "f16s"), n=256, tile=None):
    """Aggregate MLUPS of `n` uneven domains: one persistent tile-queue launch per step replayed from a
    CUDA graph (tiles autotuned, or `tile` = set_tile's arguments for the 2-byte forms) against one
    launch per domain per step."""
    doms = batch_domains(plbm, n=n)
    out = {"domains": len(doms)}
    for prec in precisions:
        b = plbm.Batch(doms, precision=prec)
        nodes, _ = b.info()
        if tile is not None and BYTES_PER_NODE[prec] == 36:
            b.set_tile(*tile)
            used = tuple(tile)
        else:
            used = b.autotune(steps=3)
        _, tiles = b.info()
        b.run(16, mode="persistent_graph")
        ms_graph = b.run(steps, mode="persistent_graph")
        ms_pers = b.run(steps, mode="persistent")
        b.run(4, mode="per_domain")
        ms_per = b.run(steps, mode="per_domain")
        bpn = BYTES_PER_NODE[prec]
        out[prec] = {"nodes": nodes, "tiles": tiles,
                     "tile": {"threads": [used[0], used[1] & 255], "rows_per_thread": max(1, (used[1] >> 8) & 255),
                              "vectorised_rows": bool(used[1] & plbm.BATCH_TILE_VEC),
                              "blocks_per_sm": used[2], "autotuned": tile is None or BYTES_PER_NODE[prec] != 36},
                     "mlups_persistent_graph": round(nodes / ms_graph / 1e3, 1),
                     "mlups_persistent": round(nodes / ms_pers / 1e3, 1),
                     "mlups_per_domain_launches": round(nodes / ms_per / 1e3, 1),
                     "hbm_gbs_persistent_graph": round(bpn * nodes / ms_graph / 1e6, 1)}
        b.close()
    return out


def sweep(plbm, steps=50, warmup=5, sizes=((2000, 500), (8192, 8192)), taus=(0.55, 0.6, 1.0),
          precisions=("f64_q60", "f64_strict")):
    """The FP64 drop-in sweep: every algorithm x data layout on the circle channel (disk of radius
    H/8 at W/4, walls, rho 1.2 / 1.0) at each size and relaxation time, device-resident steps timed
    with CUDA events; MLUPS, algorithmic GB/s (144 B/node) and the fraction of measured HBM."""
    pk = peaks()
    rows = []
    for w, h in sizes:
        mask = circle_channel_mask(w, h)
        for prec in precisions:
            for tau in taus:
                for alg in ("nptl", "lptl", "npol", "nsol"):
                    for lay in ("stream", "collision", "bundle"):
                        ms, hd = device_run(plbm, prec, alg, lay, w, h, mask, steps, warmup, tau)
                        hd.close()
                        gbs = BYTES_PER_NODE[prec] * w * h / (ms * 1e-3) / 1e9
                        rows.append({"size": f"{w}x{h}", "precision": prec, "tau": tau, "algorithm": alg,
                                     "data_layout": lay, "mlups": round(w * h / ms / 1e3, 1), "hbm_gbs": round(gbs, 1),
                                     "frac_of_hbm": round(gbs / pk["hbm_gbs"], 4)})
    return {"steps": steps, "peak_hbm_gbs": pk["hbm_gbs"], "rows": rows}


def nn_bench(batch=16, size=256, reps=5):
    """Times the warm-start operator's kernels (csrc/plbm_nn.cu): one training step (forward,
    backward, Adam) on `batch` channels of size^2 and one inference of a single channel, with
    the convolution FLOPs (2 * pixels * 9 * Cin * Cout per layer; backward = 2 x forward).
    Each is timed launched from Python and as a replayed CUDA graph."""
    import numpy as np
    import torch
    from portlbm_gb300 import warmstart as ws
    model = ws.NeuralOperator(0)
    rng = np.random.default_rng(0)

    def flops(n):
        f, h = 0.0, size
        for lvl in range(5):
            for ci, co in ws.ENC[2 * lvl:2 * lvl + 2]:
                f += 2.0 * n * (h >> lvl) ** 2 * 9 * ci * co
        for k, lvl in enumerate((3, 2, 1, 0)):
            for ci, co in ws.DEC[2 * k:2 * k + 2]:
                f += 2.0 * n * (h >> lvl) ** 2 * 9 * ci * co
        return f + 2.0 * n * h * h * 9 * ws.HEAD[0] * ws.HEAD[1]

    masks = torch.from_numpy((rng.random((batch, size, size)) < 0.3).astype(np.int8)).cuda()
    x = model.assemble(masks, [ws.features(size, 1.02, 1.0, 0.8)] * batch)
    grad = torch.zeros((batch, size, size, 3), dtype=torch.bfloat16, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for it in range(reps + 2):
        if it == 2:
            torch.cuda.synchronize()
            e0.record()
        model.forward(x, batch, size, size)
        model.zero_grad()
        model.backward(grad)
        model.adam(lr=0.0)
    e1.record()
    torch.cuda.synchronize()
    eager_ms = e0.elapsed_time(e1) / reps
    x1 = x[:1].contiguous()
    for it in range(reps + 2):
        if it == 2:
            torch.cuda.synchronize()
            e0.record()
        model.forward(x1, 1, size, size)
    e1.record()
    torch.cuda.synchronize()
    infer_eager_ms = e0.elapsed_time(e1) / reps

    def replayed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    # the same step and inference as CUDA graphs (one launch from the host each)
    step = model.capture_train_step(x, grad, batch, size, size)
    train_ms = replayed(lambda: step(0.0))
    run, _ = model.capture_forward(x1, 1, size, size)
    infer_ms = replayed(run)
    pk = peaks()
    train_tf = 3 * flops(batch) / (train_ms * 1e-3) / 1e12
    infer_tf = flops(1) / (infer_ms * 1e-3) / 1e12
    return {"train_step_ms": round(train_ms, 3), "train_tflops": round(train_tf, 2),
            "infer_ms": round(infer_ms, 3), "infer_tflops": round(infer_tf, 2),
            "train_step_eager_ms": round(eager_ms, 3), "infer_eager_ms": round(infer_eager_ms, 3),
            "bf16_peak_tflops": pk["bf16_tflops"], "train_frac_of_bf16_peak": round(train_tf / pk["bf16_tflops"], 4),
            "config": f"U-Net 32-128 channels, train batch {batch} x {size}^2, inference 1 x {size}^2; "
                      "train_step_ms / infer_ms replay CUDA graphs, *_eager_ms launch from Python"}


def load_traffic(kind: str, nodes: int):
    v = TRAFFIC_PER_NODE.get(kind)
    return None if v is None else round(v * nodes)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def max_over_ranks(v: float, world: int, device: str = "cuda") -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


METRIC = "MLUPS (FP64 D2Q9 BGK, 8192x8192 circle channel)"


def line_config(args, world) -> dict:
    """The `config` of both arms' JSON lines (the reference arm reports the same workload)."""
    w, h = args.width, args.height
    return {"workload": f"circle channel {w}x{h} (r=H/8 at W/4), {args.algorithm}+{args.layout}, tau 0.6, "
                        f"rho 1.2/1.0", "algorithm": args.algorithm, "data_layout": args.layout,
            "precision": args.precision, "l2": "inputs larger than L2 (lattice %.1f GB)" % (2 * 9 * 8 * w * h / 1e9),
            "parallelism": f"replicas{world}"}


def run_reference(args, world, rank, budget_s=90.0):
    """Reference arm: the CPU oracle on the host cores, rank 0 only.  Each step is a bounded sample
    of the workload: when the whole run would take more than `budget_s`, the steps are taken over
    a centred band of the channel's rows (full width, the disk, walls on the band's edges) sized to
    fit, and the line says so."""
    if rank != 0:
        return
    w, h = args.width, args.height
    mask = circle_channel_mask(w, h)
    per_step = []
    from oracle import plbm_oracle
    plbm_oracle.build()

    def oracle(rows):
        m = mask if rows == h else mask[(h - rows) // 2:(h - rows) // 2 + rows].copy()
        m[0, :] = 1
        m[-1, :] = 1
        return plbm_oracle.Oracle(args.algorithm, args.layout, 1024, "Hagen-Poiseuille", w, rows, inlet_density=1.2,
                                  relaxation_time=0.6, mask=np.ascontiguousarray(m))

    rows = h
    o = oracle(rows)
    t = time.perf_counter()
    o.run(2)
    t_full = (time.perf_counter() - t) / 2
    if (args.steps + args.warmup) * t_full > budget_s:
        rows = max(64, int(h * budget_s / ((args.steps + args.warmup) * t_full)))
        if rows < h:
            o = oracle(rows)
    for _ in range(args.warmup):
        o.run(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t = time.perf_counter()
        o.run(1)
        per_step.append(time.perf_counter() - t)
    dt = time.perf_counter() - t0
    mlups = w * rows * args.steps / dt / 1e6
    sample = (f"{args.steps} full {w}x{h} timesteps" if rows == h else
              f"{args.steps} timesteps of a {w}x{rows} band of the {w}x{h} channel (full width, the disk)")
    line = {"metric": METRIC, "value": round(mlups, 2), "unit": "MLUPS",
            "impl": "reference", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * dt / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": line_config(args, world),
            "cpu_baseline": {"value": round(mlups, 2), "unit": "MLUPS", "cores": plbm_oracle.threads(),
                             "kind": "port",
                             "sample": f"{sample} of the CPU oracle (restated reference, OpenMP) after warm-up"},
            "e2e": {"value": round(mlups, 2), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=W_DEFAULT)
    ap.add_argument("--height", type=int, default=H_DEFAULT)
    ap.add_argument("--precision", default="f64_q60", choices=list(BYTES_PER_NODE))
    ap.add_argument("--algorithm", default="nptl")
    ap.add_argument("--layout", default="stream")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=0, help="CPU-baseline sample steps (0: auto)")
    ap.add_argument("--kernel-only", action="store_true", help="only the device-resident timed region (profiling)")
    ap.add_argument("--no-study", action="store_true", help="skip the precision study")
    ap.add_argument("--warmstart-study", action="store_true",
                    help="only the learned warm-start study: train on 2000 solver steady states (256x256), "
                         "then time-to-residual 1e-6 from rest vs from the prediction on 200 held-out channels")
    ap.add_argument("--warmstart-train", type=int, default=2000)
    ap.add_argument("--warmstart-test", type=int, default=200)
    ap.add_argument("--warmstart-save", default=None, help="write the trained weights (.npz) here")
    ap.add_argument("--batch-study-only", action="store_true", help="only the batching study")
    ap.add_argument("--precision-study-large", type=int, default=0, metavar="CAP",
                    help="only the 8192^2 porous precision study, each form run to residual 1e-6 "
                         "with at most CAP steps")
    ap.add_argument("--batch-domains", type=int, default=256)
    ap.add_argument("--batch-tile", default=None,
                    help="fixed tile for the 2-byte batch instead of the autotuner: W,THREADS_Y,ROWS,BLOCKS_PER_SM[,vec]")
    ap.add_argument("--nn-bench", action="store_true", help="only the warm-start operator's kernel timings")
    ap.add_argument("--sweep", action="store_true",
                    help="only the FP64 sweep: 4 algorithms x 3 layouts x tau {0.55, 0.6, 1.0} at 2000x500 and 8192^2")
    ap.add_argument("--parity-drift", action="store_true",
                    help="only the error growth of f64_q60 / f64_fast against the oracle (2000x500, up to 10^4 steps)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import portlbm_gb300 as plbm
    from portlbm_gb300 import build as b
    b.build()
    if args.batch_study_only or args.nn_bench or args.sweep or args.precision_study_large or args.parity_drift:
        if rank == 0:
            if args.sweep:
                key, res = "sweep", sweep(plbm)
            elif args.parity_drift:
                key, res = "parity_drift", parity_drift(plbm)
            elif args.precision_study_large:
                key, res = "precision_study_large", precision_study(plbm, big_cap=args.precision_study_large,
                                                                    small=False)
            else:
                key, res = (("batch_study", batch_study(plbm, n=args.batch_domains,
                                                          tile=parse_batch_tile(args.batch_tile, plbm)
                                                          if args.batch_tile else None)) if args.batch_study_only
                            else ("nn_bench", nn_bench()))
            print(json.dumps({key: res}), flush=True)
        return
    if args.warmstart_study:
        if rank == 0:
            from portlbm_gb300 import warmstart
            t0 = time.perf_counter()
            res = warmstart.study(n_train=args.warmstart_train, n_test=args.warmstart_test,
                                  save=args.warmstart_save, log=lambda m: print(m, file=sys.stderr, flush=True))
            res["wall_s"] = round(time.perf_counter() - t0, 1)
            print(json.dumps({"warmstart_study": res}), flush=True)
        return
    w, h = args.width, args.height
    mask = circle_channel_mask(w, h)
    pk = peaks()

    # -- device-resident timed region (value + roofline) --
    barrier(world)
    window = []
    # sampled from the first device step to the end of the e2e and variant runs (every 50 ms after
    # the device-timed steps): `clocks` keeps the timed window, `clocks_run` every sample of that
    # busy stretch
    clocks = ClockSampler(local).__enter__()
    run_t0 = time.time()
    ms, hd = device_run(plbm, args.precision, args.algorithm, args.layout, w, h, mask, args.steps, args.warmup,
                        window=window)
    barrier(world)
    ms = max_over_ranks(ms, world)
    launches = hd.launches_per_step() * args.steps
    bpn = BYTES_PER_NODE[args.precision]
    mlups_rank = w * h / (ms * 1e-3) / 1e6
    value = mlups_rank * world
    achieved_gbs = bpn * w * h / (ms * 1e-3) / 1e9
    hd.close()

    if args.kernel_only:
        clocks.__exit__()
        if rank == 0:
            print(json.dumps({"value": round(value, 1), "unit": "MLUPS", "ms_per_step": round(ms, 4),
                              "achieved_gbs": round(achieved_gbs, 1), "precision": args.precision}), flush=True)
        return

    # -- end-to-end through the public API with host buffers --
    clocks.relax()
    e2e_steps = args.steps
    e2e_ms, _ = e2e_run(plbm, args.precision, args.algorithm, args.layout, w, h, mask, e2e_steps)
    e2e_ms = max_over_ranks(e2e_ms, world)
    e2e_mlups = world * w * h * e2e_steps / (e2e_ms * 1e-3) / 1e6

    # -- other forms of the same step (device-resident, same K), reported beside --
    # Each form is timed over VARIANT_STEPS device-resident steps whatever --steps is, so that the
    # one observables-writing step that ends a run weighs < 1 % of the window.
    variants = {}
    if not args.no_variants and rank == 0:
        for prec in ("f64_q60", "f64_strict", "f64_fast", "f32", "f16s", "f16c", "bf16s"):
            vms, vh = device_run(plbm, prec, args.algorithm, args.layout, w, h, mask, VARIANT_STEPS, 10)
            vh.close()
            variants[prec] = {"mlups": round(w * h / vms / 1e3, 1), "ms_per_step": round(vms, 4),
                              "steps": VARIANT_STEPS,
                              "hbm_gbs": round(BYTES_PER_NODE[prec] * w * h / vms / 1e6, 1),
                              "frac_of_hbm": round(BYTES_PER_NODE[prec] * w * h / vms / 1e6 / pk["hbm_gbs"], 4)}
        variants["ratios"] = {f"{p}_over_{q}": round(variants[p]["mlups"] / variants[q]["mlups"], 3)
                              for p in ("f16s", "f16c") for q in ("f64_q60", "f64_strict")}

    run_t1 = time.time()
    clocks.__exit__()
    err = None
    if rank == 0:
        err = {"poiseuille_400x100_2000_steps": err_vs_oracle(plbm, args.precision),
               f"circle_{w}x{h}_{ERR_HEADLINE_STEPS}_steps": err_vs_oracle(plbm, args.precision, ERR_HEADLINE_STEPS,
                                                                           w, h, mask=mask, alg=args.algorithm,
                                                                           lay=args.layout)}
    study = precision_study(plbm) if (rank == 0 and not args.no_study and not args.no_variants) else None
    batch = batch_study(plbm) if (rank == 0 and not args.no_study and not args.no_variants) else None
    # the warm-start operator's kernels (a few seconds): training step and inference times
    try:
        nn = nn_bench() if (rank == 0 and not args.no_study and not args.no_variants) else None
    except Exception as exc:   # recorded, never fatal to the solver's line
        nn = {"error": str(exc)[:200]}

    # -- CPU baseline (rank 0, N = 1) --
    cpu = None
    if rank == 0 and world == 1:
        steps = args.cpu_steps or 20
        v, cores, dt = cpu_oracle_sample(w, h, steps, mask)
        cpu = {"value": round(v, 2), "unit": "MLUPS", "cores": cores, "kind": "port",
               "sample": f"{steps} full {w}x{h} timesteps of the CPU oracle (restated reference, OpenMP, "
                         f"{dt:.1f} s)"}

    if rank == 0:
        traffic = load_traffic(f"{args.algorithm}_{args.layout}_{args.precision}", w * h)
        line = {
            "metric": METRIC,
            "value": round(value, 1), "unit": "MLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int64 (Q3.60 fixed point, FP64 accuracy)" if args.precision == "f64_q60" else "f64",
            "data": "synthetic", "err_vs_oracle": err,
            "config": line_config(args, world),
            "roofline": {"bound": "hbm", "achieved": round(achieved_gbs, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": round(achieved_gbs / pk["hbm_gbs"], 4), "traffic": traffic,
                         # DRAM bytes the launch actually moves (ncu traffic; solid nodes move none)
                         # over the same live launch time
                         "dram_frac": (round(traffic / (ms * 1e-3) / 1e9 / pk["hbm_gbs"], 4)
                                       if traffic else None),
                         "peak_source": pk["source"],
                         "note": ("f64_strict/f64_fast are bound by the FP64 pipe (0.5 T DP instr/s measured); "
                                  "f64_q60 runs the update on the integer pipe")},
            "e2e": {"value": round(e2e_mlups, 1), "unit": "MLUPS", "h2d_bytes_per_step": round(w * h / e2e_steps),
                    "d2h_bytes_per_step": round(4 * 8 * w * h / e2e_steps)},
            "gpu_launches": launches,
            "clocks": clocks.summary(window),
            "clocks_run": clocks.summary((run_t0, run_t1)),
            "cpu_baseline": cpu,
            "variants": variants,
            "precision_study": study,
            "batch_study": batch,
            "nn_bench": nn,
        }
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

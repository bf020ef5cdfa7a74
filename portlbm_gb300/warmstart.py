"""Learned warm start: a convolutional neural operator that maps a porous channel (solid mask,
inlet/outlet density, relaxation time) to a predicted steady state (rho, jx, jy).  The solver is
then initialised with the equilibrium populations of the prediction and iterates to the same
residual as from rest; it falls back to the rest state whenever the prediction's first residual
is worse.  No counterpart in the reference (PortLBM always starts from rest,
include/lbm/core/domain_initialization.hpp:311-333).

Network (all 3x3 convolutions, BF16 weights/activations, FP32 accumulation, on the project's own
tensor-core kernels in csrc/plbm_nn.cu; torch only provides device buffers):

    encoder  4->32->32 | pool | 32->64->64 | pool | 64->96->96 | pool | 96->128->128 | pool | 128->128->128
    decoder  per level: nearest x2, conv to the level's width (ReLU), + encoder skip, conv (ReLU)
    head     32->3   (targets: (rho - 1) and j, each divided by its training-set std)

Training data are steady states the solver itself produces (batches of porous channels,
csrc/plbm_batch.cu), see `generate_dataset`.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import Batch, Properties, create_handler, load_library, porous_disks

C_IN = 4
ENC = [(C_IN, 32), (32, 32), (32, 64), (64, 64), (64, 96), (96, 96), (96, 128), (128, 128), (128, 128), (128, 128)]
DEC = [(128, 128), (128, 128), (128, 96), (96, 96), (96, 64), (64, 64), (64, 32), (32, 32)]
HEAD = (32, 3)
WIDTHS = [32, 64, 96, 128, 128]


def _fns():
    lib = load_library()
    vp, i, ll, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_float
    sig = {
        "plbm_nn_conv_fwd": [vp, vp, vp, vp, i, i, i, i, i, i, vp],
        "plbm_nn_conv_dgrad": [vp, vp, vp, i, i, i, i, i, vp],
        "plbm_nn_conv_wgrad": [vp, vp, vp, vp, i, i, i, i, i, vp],
        "plbm_nn_relu_bwd": [vp, vp, ll, vp],
        "plbm_nn_pool2": [vp, vp, i, i, i, i, vp],
        "plbm_nn_pool2_bwd": [vp, vp, i, i, i, i, vp],
        "plbm_nn_up2": [vp, vp, i, i, i, i, vp],
        "plbm_nn_up2_bwd": [vp, vp, i, i, i, i, vp],
        "plbm_nn_add": [vp, vp, vp, ll, vp],
        "plbm_nn_mse": [vp, vp, vp, vp, vp, ll, i, f, vp],
        "plbm_nn_adam": [vp, vp, vp, vp, vp, ll, f, f, f, f, i, vp],
        "plbm_nn_assemble": [vp, vp, vp, vp, vp, i, i, i, i, vp],
        "plbm_set_equilibrium": [vp, vp, vp, vp],
    }
    for name, args in sig.items():
        getattr(lib, name).argtypes = args
        getattr(lib, name).restype = ctypes.c_int
    return lib


def _ok(rc):
    if rc != 0:
        raise RuntimeError(f"plbm_nn call failed ({rc})")


class ConvLayer:
    def __init__(self, cin, cout, relu, rng, torch):
        self.cin, self.cout, self.relu = cin, cout, relu
        w = (rng.standard_normal((cout, 9 * cin)) * np.sqrt(2.0 / (9 * cin))).astype(np.float32)
        self.w = torch.from_numpy(w).cuda()                        # FP32 master
        assert self.w.dtype == torch.float32
        self.wb = self.w.to(torch.bfloat16)                         # BF16 copy used by the kernels
        self.b = torch.zeros(cout, dtype=torch.float32, device="cuda")
        self.gw = torch.zeros_like(self.w)
        self.gb = torch.zeros_like(self.b)
        self.m = [torch.zeros_like(self.w), torch.zeros_like(self.b)]
        self.v = [torch.zeros_like(self.w), torch.zeros_like(self.b)]


class NeuralOperator:
    """U-Net-style operator; forward/backward/Adam all run in libplbm's kernels."""

    def __init__(self, seed: int = 0):
        import torch
        self.torch = torch
        self.lib = _fns()
        rng = np.random.default_rng(seed)
        self.enc = [ConvLayer(ci, co, True, rng, torch) for ci, co in ENC]
        self.dec = [ConvLayer(ci, co, True, rng, torch) for ci, co in DEC]
        self.head = ConvLayer(HEAD[0], HEAD[1], False, rng, torch)
        self.layers = self.enc + self.dec + [self.head]
        self.scale = np.array([1.0, 1.0, 1.0], dtype=np.float32)
        self.step_count = 0

    def _buf(self, n, h, w, c):
        return self.torch.empty((n, h, w, c), dtype=self.torch.bfloat16, device="cuda")

    def _conv(self, layer, x, n, h, w):
        y = self._buf(n, h, w, layer.cout)
        _ok(self.lib.plbm_nn_conv_fwd(x.data_ptr(), layer.wb.data_ptr(), layer.b.data_ptr(), y.data_ptr(), n, h, w,
                                      layer.cin, layer.cout, int(layer.relu), None))
        return y

    def forward(self, x, n, h, w):
        """x: [n,h,w,4] bf16 input; returns the [n,h,w,3] prediction and keeps activations for backward."""
        acts = {"in": x}
        cur, hh, ww = x, h, w
        skips = []
        for lvl in range(5):
            a = self._conv(self.enc[2 * lvl], cur, n, hh, ww)
            b = self._conv(self.enc[2 * lvl + 1], a, n, hh, ww)
            acts[f"e{lvl}a"], acts[f"e{lvl}b"] = a, b
            skips.append((b, hh, ww))
            if lvl < 4:
                p = self._buf(n, hh // 2, ww // 2, b.shape[-1])
                _ok(self.lib.plbm_nn_pool2(b.data_ptr(), p.data_ptr(), n, hh, ww, b.shape[-1], None))
                acts[f"p{lvl}"] = p
                cur, hh, ww = p, hh // 2, ww // 2
            else:
                cur = b
        for k, lvl in enumerate((3, 2, 1, 0)):
            sh, sw = skips[lvl][1], skips[lvl][2]
            u = self._buf(n, sh, sw, cur.shape[-1])
            _ok(self.lib.plbm_nn_up2(cur.data_ptr(), u.data_ptr(), n, sh, sw, cur.shape[-1], None))
            a = self._conv(self.dec[2 * k], u, n, sh, sw)
            s = self._buf(n, sh, sw, a.shape[-1])
            _ok(self.lib.plbm_nn_add(a.data_ptr(), skips[lvl][0].data_ptr(), s.data_ptr(), s.numel(), None))
            b = self._conv(self.dec[2 * k + 1], s, n, sh, sw)
            acts[f"u{lvl}"], acts[f"d{lvl}a"], acts[f"s{lvl}"], acts[f"d{lvl}b"] = u, a, s, b
            cur = b
        out = self._conv(self.head, cur, n, h, w)
        acts["out"] = out
        self.acts, self.shape = acts, (n, h, w)
        return out

    def _conv_bwd(self, layer, x, y, gy, n, h, w, need_gx=True):
        if layer.relu:
            _ok(self.lib.plbm_nn_relu_bwd(y.data_ptr(), gy.data_ptr(), gy.numel(), None))
        _ok(self.lib.plbm_nn_conv_wgrad(x.data_ptr(), gy.data_ptr(), layer.gw.data_ptr(), layer.gb.data_ptr(), n, h,
                                        w, layer.cin, layer.cout, None))
        if not need_gx:
            return None
        gx = self._buf(n, h, w, layer.cin)
        _ok(self.lib.plbm_nn_conv_dgrad(gy.data_ptr(), layer.wb.data_ptr(), gx.data_ptr(), n, h, w, layer.cin,
                                        layer.cout, None))
        return gx

    def backward(self, gout):
        a, (n, h, w) = self.acts, self.shape
        g = self._conv_bwd(self.head, a["d0b"], a["out"], gout, n, h, w)
        gskip = {}
        sizes = {lvl: (h >> lvl, w >> lvl) for lvl in range(5)}
        for k, lvl in enumerate((0, 1, 2, 3)):
            kk = 3 - k
            sh, sw = sizes[lvl]
            gs = self._conv_bwd(self.dec[2 * kk + 1], a[f"s{lvl}"], a[f"d{lvl}b"], g, n, sh, sw)
            gskip[lvl] = gs                                     # the skip addition passes g to both inputs
            gu = self._conv_bwd(self.dec[2 * kk], a[f"u{lvl}"], a[f"d{lvl}a"], gs.clone(), n, sh, sw)
            ch, cw = sizes[lvl + 1]
            g = self._buf(n, ch, cw, gu.shape[-1])
            _ok(self.lib.plbm_nn_up2_bwd(gu.data_ptr(), g.data_ptr(), n, ch, cw, gu.shape[-1], None))
        for lvl in (4, 3, 2, 1, 0):
            hh, ww = sizes[lvl]
            if lvl < 4:
                # gradient of e{lvl}b: skip gradient + pooled path gradient
                gp = self._buf(n, hh, ww, g.shape[-1])
                _ok(self.lib.plbm_nn_pool2_bwd(g.data_ptr(), gp.data_ptr(), n, hh, ww, g.shape[-1], None))
                gb_ = self._buf(n, hh, ww, g.shape[-1])
                _ok(self.lib.plbm_nn_add(gp.data_ptr(), gskip[lvl].data_ptr(), gb_.data_ptr(), gb_.numel(), None))
                g = gb_
            xin = a["in"] if lvl == 0 else a[f"p{lvl - 1}"]
            ga = self._conv_bwd(self.enc[2 * lvl + 1], a[f"e{lvl}a"], a[f"e{lvl}b"], g, n, hh, ww)
            g = self._conv_bwd(self.enc[2 * lvl], xin, a[f"e{lvl}a"], ga, n, hh, ww, need_gx=lvl > 0)

    def zero_grad(self):
        for layer in self.layers:
            layer.gw.zero_()
            layer.gb.zero_()

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        for layer in self.layers:
            _ok(self.lib.plbm_nn_adam(layer.w.data_ptr(), layer.gw.data_ptr(), layer.m[0].data_ptr(),
                                      layer.v[0].data_ptr(), layer.wb.data_ptr(), layer.w.numel(), lr, b1, b2, eps,
                                      self.step_count, None))
            _ok(self.lib.plbm_nn_adam(layer.b.data_ptr(), layer.gb.data_ptr(), layer.m[1].data_ptr(),
                                      layer.v[1].data_ptr(), None, layer.b.numel(), lr, b1, b2, eps, self.step_count,
                                      None))

    def assemble(self, masks, rin, rout, tau):
        torch = self.torch
        n, h, w = masks.shape
        x = self._buf(n, h, w, C_IN)
        r1 = torch.tensor(rin, dtype=torch.float32, device="cuda")
        r2 = torch.tensor(rout, dtype=torch.float32, device="cuda")
        t = torch.tensor(tau, dtype=torch.float32, device="cuda")
        _ok(self.lib.plbm_nn_assemble(masks.data_ptr(), r1.data_ptr(), r2.data_ptr(), t.data_ptr(), x.data_ptr(), n, h,
                                      w, C_IN, None))
        return x

    def predict(self, mask: np.ndarray, rin: float, rout: float, tau: float):
        """Predicted (rho, jx, jy) fields (float64, H*W) for one channel."""
        torch = self.torch
        m = torch.from_numpy(np.ascontiguousarray(mask, dtype=np.int8)[None]).cuda()
        x = self.assemble(m, [rin], [rout], [tau])
        out = self.forward(x, 1, mask.shape[0], mask.shape[1]).float().cpu().numpy().reshape(-1, 3)
        rho = 1.0 + out[:, 0] / self.scale[0]
        jx, jy = out[:, 1] / self.scale[1], out[:, 2] / self.scale[2]
        return rho.astype(np.float64), jx.astype(np.float64), jy.astype(np.float64)


def random_channel(rng, w, h):
    return dict(mask=porous_disks(w, h, int(rng.integers(1 << 62)), float(rng.uniform(0.6, 0.8))),
                tau=float(rng.uniform(0.55, 1.0)), rin=float(rng.uniform(1.001, 1.05)), rout=1.0)


def generate_dataset(n, w, h, seed, steps, per_batch=256, precision="f32"):
    """n steady states of random porous channels from the batch solver (fixed `steps`)."""
    rng = np.random.default_rng(seed)
    samples = []
    while len(samples) < n:
        k = min(per_batch, n - len(samples))
        chans = [random_channel(rng, w, h) for _ in range(k)]
        b = Batch([{"mask": c["mask"], "relaxation_time": c["tau"], "inlet_density": c["rin"],
                    "outlet_density": c["rout"]} for c in chans], precision=precision)
        b.set_tile(32, 4 + 256 * 8, 16)
        b.run(steps, mode="persistent_graph")
        for i, c in enumerate(chans):
            c["rho"], c["jx"], c["jy"] = b.result(i, 0), b.result(i, 1), b.result(i, 2)
            samples.append(c)
        b.close()
    return samples


def train(model: NeuralOperator, samples, epochs=10, batch=16, lr=2e-3, log=None):
    torch = model.torch
    n = len(samples)
    h, w = samples[0]["mask"].shape
    masks_np = np.stack([s["mask"] for s in samples])
    masks = torch.from_numpy(masks_np).cuda()
    fl = masks_np.reshape(n, -1) == 0
    drho = np.stack([s["rho"] - 1.0 for s in samples]).reshape(n, -1)
    jx = np.stack([s["jx"] for s in samples]).reshape(n, -1)
    jy = np.stack([s["jy"] for s in samples]).reshape(n, -1)
    model.scale = np.array([1.0 / drho[fl].std(), 1.0 / np.concatenate([jx[fl], jy[fl]]).std(),
                            1.0 / np.concatenate([jx[fl], jy[fl]]).std()], dtype=np.float32)
    tgt = np.stack([drho * model.scale[0], jx * model.scale[1], jy * model.scale[2]], axis=-1).astype(np.float32)
    targets = torch.from_numpy(tgt.reshape(n, h, w, 3)).cuda()
    rin = np.array([s["rin"] for s in samples], dtype=np.float32)
    rout = np.array([s["rout"] for s in samples], dtype=np.float32)
    tau = np.array([s["tau"] for s in samples], dtype=np.float32)
    loss_d = torch.zeros(1, dtype=torch.float32, device="cuda")
    grad = torch.empty((batch, h, w, 3), dtype=torch.bfloat16, device="cuda")
    rng = np.random.default_rng(1)
    hist = []
    steps_total = epochs * (n // batch)
    t0 = time.perf_counter()
    for ep in range(epochs):
        order = rng.permutation(n)
        tot = 0.0
        for it in range(n // batch):
            sel = order[it * batch:(it + 1) * batch]
            idx = torch.from_numpy(sel).cuda()
            m = masks.index_select(0, idx).contiguous()
            x = model.assemble(m, rin[order[it * batch:(it + 1) * batch]], rout[order[it * batch:(it + 1) * batch]],
                               tau[order[it * batch:(it + 1) * batch]])
            pred = model.forward(x, batch, h, w)
            t = targets.index_select(0, idx).contiguous()
            loss_d.zero_()
            count = float(fl[sel].sum() * 3)
            _ok(model.lib.plbm_nn_mse(pred.data_ptr(), t.data_ptr(), m.data_ptr(), grad.data_ptr(), loss_d.data_ptr(),
                                      batch * h * w, 3, 1.0 / count, None))
            model.zero_grad()
            model.backward(grad)
            step = ep * (n // batch) + it
            model.adam(lr=lr * 0.5 * (1 + np.cos(np.pi * step / steps_total)))
            tot += float(loss_d.item())
        hist.append(tot / (n // batch))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.5f}")
    return {"loss_history": hist, "seconds": time.perf_counter() - t0}


def solve(chan, precision="f64_q60", init=None, target=1e-6, k=100, max_steps=400000):
    """Runs the plain solver to `target`; init = (rho, jx, jy) to start from their equilibrium."""
    h, w = chan["mask"].shape
    props = Properties("nptl", "stream", False, 1024, 10 ** 9, 10 ** 9, "Hagen-Poiseuille", h, w, 0.0, 0.0,
                       chan["rin"], 0.0, 0.0, chan["rout"], chan["tau"])
    hd = create_handler(props, precision=precision, mask=chan["mask"])
    lib = load_library()
    if init is not None:
        rho, jx, jy = (np.ascontiguousarray(a, dtype=np.float64) for a in init)
        rc = lib.plbm_set_equilibrium(hd._h, rho.ctypes.data, jx.ctypes.data, jy.ctypes.data)
        if rc != 0:
            raise RuntimeError("set_equilibrium failed")
    t0 = time.perf_counter()
    steps, r = hd.run_to_residual(target, k, 2 * k)      # first residual: compares inits
    first = r
    if r >= target:
        more, r = hd.run_to_residual(target, k, max_steps)
        steps += more
    dt = time.perf_counter() - t0
    hd.close()
    return {"steps": steps, "seconds": dt, "first_residual": first, "residual": r}


def study(n_train=2000, n_test=200, size=(256, 256), large=(1024, 256), steps=8000, large_steps=24000, epochs=12,
          seed=7, log=None):
    """Trains on solver-generated steady states and measures steps / wall time to residual 1e-6
    from rest versus from the prediction on held-out geometries (half at `size`, half at `large`)."""
    t0 = time.perf_counter()
    w, h = size
    data = generate_dataset(n_train, w, h, seed, steps)
    t_data = time.perf_counter() - t0
    model = NeuralOperator(seed)
    hist = train(model, data, epochs=epochs, log=log)
    rng = np.random.default_rng(seed + 99)
    rows = []
    for i in range(n_test):
        ww, hh = size if i % 2 == 0 else large
        chan = random_channel(rng, ww, hh)
        cold = solve(chan)
        ti = time.perf_counter()
        pred = model.predict(chan["mask"], chan["rin"], chan["rout"], chan["tau"])
        infer = time.perf_counter() - ti
        warm = solve(chan, init=pred)
        used = warm if warm["first_residual"] <= cold["first_residual"] else None
        rows.append({"size": f"{ww}x{hh}", "cold_steps": cold["steps"], "cold_s": cold["seconds"],
                     "warm_steps": warm["steps"], "warm_s": warm["seconds"] + infer, "fallback": used is None,
                     "infer_s": infer})
    def agg(sel):
        cs = np.array([r["cold_steps"] for r in sel], dtype=float)
        ws = np.array([r["cold_steps"] if r["fallback"] else r["warm_steps"] for r in sel], dtype=float)
        ct = np.array([r["cold_s"] for r in sel])
        wt = np.array([r["cold_s"] + r["warm_s"] if r["fallback"] else r["warm_s"] for r in sel])
        return {"n": len(sel), "median_cold_steps": float(np.median(cs)), "median_warm_steps": float(np.median(ws)),
                "steps_reduction_total": float(cs.sum() / ws.sum()), "time_reduction_total": float(ct.sum() / wt.sum()),
                "fallbacks": int(sum(r["fallback"] for r in sel))}
    return {"train": {"samples": n_train, "size": f"{w}x{h}", "solver_steps": steps, "dataset_s": round(t_data, 1),
                      "epochs": epochs, "train_s": round(hist["seconds"], 1),
                      "loss_first": hist["loss_history"][0], "loss_last": hist["loss_history"][-1]},
            "held_out": {"all": agg(rows), f"{w}x{h}": agg([r for r in rows if r["size"] == f"{w}x{h}"]),
                         f"{large[0]}x{large[1]}": agg([r for r in rows if r["size"] == f"{large[0]}x{large[1]}"])}}

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
    head     32->3

Inputs are the solid mask and three per-sample scalars (a constant 1, which marks the domain
edges through the zero padding, the relaxation time and the log of the Stokes velocity scale).
Targets are made independent of the pressure drop, viscosity and channel length: with
G = (rho_in - rho_out)/(W + 1) the mean density gradient and nu = (tau - 1/2)/3,

    t_rho = (rho - rho_lin(x)) / G          rho_lin the linear profile between the ghost columns
    t_j   = j * nu / (c_s^2 * G)            the Darcy-scaled momentum

each divided by its training-set standard deviation.  At inference a 1-D series-resistance pass
(`series_profile`) rescales the columns so the column mass fluxes agree, which sets the
channel-scale density profile that a finite receptive field cannot see.

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
        "plbm_nn_conv_dgrad_pre": [vp, vp, vp, vp, i, i, i, i, i, vp],
        "plbm_nn_flip_layers": [vp, vp, vp, i, i, vp],
        "plbm_nn_conv_wgrad": [vp, vp, vp, vp, i, i, i, i, i, vp],
        "plbm_nn_relu_bwd": [vp, vp, ll, vp],
        "plbm_nn_relu_bwd_bias": [vp, vp, vp, ll, i, vp],
        "plbm_nn_pool2": [vp, vp, i, i, i, i, vp],
        "plbm_nn_pool2_bwd": [vp, vp, i, i, i, i, vp],
        "plbm_nn_up2": [vp, vp, i, i, i, i, vp],
        "plbm_nn_up2_bwd": [vp, vp, i, i, i, i, vp],
        "plbm_nn_add": [vp, vp, vp, ll, vp],
        "plbm_nn_mse": [vp, vp, vp, vp, vp, ll, i, f, vp],
        "plbm_nn_adam": [vp, vp, vp, vp, vp, ll, f, f, f, f, i, vp],
        "plbm_nn_adam_dev": [vp, vp, vp, vp, vp, ll, vp, f, f, f, vp, vp],
        "plbm_nn_assemble": [vp, vp, vp, i, i, i, i, vp],
    }
    for name, args in sig.items():
        getattr(lib, name).argtypes = args
        getattr(lib, name).restype = ctypes.c_int
    return lib


CS2 = 1.0 / 3.0
STOKES_LENGTH = 8.0


def channel_scales(w, rin, rout, tau):
    """Mean density gradient G over the W + 1 links between the inlet and outlet ghost columns,
    and the kinematic viscosity nu = (tau - 1/2)/3."""
    return (rin - rout) / (w + 1), (tau - 0.5) / 3.0


def linear_profile(w, rin, rout):
    """Density of the straight profile at inner columns x = 0..W-1 (ghost x = -1 at rin, x = W at rout)."""
    return rin - (rin - rout) * (np.arange(w) + 1.0) / (w + 1)


def features(w, rin, rout, tau):
    g, nu = channel_scales(w, rin, rout, tau)
    u = CS2 * abs(g) * STOKES_LENGTH ** 2 / nu
    return [1.0, (tau - 0.775) * 4.0, float(np.log10(max(u, 1e-12))) + 2.25]


def series_profile(jx_pred, mask, w, rin, rout, sigma):
    """Per-column gradient scale s(x) (mean 1) from the predicted column fluxes Q(x): in a steady
    channel every column carries the same flux, so with local resistance 1/Q the gradient is
    proportional to 1/Q (Q smoothed over `sigma` columns).  Returns s and the corrected profile
    rho_b(x), or None when the prediction has no positive net flux everywhere."""
    q = np.where(mask == 0, jx_pred, 0.0).sum(axis=0)
    if sigma > 0:
        r = int(3 * sigma)
        k = np.exp(-0.5 * (np.arange(-r, r + 1) / sigma) ** 2)
        q = np.convolve(np.pad(q, r, mode="reflect"), k / k.sum(), mode="valid")
    if np.any(q <= 0):
        return None
    s = (1.0 / q) / np.mean(1.0 / q)
    links = np.concatenate([[s[0]], 0.5 * (s[1:] + s[:-1]), [s[-1]]])      # W + 1 link gradients
    drop = np.cumsum(links) / links.sum() * (rin - rout)
    return s, rin - drop[:-1]


def _ok(rc):
    if rc != 0:
        raise RuntimeError(f"plbm_nn call failed ({rc})")


PARAM_ALIGN = 128   # elements: every parameter segment starts 256-byte (FP32) / 128-byte (BF16) aligned


class ConvLayer:
    """One 3x3 convolution's parameters: views into the operator's flat buffers (`Params`)."""

    def __init__(self, cin, cout, relu, rng, params):
        self.cin, self.cout, self.relu = cin, cout, relu
        w = (rng.standard_normal((cout, 9 * cin)) * np.sqrt(2.0 / (9 * cin))).astype(np.float32)
        # FP32 master, BF16 copy and the BF16 copy re-laid out for the input gradient (wbt)
        self.w_off = params.off
        self.w, self.gw, self.m0, self.v0, self.wb, self.wbt = params.segment((cout, 9 * cin))
        self.b, self.gb, self.m1, self.v1, _, _ = params.segment((cout,))
        self.w.copy_(params.torch.from_numpy(w))
        self.wb.copy_(self.w.to(params.torch.bfloat16))
        self.m, self.v = [self.m0, self.m1], [self.v0, self.v1]


class Params:
    """Flat FP32 buffers for the weights and biases, their gradients and Adam's two moments, a BF16
    copy of the weights and that copy re-laid out for the input gradients: zeroing the gradients,
    the Adam update and the re-layout are one launch each."""

    def __init__(self, sizes, torch):
        self.torch = torch
        self.total = sum(-(-int(np.prod(s)) // PARAM_ALIGN) * PARAM_ALIGN for s in sizes)
        f32 = dict(dtype=torch.float32, device="cuda")
        self.w, self.g, self.m, self.v = (torch.zeros(self.total, **f32) for _ in range(4))
        self.wb = torch.zeros(self.total, dtype=torch.bfloat16, device="cuda")
        self.wbt = torch.zeros(self.total, dtype=torch.bfloat16, device="cuda")
        self.off = 0

    def segment(self, shape):
        n = int(np.prod(shape))
        a, self.off = self.off, self.off + -(-n // PARAM_ALIGN) * PARAM_ALIGN
        return tuple(t[a:a + n].view(shape) for t in (self.w, self.g, self.m, self.v, self.wb, self.wbt))


class NeuralOperator:
    """U-Net-style operator; forward/backward/Adam all run in libplbm's kernels."""

    def __init__(self, seed: int = 0):
        import torch
        self.torch = torch
        self.lib = _fns()
        rng = np.random.default_rng(seed)
        shapes = []
        for ci, co in ENC + DEC + [HEAD]:
            shapes += [(co, 9 * ci), (co,)]
        self.params = Params(shapes, torch)
        self.enc = [ConvLayer(ci, co, True, rng, self.params) for ci, co in ENC]
        self.dec = [ConvLayer(ci, co, True, rng, self.params) for ci, co in DEC]
        self.head = ConvLayer(HEAD[0], HEAD[1], False, rng, self.params)
        self.layers = self.enc + self.dec + [self.head]
        # (weight offset, Cin, Cout) of every layer for the one-launch re-layout of the weights
        self._segs = torch.tensor([[l.w_off, l.cin, l.cout] for l in self.layers], dtype=torch.int32, device="cuda")
        self._max_elems = max(9 * l.cin * l.cout for l in self.layers)
        self.norm = np.array([1.0, 1.0])          # std of t_rho and of t_j over the training set
        self.step_count = 0
        self._s = None

    def save(self, path):
        """Writes the FP32 master weights, biases and target scales to an .npz file."""
        arrs = {"norm": self.norm}
        for i, layer in enumerate(self.layers):
            arrs[f"w{i}"] = layer.w.cpu().numpy()
            arrs[f"b{i}"] = layer.b.cpu().numpy()
        np.savez(path, **arrs)

    def load(self, path):
        z = np.load(path)
        self.norm = z["norm"]
        for i, layer in enumerate(self.layers):
            w = self.torch.from_numpy(z[f"w{i}"].astype(np.float32))
            if tuple(w.shape) != tuple(layer.w.shape):
                raise ValueError(f"layer {i}: shape {tuple(w.shape)} != {tuple(layer.w.shape)}")
            layer.w.copy_(w)
            layer.wb.copy_(layer.w.to(self.torch.bfloat16))
            layer.b.copy_(self.torch.from_numpy(z[f"b{i}"].astype(np.float32)))
        return self

    def _stream(self):
        """The handle of torch's current CUDA stream (None for the legacy default stream): every
        kernel of a call goes there, so the calls order with torch's work and can be captured."""
        return self.torch.cuda.current_stream().cuda_stream or None

    def _buf(self, n, h, w, c):
        return self.torch.empty((n, h, w, c), dtype=self.torch.bfloat16, device="cuda")

    def _conv(self, layer, x, n, h, w):
        y = self._buf(n, h, w, layer.cout)
        _ok(self.lib.plbm_nn_conv_fwd(x.data_ptr(), layer.wb.data_ptr(), layer.b.data_ptr(), y.data_ptr(), n, h, w,
                                      layer.cin, layer.cout, int(layer.relu), self._s))
        return y

    def forward(self, x, n, h, w):
        """x: [n,h,w,4] bf16 input; returns the [n,h,w,3] prediction and keeps activations for backward."""
        self._s = self._stream()
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
                _ok(self.lib.plbm_nn_pool2(b.data_ptr(), p.data_ptr(), n, hh, ww, b.shape[-1], self._s))
                acts[f"p{lvl}"] = p
                cur, hh, ww = p, hh // 2, ww // 2
            else:
                cur = b
        for k, lvl in enumerate((3, 2, 1, 0)):
            sh, sw = skips[lvl][1], skips[lvl][2]
            u = self._buf(n, sh, sw, cur.shape[-1])
            _ok(self.lib.plbm_nn_up2(cur.data_ptr(), u.data_ptr(), n, sh, sw, cur.shape[-1], self._s))
            a = self._conv(self.dec[2 * k], u, n, sh, sw)
            s = self._buf(n, sh, sw, a.shape[-1])
            _ok(self.lib.plbm_nn_add(a.data_ptr(), skips[lvl][0].data_ptr(), s.data_ptr(), s.numel(), self._s))
            b = self._conv(self.dec[2 * k + 1], s, n, sh, sw)
            acts[f"u{lvl}"], acts[f"d{lvl}a"], acts[f"s{lvl}"], acts[f"d{lvl}b"] = u, a, s, b
            cur = b
        out = self._conv(self.head, cur, n, h, w)
        acts["out"] = out
        self.acts, self.shape = acts, (n, h, w)
        return out

    def _conv_bwd(self, layer, x, y, gy, n, h, w, need_gx=True):
        gb = layer.gb.data_ptr()
        if layer.relu:   # the ReLU backward and the bias gradient in one pass over the gradient
            _ok(self.lib.plbm_nn_relu_bwd_bias(y.data_ptr(), gy.data_ptr(), gb, n * h * w, layer.cout, self._s))
            gb = None
        _ok(self.lib.plbm_nn_conv_wgrad(x.data_ptr(), gy.data_ptr(), layer.gw.data_ptr(), gb, n, h, w, layer.cin,
                                        layer.cout, self._s))
        if not need_gx:
            return None
        gx = self._buf(n, h, w, layer.cin)
        _ok(self.lib.plbm_nn_conv_dgrad_pre(gy.data_ptr(), layer.wb.data_ptr(), layer.wbt.data_ptr(), gx.data_ptr(),
                                            n, h, w, layer.cin, layer.cout, self._s))
        return gx

    def backward(self, gout):
        self._s = self._stream()
        p = self.params
        _ok(self.lib.plbm_nn_flip_layers(p.wb.data_ptr(), p.wbt.data_ptr(), self._segs.data_ptr(), len(self.layers),
                                         self._max_elems, self._s))
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
            _ok(self.lib.plbm_nn_up2_bwd(gu.data_ptr(), g.data_ptr(), n, ch, cw, gu.shape[-1], self._s))
        for lvl in (4, 3, 2, 1, 0):
            hh, ww = sizes[lvl]
            if lvl < 4:
                # gradient of e{lvl}b: skip gradient + pooled path gradient
                gp = self._buf(n, hh, ww, g.shape[-1])
                _ok(self.lib.plbm_nn_pool2_bwd(g.data_ptr(), gp.data_ptr(), n, hh, ww, g.shape[-1], self._s))
                gb_ = self._buf(n, hh, ww, g.shape[-1])
                _ok(self.lib.plbm_nn_add(gp.data_ptr(), gskip[lvl].data_ptr(), gb_.data_ptr(), gb_.numel(), self._s))
                g = gb_
            xin = a["in"] if lvl == 0 else a[f"p{lvl - 1}"]
            ga = self._conv_bwd(self.enc[2 * lvl + 1], a[f"e{lvl}a"], a[f"e{lvl}b"], g, n, hh, ww)
            g = self._conv_bwd(self.enc[2 * lvl], xin, a[f"e{lvl}a"], ga, n, hh, ww, need_gx=lvl > 0)

    def zero_grad(self):
        self.params.g.zero_()

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        """One Adam update of every weight and bias (one launch over the flat buffers; the padding
        between segments has zero gradients and stays zero)."""
        self.step_count += 1
        self._s = self._stream()
        p = self.params
        _ok(self.lib.plbm_nn_adam(p.w.data_ptr(), p.g.data_ptr(), p.m.data_ptr(), p.v.data_ptr(), p.wb.data_ptr(),
                                  p.total, lr, b1, b2, eps, self.step_count, self._s))

    def adam_dev(self, lr, state, b1=0.9, b2=0.999, eps=1e-8):
        """Adam with the learning rate lr ([1] FP32 device tensor) and the step count state ([2]
        int32 device tensor: the count, and a block counter left at zero) read on the device, so
        that a captured launch advances the count on each replay."""
        self._s = self._stream()
        p = self.params
        _ok(self.lib.plbm_nn_adam_dev(p.w.data_ptr(), p.g.data_ptr(), p.m.data_ptr(), p.v.data_ptr(), p.wb.data_ptr(),
                                      p.total, lr.data_ptr(), b1, b2, eps, state.data_ptr(), self._s))

    def capture_train_step(self, x, gout, n, h, w, b1=0.9, b2=0.999, eps=1e-8):
        """One training step on fixed buffers -- forward on x, zeroed gradients, backward of the
        output gradient gout, Adam -- captured as a CUDA graph.  Returns step(lr), which sets the
        learning rate and replays the graph on torch's current stream; new data goes into x and
        gout in place between replays.  The activations live in the graph's memory pool."""
        torch = self.torch
        lr_d = torch.zeros(1, dtype=torch.float32, device="cuda")
        state = torch.tensor([self.step_count, 0], dtype=torch.int32, device="cuda")
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):          # first calls: kernel attributes, scratch sizes
            self.forward(x, n, h, w)
            self.backward(gout)
            self.zero_grad()
        torch.cuda.current_stream().wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            self.forward(x, n, h, w)
            self.zero_grad()
            self.backward(gout)
            self.adam_dev(lr_d, state, b1, b2, eps)

        def step(lr):
            lr_d.fill_(float(lr))
            graph.replay()
            self.step_count += 1

        step.graph, step.state, step.out = graph, state, self.acts["out"]
        return step

    def capture_forward(self, x, n, h, w):
        """The forward pass on the fixed input buffer x captured as a CUDA graph: returns
        (run, out), run() replaying it on torch's current stream into the prediction buffer out."""
        torch = self.torch
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.forward(x, n, h, w)
        torch.cuda.current_stream().wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            out = self.forward(x, n, h, w)
        return graph.replay, out

    def assemble(self, masks, feats):
        """masks: [n,h,w] int8 device tensor; feats: n rows of `features` -> [n,h,w,4] bf16 input."""
        torch = self.torch
        n, h, w = masks.shape
        self._s = self._stream()
        x = self._buf(n, h, w, C_IN)
        f = torch.tensor(np.asarray(feats, dtype=np.float32).reshape(n, 3), device="cuda")
        _ok(self.lib.plbm_nn_assemble(masks.data_ptr(), f.data_ptr(), x.data_ptr(), n, h, w, C_IN, self._s))
        return x

    def predict(self, mask: np.ndarray, rin: float, rout: float, tau: float, sigma: float = 16.0):
        """Predicted steady (rho, jx, jy) fields (float64, H*W) for one channel; sigma < 0 skips
        the series-resistance pass."""
        torch = self.torch
        h, w = mask.shape
        g, nu = channel_scales(w, rin, rout, tau)
        if g == 0.0:
            return np.full(h * w, rout), np.zeros(h * w), np.zeros(h * w)
        m = torch.from_numpy(np.ascontiguousarray(mask, dtype=np.int8)[None]).cuda()
        x = self.assemble(m, [features(w, rin, rout, tau)])
        out = self.forward(x, 1, h, w).float().cpu().numpy().astype(np.float64).reshape(h, w, 3)
        t_rho = out[..., 0] * self.norm[0]
        jscale = self.norm[1] * CS2 * g / nu
        jx, jy = out[..., 1] * jscale, out[..., 2] * jscale
        rho = linear_profile(w, rin, rout)[None, :] + g * t_rho
        if sigma >= 0:
            sp = series_profile(jx, mask, w, rin, rout, sigma)
            if sp is not None:
                s, rho_b = sp
                rho = rho_b[None, :] + g * s[None, :] * t_rho
                jx, jy = jx * s[None, :], jy * s[None, :]
        return rho.reshape(-1), jx.reshape(-1), jy.reshape(-1)


def random_channel(rng, w, h):
    return dict(mask=porous_disks(w, h, int(rng.integers(1 << 62)), float(rng.uniform(0.6, 0.8))),
                tau=float(rng.uniform(0.55, 1.0)), rin=float(rng.uniform(1.001, 1.05)), rout=1.0)


def converged_fields(mask, rho, jx, jy):
    """False for a diverged run: BGK at relaxation times near 1/2 with a large inlet density can
    blow up, and the NaN guard then leaves zeros (or a non-finite value) in the results."""
    fl = mask.reshape(-1) == 0
    return bool(np.all(np.isfinite(rho)) and np.all(np.isfinite(jx)) and np.all(np.isfinite(jy))
                and np.all(rho[fl] > 0.5))


def generate_dataset(n, w, h, seed, steps, per_batch=256, precision="f32", stats=None):
    """n steady states of random porous channels from the batch solver (fixed `steps`); channels
    whose run diverged are drawn again (their count goes to stats["diverged"])."""
    rng = np.random.default_rng(seed)
    samples = []
    diverged = 0
    while len(samples) < n:
        k = min(per_batch, n - len(samples))
        chans = [random_channel(rng, w, h) for _ in range(k)]
        b = Batch([{"mask": c["mask"], "relaxation_time": c["tau"], "inlet_density": c["rin"],
                    "outlet_density": c["rout"]} for c in chans], precision=precision)
        b.set_tile(32, 4 + 256 * 8, 16)
        b.run(steps, mode="persistent_graph")
        for i, c in enumerate(chans):
            c["rho"], c["jx"], c["jy"] = b.result(i, 0), b.result(i, 1), b.result(i, 2)
            if converged_fields(c["mask"], c["rho"], c["jx"], c["jy"]):
                samples.append(c)
            else:
                diverged += 1
        b.close()
    if stats is not None:
        stats["diverged"] = diverged
    return samples


def train(model: NeuralOperator, samples, epochs=10, batch=16, lr=2e-3, flip=True, log=None):
    """Adam with a cosine learning rate over `epochs`; flip=True adds every sample mirrored about
    the channel axis (y -> H-1-y, jy -> -jy), a symmetry of the walled channel."""
    torch = model.torch
    n = len(samples)
    h, w = samples[0]["mask"].shape
    masks_np = np.stack([s["mask"] for s in samples])
    t_rho = np.empty((n, h, w))
    t_j = np.empty((n, h, w, 2))
    feats = np.empty((n, 3), dtype=np.float32)
    for i, s in enumerate(samples):
        g, nu = channel_scales(w, s["rin"], s["rout"], s["tau"])
        t_rho[i] = (s["rho"].reshape(h, w) - linear_profile(w, s["rin"], s["rout"])[None, :]) / g
        t_j[i, ..., 0] = s["jx"].reshape(h, w) * nu / (CS2 * g)
        t_j[i, ..., 1] = s["jy"].reshape(h, w) * nu / (CS2 * g)
        feats[i] = features(w, s["rin"], s["rout"], s["tau"])
    if flip:
        masks_np = np.concatenate([masks_np, masks_np[:, ::-1]])
        t_rho = np.concatenate([t_rho, t_rho[:, ::-1]])
        t_j = np.concatenate([t_j, t_j[:, ::-1] * np.array([1.0, -1.0])])
        feats = np.concatenate([feats, feats])
        n *= 2
    masks = torch.from_numpy(np.ascontiguousarray(masks_np)).cuda()
    fl = masks_np.reshape(n, -1) == 0
    fl3 = fl.reshape(n, h, w)
    model.norm = np.array([t_rho[fl3].std(), t_j[fl3].std()])
    tgt = np.concatenate([t_rho[..., None] / model.norm[0], t_j / model.norm[1]], axis=-1).astype(np.float32)
    targets = torch.from_numpy(tgt).cuda()
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
            x = model.assemble(m, feats[sel])
            pred = model.forward(x, batch, h, w)
            t = targets.index_select(0, idx).contiguous()
            loss_d.zero_()
            count = float(fl[sel].sum() * 3)
            _ok(model.lib.plbm_nn_mse(pred.data_ptr(), t.data_ptr(), m.data_ptr(), grad.data_ptr(), loss_d.data_ptr(),
                                      batch * h * w, 3, 1.0 / count, model._stream()))
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
    """Runs the plain solver to `target`; init = (rho, jx, jy) to start from their equilibrium.
    The first residual is taken after 2k steps (the fallback comparison); wall time includes
    loading the initial state."""
    h, w = chan["mask"].shape
    props = Properties("nptl", "stream", False, 1024, 10 ** 9, 10 ** 9, "Hagen-Poiseuille", h, w, 0.0, 0.0,
                       chan["rin"], 0.0, 0.0, chan["rout"], chan["tau"])
    hd = create_handler(props, precision=precision, mask=chan["mask"])
    t0 = time.perf_counter()
    if init is not None:
        hd.set_equilibrium(*init)
    steps, r = hd.run_to_residual(target, k, 2 * k)
    first, first_s, first_steps = r, time.perf_counter() - t0, steps
    if r >= target:
        more, r = hd.run_to_residual(target, k, max_steps)
        steps += more
    dt = time.perf_counter() - t0
    jx, jy = hd.get_x_velocities(), hd.get_y_velocities()
    hd.close()
    return {"steps": steps, "seconds": dt, "first_residual": first, "first_seconds": first_s,
            "first_steps": first_steps, "residual": r, "j": (jx, jy)}


def state_difference(mask, a, b):
    """Relative L2 distance of two momentum fields over the fluid nodes."""
    fl = mask.reshape(-1) == 0
    num = np.sqrt(np.sum((a[0] - b[0])[fl] ** 2) + np.sum((a[1] - b[1])[fl] ** 2))
    den = np.sqrt(np.sum(b[0][fl] ** 2) + np.sum(b[1][fl] ** 2))
    return float(num / den) if den > 0 else float(num)


def rest_ramp_init(chan):
    """Initial state without the network: the straight density profile and zero momentum."""
    h, w = chan["mask"].shape
    return np.tile(linear_profile(w, chan["rin"], chan["rout"]), h), np.zeros(h * w), np.zeros(h * w)


def evaluate(model, chans, sigma=16.0, ablation=True, log=None):
    """Rest start vs warm start (with fallback) on each channel; time to residual 1e-6.  A channel
    whose rest start diverges is reported with cold_steps None (excluded from the comparison); a
    warm start that diverges counts as a fallback."""
    rows = []
    for chan in chans:
        h, w = chan["mask"].shape
        row = {"size": f"{w}x{h}", "tau": chan["tau"], "rin": chan["rin"]}
        try:
            cold = solve(chan)
        except Exception:
            row.update(cold_steps=None, fallback=None)
            rows.append(row)
            if log:
                log(row)
            continue
        t0 = time.perf_counter()
        pred = model.predict(chan["mask"], chan["rin"], chan["rout"], chan["tau"], sigma=sigma)
        infer = time.perf_counter() - t0
        try:
            warm = solve(chan, init=pred)
            fb = warm["first_residual"] > cold["first_residual"]
        except Exception:
            warm, fb = None, True
        if fb:   # the warm start's probe phase was spent, then the rest start runs in full
            probe_steps = warm["first_steps"] if warm else 0
            probe_s = warm["first_seconds"] if warm else 0.0
            w_steps, w_s = probe_steps + cold["steps"], infer + probe_s + cold["seconds"]
        else:    # the rest start's probe phase was spent to decide
            w_steps = warm["steps"] + cold["first_steps"]
            w_s = infer + warm["seconds"] + cold["first_seconds"]
        row.update(cold_steps=cold["steps"], cold_s=cold["seconds"], warm_steps=w_steps, warm_s=w_s, fallback=bool(fb),
                   infer_s=infer, cold_r0=cold["first_residual"], warm_r0=warm["first_residual"] if warm else None,
                   state_diff=state_difference(chan["mask"], warm["j"], cold["j"]) if warm else None)
        if ablation:   # the same warm start from the straight profile alone (no network)
            try:
                ramp = solve(chan, init=rest_ramp_init(chan))
                row.update(ramp_steps=ramp["steps"], ramp_s=ramp["seconds"])
            except Exception:
                row.update(ramp_steps=None, ramp_s=None)
        rows.append(row)
        if log:
            log(row)
    return rows


def aggregate(rows):
    diverged = sum(r["cold_steps"] is None for r in rows)
    rows = [r for r in rows if r["cold_steps"] is not None]
    if not rows:
        return {"n": 0, "diverged": diverged}
    cs = np.array([r["cold_steps"] for r in rows], dtype=float)
    ws = np.array([r["warm_steps"] for r in rows], dtype=float)
    ct = np.array([r["cold_s"] for r in rows])
    wt = np.array([r["warm_s"] for r in rows])
    return {"n": len(rows), "median_cold_steps": float(np.median(cs)), "median_warm_steps": float(np.median(ws)),
            "steps_reduction_total": float(cs.sum() / ws.sum()), "time_reduction_total": float(ct.sum() / wt.sum()),
            "time_reduction_median": float(np.median(ct / wt)), "cold_s_total": float(ct.sum()),
            "warm_s_total": float(wt.sum()), "fallbacks": int(sum(r["fallback"] for r in rows)),
            "ramp_only_steps_reduction_total": (float(cs.sum() / sum(r["ramp_steps"] for r in rows))
                                                if all(r.get("ramp_steps") for r in rows) else None),
            "max_state_diff": max((r["state_diff"] for r in rows if r["state_diff"] is not None), default=None),
            "diverged": diverged}


def study(n_train=2000, n_test=200, size=(256, 256), large=(1024, 256), steps=20000, epochs=16, seed=7,
          sigma=16.0, save=None, log=None):
    """Trains on solver-generated steady states and measures steps / wall time to residual 1e-6
    from rest versus from the prediction on held-out geometries (half at `size`, half at `large`)."""
    t0 = time.perf_counter()
    w, h = size
    gen = {}
    data = generate_dataset(n_train, w, h, seed, steps, stats=gen)
    t_data = time.perf_counter() - t0
    model = NeuralOperator(seed)
    hist = train(model, data, epochs=epochs, log=log)
    if save:
        model.save(save)
    del data
    rng = np.random.default_rng(seed + 99)
    chans = [random_channel(rng, *(size if i % 2 == 0 else large)) for i in range(n_test)]
    rows = evaluate(model, chans, sigma=sigma, log=log)
    out = {"train": {"samples": n_train, "size": f"{w}x{h}", "solver_steps": steps, "dataset_s": round(t_data, 1),
                     "diverged_redrawn": gen["diverged"],
                     "epochs": epochs, "train_s": round(hist["seconds"], 1),
                     "loss_first": hist["loss_history"][0], "loss_last": hist["loss_history"][-1]},
           "held_out": {"all": aggregate(rows)}}
    for sz in (size, large):
        key = f"{sz[0]}x{sz[1]}"
        out["held_out"][key] = aggregate([r for r in rows if r["size"] == key])
    return out

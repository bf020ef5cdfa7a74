"""The neural operator's tensor-core kernels (plbm_nn_* in include/plbm_c.h) against the float64
CPU reference (oracle/nn_ref.py) on bfloat16-rounded operands.  Tolerance: outputs are rounded to
bfloat16 (relative 2^-8), so |gpu - ref| <= 1e-2 * max|ref| + 1e-3; weight gradients accumulate in
FP32 and must agree to 1e-3 relative."""
import ctypes

import numpy as np
import pytest

from oracle import nn_ref

pytestmark = pytest.mark.gpu


def _lib(plbm):
    lib = plbm.load_library()
    vp, i = ctypes.c_void_p, ctypes.c_int
    lib.plbm_nn_conv_fwd.argtypes = [vp, vp, vp, vp, i, i, i, i, i, i, vp]
    lib.plbm_nn_conv_dgrad.argtypes = [vp, vp, vp, i, i, i, i, i, vp]
    lib.plbm_nn_conv_wgrad.argtypes = [vp, vp, vp, vp, i, i, i, i, i, vp]
    lib.plbm_nn_pool2.argtypes = [vp, vp, i, i, i, i, vp]
    lib.plbm_nn_up2.argtypes = [vp, vp, i, i, i, i, vp]
    lib.plbm_nn_pool2_bwd.argtypes = [vp, vp, i, i, i, i, vp]
    lib.plbm_nn_up2_bwd.argtypes = [vp, vp, i, i, i, i, vp]
    return lib


def _bf(t):
    import torch
    return torch.tensor(t, dtype=torch.float32).to(torch.bfloat16).cuda()


def _np(t):
    return t.float().cpu().numpy().astype(np.float64)


def _close(got, ref, rel=1e-2):
    assert np.max(np.abs(got - ref)) <= rel * np.max(np.abs(ref)) + 1e-3


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 16, 24, 4, 32), (1, 32, 32, 32, 64), (2, 8, 16, 96, 128),
                                           (1, 16, 16, 64, 3)])
def test_conv_forward_and_gradients(plbm, n, h, w, cin, cout):
    import torch
    lib = _lib(plbm)
    rng = np.random.default_rng(n * 1000 + cin)
    x = nn_ref.bf16_round(rng.standard_normal((n, h, w, cin)))
    wt = nn_ref.bf16_round(rng.standard_normal((cout, 9 * cin)) / np.sqrt(9 * cin))
    b = rng.standard_normal(cout).astype(np.float32)
    g = nn_ref.bf16_round(rng.standard_normal((n, h, w, cout)))
    xd, wd, gd = _bf(x), _bf(wt), _bf(g)
    bd = torch.tensor(b).cuda()
    y = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    gx = torch.empty((n, h, w, cin), dtype=torch.bfloat16, device="cuda")
    gw = torch.zeros((cout, 9 * cin), dtype=torch.float32, device="cuda")
    gb = torch.zeros(cout, dtype=torch.float32, device="cuda")
    for relu in (0, 1):
        assert lib.plbm_nn_conv_fwd(xd.data_ptr(), wd.data_ptr(), bd.data_ptr(), y.data_ptr(), n, h, w, cin, cout,
                                    relu, None) == 0
        torch.cuda.synchronize()
        _close(_np(y), nn_ref.conv_fwd(x, wt, b.astype(np.float64), bool(relu)))
    assert lib.plbm_nn_conv_dgrad(gd.data_ptr(), wd.data_ptr(), gx.data_ptr(), n, h, w, cin, cout, None) == 0
    assert lib.plbm_nn_conv_wgrad(xd.data_ptr(), gd.data_ptr(), gw.data_ptr(), gb.data_ptr(), n, h, w, cin, cout,
                                  None) == 0
    torch.cuda.synchronize()
    _close(_np(gx), nn_ref.conv_dgrad(g, wt, cin))
    rgw, rgb = nn_ref.conv_wgrad(x, g)
    assert np.max(np.abs(_np(gw) - rgw)) <= 1e-3 * np.max(np.abs(rgw))
    assert np.max(np.abs(_np(gb) - rgb)) <= 1e-2 * np.max(np.abs(rgb)) + 1e-2


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 8, 256, 32, 32), (1, 16, 128, 128, 96), (3, 4, 64, 64, 48),
                                           (2, 32, 16, 32, 16), (1, 16, 32, 96, 128), (1, 3, 256, 64, 64),
                                           (2, 2, 128, 96, 64), (1, 5, 384, 64, 32), (1, 2, 128, 32, 3)])
def test_tensor_core_convolution(plbm, n, h, w, cin, cout):
    """The tcgen05 path (TMA-staged implicit GEMM, TMEM accumulator) against the CPU oracle, for the
    forward pass and, with the channel counts exchanged, the input gradient.  Rows of a multiple of
    128 pixels whose weights fit in shared memory run the persistent halo-row kernel (three halo
    rows per 32-channel block, tap operands at 0, 64 and 128 bytes into a row buffer)."""
    import torch
    lib = _lib(plbm)
    lib.plbm_nn_conv_on_tensor_cores.argtypes = [ctypes.c_int] * 4
    lib.plbm_nn_status.argtypes = [ctypes.POINTER(ctypes.c_int)]
    assert lib.plbm_nn_conv_on_tensor_cores(h, w, cin, cout) == 1
    rng = np.random.default_rng(7 * cin + cout)
    x = nn_ref.bf16_round(rng.standard_normal((n, h, w, cin)))
    wt = nn_ref.bf16_round(rng.standard_normal((cout, 9 * cin)) / np.sqrt(9 * cin))
    b = rng.standard_normal(cout).astype(np.float32)
    y = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    xd, wd, bd = _bf(x), _bf(wt), torch.tensor(b).cuda()
    for relu in (0, 1):
        assert lib.plbm_nn_conv_fwd(xd.data_ptr(), wd.data_ptr(), bd.data_ptr(), y.data_ptr(), n, h, w, cin, cout,
                                    relu, None) == 0
        torch.cuda.synchronize()
        _close(_np(y), nn_ref.conv_fwd(x, wt, b.astype(np.float64), bool(relu)))
    if cin <= 128 and cout % 32 == 0:
        assert lib.plbm_nn_conv_on_tensor_cores(h, w, cout, cin) == 1
        g = nn_ref.bf16_round(rng.standard_normal((n, h, w, cout)))
        gx = torch.empty((n, h, w, cin), dtype=torch.bfloat16, device="cuda")
        assert lib.plbm_nn_conv_dgrad(_bf(g).data_ptr(), wd.data_ptr(), gx.data_ptr(), n, h, w, cin, cout, None) == 0
        torch.cuda.synchronize()
        _close(_np(gx), nn_ref.conv_dgrad(g, wt, cin))
    failed = ctypes.c_int(-1)
    assert lib.plbm_nn_status(ctypes.byref(failed)) == 0 and failed.value == 0


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 8, 256, 32, 32), (1, 16, 128, 128, 96), (4, 16, 128, 64, 64),
                                           (2, 32, 16, 32, 128), (1, 8, 64, 96, 32), (1, 3, 256, 64, 64),
                                           (2, 4, 384, 32, 3), (1, 2, 128, 64, 32), (1, 5, 128, 96, 32)])
def test_tensor_core_weight_gradient(plbm, n, h, w, cin, cout):
    """The weight gradient on tcgen05 (both operands MN-major TMA tiles, split over the pixels,
    FP32 atomics) against the CPU oracle; it accumulates into gw like the other path.  Rows of a
    multiple of 128 pixels whose accumulators fit the TMEM run the halo-row form (an M tile's
    chunks read one halo row at 64-byte offsets), narrow Cout with the gradient written by warps."""
    import torch
    lib = _lib(plbm)
    lib.plbm_nn_status.argtypes = [ctypes.POINTER(ctypes.c_int)]
    rng = np.random.default_rng(11 * cin + cout)
    x = nn_ref.bf16_round(rng.standard_normal((n, h, w, cin)))
    g = nn_ref.bf16_round(rng.standard_normal((n, h, w, cout)))
    rgw, rgb = nn_ref.conv_wgrad(x, g)
    start = rng.standard_normal((cout, 9 * cin)).astype(np.float32)
    gw = torch.tensor(start).cuda()
    gb = torch.zeros(cout, dtype=torch.float32, device="cuda")
    assert lib.plbm_nn_conv_wgrad(_bf(x).data_ptr(), _bf(g).data_ptr(), gw.data_ptr(), gb.data_ptr(), n, h, w, cin,
                                  cout, None) == 0
    torch.cuda.synchronize()
    got = gw.cpu().numpy().astype(np.float64) - start
    assert np.max(np.abs(got - rgw)) <= 1e-3 * np.max(np.abs(rgw)), np.max(np.abs(got - rgw))
    assert np.max(np.abs(_np(gb) - rgb)) <= 1e-2 * np.max(np.abs(rgb)) + 1e-2
    failed = ctypes.c_int(-1)
    assert lib.plbm_nn_status(ctypes.byref(failed)) == 0 and failed.value == 0


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 8, 256, 4, 32), (2, 16, 64, 32, 3), (1, 16, 128, 3, 16),
                                           (1, 8, 128, 5, 7), (2, 4, 32, 16, 8)])
def test_narrow_layers_on_tensor_cores(plbm, n, h, w, cin, cout):
    """Layers with a narrow side (the 4-channel input layer, the 3-channel head and other shapes
    under TMA's 16-byte rows) on tcgen05 with thread-written im2col tiles: the forward pass for
    9 * Cin <= 64, the input gradient for 9 * Cout <= 64 and the weight gradient for Cin <= 32,
    against the CPU oracle; the weight gradient accumulates into a non-zero gw."""
    import torch
    lib = _lib(plbm)
    lib.plbm_nn_conv_on_tensor_cores.argtypes = [ctypes.c_int] * 4
    lib.plbm_nn_wgrad_on_tensor_cores.argtypes = [ctypes.c_int] * 4
    lib.plbm_nn_status.argtypes = [ctypes.POINTER(ctypes.c_int)]
    assert lib.plbm_nn_wgrad_on_tensor_cores(h, w, cin, cout) == 1
    rng = np.random.default_rng(13 * cin + cout)
    x = nn_ref.bf16_round(rng.standard_normal((n, h, w, cin)))
    wt = nn_ref.bf16_round(rng.standard_normal((cout, 9 * cin)) / np.sqrt(9 * cin))
    b = rng.standard_normal(cout).astype(np.float32)
    g = nn_ref.bf16_round(rng.standard_normal((n, h, w, cout)))
    xd, wd, gd, bd = _bf(x), _bf(wt), _bf(g), torch.tensor(b).cuda()
    if 9 * cin <= 64:
        assert lib.plbm_nn_conv_on_tensor_cores(h, w, cin, cout) == 1
        y = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
        for relu in (0, 1):
            assert lib.plbm_nn_conv_fwd(xd.data_ptr(), wd.data_ptr(), bd.data_ptr(), y.data_ptr(), n, h, w, cin,
                                        cout, relu, None) == 0
            torch.cuda.synchronize()
            _close(_np(y), nn_ref.conv_fwd(x, wt, b.astype(np.float64), bool(relu)))
    if 9 * cout <= 64:
        assert lib.plbm_nn_conv_on_tensor_cores(h, w, cout, cin) == 1
        gx = torch.empty((n, h, w, cin), dtype=torch.bfloat16, device="cuda")
        assert lib.plbm_nn_conv_dgrad(gd.data_ptr(), wd.data_ptr(), gx.data_ptr(), n, h, w, cin, cout, None) == 0
        torch.cuda.synchronize()
        _close(_np(gx), nn_ref.conv_dgrad(g, wt, cin))
    rgw, rgb = nn_ref.conv_wgrad(x, g)
    start = rng.standard_normal((cout, 9 * cin)).astype(np.float32)
    gw = torch.tensor(start).cuda()
    gb = torch.zeros(cout, dtype=torch.float32, device="cuda")
    assert lib.plbm_nn_conv_wgrad(xd.data_ptr(), gd.data_ptr(), gw.data_ptr(), gb.data_ptr(), n, h, w, cin, cout,
                                  None) == 0
    torch.cuda.synchronize()
    got = gw.cpu().numpy().astype(np.float64) - start
    assert np.max(np.abs(got - rgw)) <= 1e-3 * np.max(np.abs(rgw)), np.max(np.abs(got - rgw))
    assert np.max(np.abs(_np(gb) - rgb)) <= 1e-2 * np.max(np.abs(rgb)) + 1e-2
    failed = ctypes.c_int(-1)
    assert lib.plbm_nn_status(ctypes.byref(failed)) == 0 and failed.value == 0


def test_pool_and_upsample(plbm):
    import torch
    lib = _lib(plbm)
    rng = np.random.default_rng(3)
    x = nn_ref.bf16_round(rng.standard_normal((2, 8, 12, 16)))
    xd = _bf(x)
    p = torch.empty((2, 4, 6, 16), dtype=torch.bfloat16, device="cuda")
    u = torch.empty((2, 16, 24, 16), dtype=torch.bfloat16, device="cuda")
    gp = torch.empty((2, 8, 12, 16), dtype=torch.bfloat16, device="cuda")
    gu = torch.empty((2, 4, 6, 16), dtype=torch.bfloat16, device="cuda")
    assert lib.plbm_nn_pool2(xd.data_ptr(), p.data_ptr(), 2, 8, 12, 16, None) == 0
    assert lib.plbm_nn_up2(xd.data_ptr(), u.data_ptr(), 2, 16, 24, 16, None) == 0
    assert lib.plbm_nn_pool2_bwd(p.data_ptr(), gp.data_ptr(), 2, 8, 12, 16, None) == 0
    assert lib.plbm_nn_up2_bwd(xd.data_ptr(), gu.data_ptr(), 2, 4, 6, 16, None) == 0
    torch.cuda.synchronize()
    _close(_np(p), nn_ref.pool2(x))
    assert np.array_equal(_np(u), nn_ref.up2(x))
    # adjoints: <pool(x), y> = <x, pool_bwd(y)> and <up(x), z> = <x, up_bwd(z)>
    _close(_np(gp), nn_ref.up2(_np(p)) / 4.0)
    _close(_np(gu), nn_ref.pool2(x) * 4.0)


def test_one_launch_weight_relayout_and_input_gradient(plbm):
    """plbm_nn_flip_layers re-lays out several layers of a flat buffer at once as
    wt[ci][8 - tap][co] = w[co][tap][ci], and plbm_nn_conv_dgrad_pre with it gives
    plbm_nn_conv_dgrad's input gradient bit for bit (TMA-fed, thread-written and mma.sync shapes)."""
    import torch
    lib = _lib(plbm)
    vp, i = ctypes.c_void_p, ctypes.c_int
    lib.plbm_nn_flip_layers.argtypes = [vp, vp, vp, i, i, vp]
    lib.plbm_nn_conv_dgrad_pre.argtypes = [vp, vp, vp, vp, i, i, i, i, i, vp]
    rng = np.random.default_rng(12)
    shapes = [(32, 64), (4, 32), (32, 3), (96, 128), (24, 40)]   # (Cin, Cout)
    offs, off = [], 0
    for ci, co in shapes:
        offs.append(off)
        off += -(-9 * ci * co // 128) * 128
    wflat = np.zeros(off)
    for (ci, co), o in zip(shapes, offs):
        wflat[o:o + 9 * ci * co] = rng.standard_normal(9 * ci * co) * 0.1
    wflat = nn_ref.bf16_round(wflat)
    wd = _bf(wflat)
    wt = torch.zeros_like(wd)
    segs = torch.tensor([[o, ci, co] for (ci, co), o in zip(shapes, offs)], dtype=torch.int32, device="cuda")
    assert lib.plbm_nn_flip_layers(wd.data_ptr(), wt.data_ptr(), segs.data_ptr(), len(shapes),
                                   max(9 * ci * co for ci, co in shapes), None) == 0
    torch.cuda.synchronize()
    wtn = _np(wt)
    for (ci, co), o in zip(shapes, offs):
        w4 = wflat[o:o + 9 * ci * co].reshape(co, 9, ci)
        assert np.array_equal(wtn[o:o + 9 * ci * co].reshape(ci, 9, co), w4[:, ::-1, :].transpose(2, 1, 0))
    for (ci, co), o, (n, h, w) in zip(shapes, offs, [(2, 8, 256), (2, 16, 64), (1, 8, 256), (1, 32, 32), (2, 8, 24)]):
        g = _bf(nn_ref.bf16_round(rng.standard_normal((n, h, w, co))))
        a = torch.empty((n, h, w, ci), dtype=torch.bfloat16, device="cuda")
        b = torch.empty_like(a)
        n_el = 9 * ci * co
        assert lib.plbm_nn_conv_dgrad(g.data_ptr(), wd[o:].data_ptr(), a.data_ptr(), n, h, w, ci, co, None) == 0
        assert lib.plbm_nn_conv_dgrad_pre(g.data_ptr(), wd[o:].data_ptr(), wt[o:].data_ptr(), b.data_ptr(), n, h, w,
                                          ci, co, None) == 0
        torch.cuda.synchronize()
        assert torch.equal(a, b), (ci, co, n_el)


@pytest.mark.parametrize("p,c", [(4096, 32), (3000, 96), (777, 128), (500, 12)])
def test_relu_backward_with_bias_gradient(plbm, p, c):
    """plbm_nn_relu_bwd_bias masks the gradient where the activation is not positive (bit-exact) and
    adds the masked gradient's per-channel sums to gb (FP32 sums: 1e-4 relative); c = 12 runs the
    element-wise fallback."""
    import torch
    lib = plbm.load_library()
    vp, ll, i = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int
    lib.plbm_nn_relu_bwd_bias.argtypes = [vp, vp, vp, ll, i, vp]
    rng = np.random.default_rng(p + c)
    y = nn_ref.bf16_round(rng.standard_normal((p, c)))
    y[rng.random((p, c)) < 0.05] = 0.0
    g = nn_ref.bf16_round(rng.standard_normal((p, c)))
    yd, gd = _bf(y), _bf(g)
    gb0 = rng.standard_normal(c).astype(np.float32)
    gb = torch.from_numpy(gb0.copy()).cuda()
    assert lib.plbm_nn_relu_bwd_bias(yd.data_ptr(), gd.data_ptr(), gb.data_ptr(), p, c, None) == 0
    torch.cuda.synchronize()
    masked = np.where(y > 0, g, 0.0)
    assert np.array_equal(_np(gd), masked)
    ref = gb0.astype(np.float64) + masked.sum(axis=0)
    assert np.max(np.abs(gb.cpu().numpy() - ref)) <= 1e-4 * np.max(np.abs(masked).sum(axis=0)) + 1e-5


def test_adam_on_device_matches_host_adam(plbm):
    """plbm_nn_adam_dev (learning rate and step count read on the device, the count advanced by
    the launch) gives plbm_nn_adam's update for steps 1..3, and leaves its block counter at zero."""
    import torch
    lib = plbm.load_library()
    vp, ll, f, i = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_float, ctypes.c_int
    lib.plbm_nn_adam.argtypes = [vp, vp, vp, vp, vp, ll, f, f, f, f, i, vp]
    lib.plbm_nn_adam_dev.argtypes = [vp, vp, vp, vp, vp, ll, vp, f, f, f, vp, vp]
    n = 100_003
    gen = torch.Generator().manual_seed(4)
    w0, g0 = torch.randn(n, generator=gen), torch.randn(n, generator=gen) * 1e-2
    bufs = []
    for _ in range(2):
        w, g, m, v = w0.cuda(), g0.cuda(), torch.zeros(n, device="cuda"), torch.zeros(n, device="cuda")
        bufs.append((w, g, m, v, torch.zeros(n, dtype=torch.bfloat16, device="cuda")))
    lr = torch.tensor([2e-3], device="cuda")
    state = torch.zeros(2, dtype=torch.int32, device="cuda")
    for t in (1, 2, 3):
        w, g, m, v, wb = bufs[0]
        assert lib.plbm_nn_adam(w.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(), wb.data_ptr(), n, 2e-3, 0.9,
                                0.999, 1e-8, t, None) == 0
        w, g, m, v, wb = bufs[1]
        assert lib.plbm_nn_adam_dev(w.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(), wb.data_ptr(), n,
                                    lr.data_ptr(), 0.9, 0.999, 1e-8, state.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert state.tolist() == [3, 0]
    for a, b in zip(bufs[0], bufs[1]):
        a, b = a.float(), b.float()
        assert torch.allclose(a, b, rtol=1e-5, atol=1e-7)
    assert (bufs[1][0] - w0.cuda()).abs().max().item() > 1e-3     # the weights moved by ~3 lr


def test_captured_training_step_matches_eager(plbm):
    """A training step captured as a CUDA graph (NeuralOperator.capture_train_step) computes the
    eager step's output bit for bit and its gradients to the weight-gradient tolerance; replays
    advance the device-held Adam step count and apply the learning rate set before each."""
    import torch
    from portlbm_gb300 import warmstart as ws
    rng = np.random.default_rng(8)
    n, h, w = 2, 128, 128
    masks = torch.from_numpy((rng.random((n, h, w)) < 0.3).astype(np.int8)).cuda()
    gout = _bf(rng.standard_normal((n, h, w, 3)) * 1e-2)
    eager, graphed = ws.NeuralOperator(seed=6), ws.NeuralOperator(seed=6)
    x = eager.assemble(masks, [ws.features(w, 1.02, 1.0, 0.8)] * n)
    out_e = eager.forward(x, n, h, w).clone()
    eager.zero_grad()
    eager.backward(gout.clone())
    torch.cuda.synchronize()
    w0 = graphed.params.w.clone()
    step = graphed.capture_train_step(x, gout, n, h, w)
    step(0.0)
    torch.cuda.synchronize()
    assert torch.equal(step.out, out_e)
    ge, gg = eager.params.g, graphed.params.g
    assert (ge - gg).abs().max().item() <= 1e-3 * ge.abs().max().item()
    assert torch.equal(graphed.params.w, w0)                        # lr 0: the weights stay
    step(1e-3)
    step(1e-3)
    torch.cuda.synchronize()
    assert step.state.tolist() == [3, 0] and graphed.step_count == 3
    moved = (graphed.params.w - w0).abs().max().item()
    assert 1e-3 < moved <= 2e-3 * 1.01


def test_operator_trains_on_solver_steady_states(plbm):
    """A short training run on 32 solver steady states (64x64) lowers the loss, and the prediction
    initialises a handler that still reaches residual 1e-6."""
    from portlbm_gb300 import warmstart as ws
    data = ws.generate_dataset(32, 64, 64, seed=3, steps=3000, per_batch=32)
    model = ws.NeuralOperator(seed=1)
    hist = ws.train(model, data, epochs=6, batch=8, lr=3e-3)
    assert hist["loss_history"][-1] < hist["loss_history"][0]
    chan = data[0]
    pred = model.predict(chan["mask"], chan["rin"], chan["rout"], chan["tau"])
    assert all(np.all(np.isfinite(a)) for a in pred)
    res = ws.solve(chan, init=pred, max_steps=100000)
    assert res["residual"] < 1e-6


def test_trained_operator_cuts_steps_to_steady_state(plbm):
    """What the network gains: trained briefly on 64x64 steady states, its prediction starts six
    held-out 256x64 channels that reach residual 1e-6 in fewer steps than from rest, at the same
    steady state (the rest start stays the fallback)."""
    from portlbm_gb300 import warmstart as ws
    data = ws.generate_dataset(192, 64, 64, seed=5, steps=8000, per_batch=192)
    model = ws.NeuralOperator(seed=2)
    ws.train(model, data, epochs=20, batch=16, lr=2e-3)
    rng = np.random.default_rng(17)
    chans = []
    while len(chans) < 6:
        c = ws.random_channel(rng, 256, 64)
        if c["tau"] >= 0.7:              # well inside the stable range of BGK
            chans.append(c)
    rows = ws.evaluate(model, chans, ablation=False)
    agg = ws.aggregate(rows)
    print(agg)
    assert agg["n"] == 6 and agg["diverged"] == 0
    assert agg["steps_reduction_total"] > 1.15       # measured 1.37 after 12 epochs
    assert agg["max_state_diff"] < 0.05

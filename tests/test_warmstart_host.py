"""Host-side logic of the learned warm start (no GPU): target scaling, the series-resistance
profile, divergence screening and the aggregation of the held-out comparison."""
import numpy as np
import pytest

ws = pytest.importorskip("portlbm_gb300.warmstart")


def test_linear_profile_spans_the_ghost_columns():
    w, rin, rout = 10, 1.05, 1.0
    p = ws.linear_profile(w, rin, rout)
    g, _ = ws.channel_scales(w, rin, rout, 0.8)
    assert p.shape == (w,)
    assert np.isclose(p[0] + g, rin) and np.isclose(p[-1] - g, rout)
    assert np.allclose(np.diff(p), -g)


def test_series_profile_uniform_flux_is_the_straight_profile():
    w, h = 12, 5
    mask = np.zeros((h, w), np.int8)
    s, rho_b = ws.series_profile(np.full((h, w), 0.01), mask, w, 1.02, 1.0, 0)
    assert np.allclose(s, 1.0)
    assert np.allclose(rho_b, ws.linear_profile(w, 1.02, 1.0))


def test_series_profile_equalises_column_fluxes():
    """With sigma = 0, scaling each column by s makes every column carry the same flux, and the
    drops over the W + 1 links still add up to rin - rout."""
    w, h = 16, 6
    rng = np.random.default_rng(3)
    mask = (rng.random((h, w)) < 0.2).astype(np.int8)
    jx = rng.uniform(0.5, 1.5, (h, w)) * 1e-3
    s, rho_b = ws.series_profile(jx, mask, w, 1.03, 1.0, 0)
    q = np.where(mask == 0, jx, 0).sum(0) * s
    assert np.allclose(q, q[0])
    assert np.isclose(s.mean(), 1.0)
    links = np.concatenate([[s[0]], 0.5 * (s[1:] + s[:-1]), [s[-1]]])
    assert np.isclose(1.03 - rho_b[-1], 0.03 * links[:-1].sum() / links.sum())
    assert np.all(np.diff(rho_b) < 0)


def test_series_profile_rejects_backward_net_flux():
    w, h = 8, 4
    jx = np.full((h, w), 1e-3)
    jx[:, 3] = -1e-3
    assert ws.series_profile(jx, np.zeros((h, w), np.int8), w, 1.02, 1.0, 0) is None


def test_features_are_order_one_over_the_parameter_range():
    for w in (256, 1024):
        for tau in (0.55, 1.0):
            for rin in (1.001, 1.05):
                f = ws.features(w, rin, 1.0, tau)
                assert f[0] == 1.0 and all(abs(v) < 3 for v in f)


def test_converged_fields_screens_diverged_runs():
    mask = np.zeros((3, 4), np.int8)
    mask[0] = 1
    ok = [np.full(12, 1.01), np.full(12, 1e-3), np.zeros(12)]
    assert ws.converged_fields(mask, *ok)
    zeros = [np.zeros(12)] * 3                      # what the NaN guard leaves
    assert not ws.converged_fields(mask, *zeros)
    bad = [ok[0].copy(), ok[1], ok[2]]
    bad[0][5] = np.nan
    assert not ws.converged_fields(mask, *bad)


def test_aggregate_counts_fallbacks_and_excludes_diverged():
    rows = [
        {"size": "a", "cold_steps": 1000, "cold_s": 1.0, "warm_steps": 250, "warm_s": 0.25, "fallback": False,
         "state_diff": 0.01, "ramp_steps": 500},
        {"size": "a", "cold_steps": 3000, "cold_s": 3.0, "warm_steps": 3200, "warm_s": 3.2, "fallback": True,
         "state_diff": 0.0, "ramp_steps": 1500},
        {"size": "a", "cold_steps": None, "fallback": None},
    ]
    a = ws.aggregate(rows)
    assert a["n"] == 2 and a["diverged"] == 1 and a["fallbacks"] == 1
    assert np.isclose(a["steps_reduction_total"], 4000 / 3450)
    assert np.isclose(a["time_reduction_total"], 4.0 / 3.45)
    assert np.isclose(a["ramp_only_steps_reduction_total"], 2.0)
    assert a["max_state_diff"] == 0.01


def test_state_difference_over_fluid_nodes():
    mask = np.array([[0, 1, 0]], np.int8)
    a = (np.array([1.0, 9.0, 1.0]), np.zeros(3))
    b = (np.array([1.0, -5.0, 2.0]), np.zeros(3))
    assert np.isclose(ws.state_difference(mask, a, b), 1.0 / np.sqrt(5.0))


@pytest.mark.parametrize("h,w", [(256, 256), (256, 1024)])
def test_tensor_core_dispatch_covers_the_network(plbm, h, w):
    """Every convolution of the operator, every input gradient and every weight gradient runs on
    tcgen05 (the TMA-fed kernels, or for the 4-channel input layer and the 3-channel head the
    kernels whose threads write the im2col tiles): the host-side dispatch predicates over each
    layer's resolution and channel counts."""
    import ctypes
    lib = plbm.load_library()
    lib.plbm_nn_conv_on_tensor_cores.argtypes = [ctypes.c_int] * 4
    lib.plbm_nn_wgrad_on_tensor_cores.argtypes = [ctypes.c_int] * 4
    tc, tcw = lib.plbm_nn_conv_on_tensor_cores, lib.plbm_nn_wgrad_on_tensor_cores
    layers = [(lvl, ci, co) for lvl in range(5) for ci, co in ws.ENC[2 * lvl:2 * lvl + 2]]
    layers += [(lvl, ci, co) for k, lvl in enumerate((3, 2, 1, 0)) for ci, co in ws.DEC[2 * k:2 * k + 2]]
    layers.append((0,) + tuple(ws.HEAD))
    for lvl, ci, co in layers:
        hh, ww = h >> lvl, w >> lvl
        assert tc(hh, ww, ci, co) == 1, (lvl, ci, co)
        assert tcw(hh, ww, ci, co) == 1, (lvl, ci, co)
        if ci != ws.C_IN:   # the input gradient: a forward kernel with the channels swapped
            assert tc(hh, ww, co, ci) == 1, (lvl, co, ci)
    # shapes neither tcgen05 kernel tiles fall back to mma.sync
    assert tc(16, 24, 4, 32) == 0 and tc(256, 256, 16, 32) == 0 and tcw(256, 256, 48, 32) == 0

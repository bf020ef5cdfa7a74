"""Parity of the CUDA path with the CPU oracle (restated reference), through the C ABI.

The drop-in form (f64_strict) must match the oracle exactly (max-abs difference 0.0) for
every algorithm x data layout; f64_fast must agree within 1e-12 (the tolerance of the
reference comparison); the buffered-outlet case (W-1 divisible by the subdomain width,
src/lbm/core/simulation.cpp + include/lbm/gpu/general/buffered.hpp:285-288) must reproduce the
reference's npol/nsol behaviour.
"""
import numpy as np
import pytest

ALGS = ["nptl", "lptl", "npol", "nsol"]
LAYOUTS = ["collision", "stream", "bundle"]
pytestmark = pytest.mark.gpu


def run_gpu(plbm, alg, lay, scenario, w, h, steps, wg=64, precision="f64_strict", rho_in=1.05, tau=0.6, mask=None,
            fui=None, gather="auto"):
    props = plbm.Properties(alg, lay, False, wg, steps, fui or steps, scenario, h, w, 0.0, 0.0, rho_in, 0.0, 0.0,
                            1.0, tau)
    hd = plbm.create_handler(props, precision=precision, mask=mask, gather=gather)
    hd.start()
    hd.block_until_finished()
    out = {"rho": hd.get_densities(), "jx": hd.get_x_velocities(), "jy": hd.get_y_velocities(),
           "jabs": hd.get_absolute_velocities()}
    hd.close()
    return out


def run_oracle(oracle_mod, alg, lay, scenario, w, h, steps, wg=64, rho_in=1.05, tau=0.6, mask=None):
    o = oracle_mod.Oracle(alg, lay, wg, scenario, w, h, inlet_density=rho_in, relaxation_time=tau, mask=mask)
    o.run(steps)
    return o.results()


def maxdiff(a, b):
    return max(float(np.max(np.abs(a[k] - b[k]))) for k in a)


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("lay", LAYOUTS)
def test_strict_matches_oracle_exactly(plbm, oracle_mod, alg, lay):
    ref = run_oracle(oracle_mod, alg, lay, "circle", 62, 30, 300)
    got = run_gpu(plbm, alg, lay, "circle", 62, 30, 300)
    assert maxdiff(got, ref) == 0.0


@pytest.mark.parametrize("alg", ALGS)
def test_fast_within_tolerance(plbm, oracle_mod, alg):
    ref = run_oracle(oracle_mod, alg, "stream", "circle", 62, 30, 300)
    got = run_gpu(plbm, alg, "stream", "circle", 62, 30, 300, precision="f64_fast")
    assert maxdiff(got, ref) <= 1e-12


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("lay", LAYOUTS)
def test_q60_within_tolerance(plbm, oracle_mod, alg, lay):
    """The integer-pipe FP64-accuracy form agrees with the reference arithmetic to <= 1e-12."""
    ref = run_oracle(oracle_mod, alg, lay, "circle", 62, 30, 300)
    got = run_gpu(plbm, alg, lay, "circle", 62, 30, 300, precision="f64_q60")
    assert maxdiff(got, ref) <= 1e-12


@pytest.mark.parametrize("precision", ["f16s", "bf16s", "f16c"])
@pytest.mark.parametrize("w,h,porous", [(203, 61, True), (300, 40, True), (62, 30, False), (520, 20, True)])
def test_vectorised_rows_match_scalar_kernel(plbm, precision, w, h, porous):
    """nptl/stream runs the 2-byte forms 8 nodes per thread with warp shuffles (open gather: solid
    sources re-gathered node by node; porous gather: bounce-back merged word-wise); lptl and the
    collision and bundle layouts run the scalar kernels: same arithmetic, bit-identical results
    (row lengths not a multiple of 8 or 256, porous obstacles, inlet, outlet, walls)."""
    mask = plbm.porous_disks(w, h, 9, 0.7) if porous else None
    scen = "Hagen-Poiseuille" if porous else "circle"
    a = run_gpu(plbm, "nptl", "stream", scen, w, h, 300, precision=precision, mask=mask, gather="open")
    others = [run_gpu(plbm, alg, lay, scen, w, h, 300, precision=precision, mask=mask, gather=g)
              for alg, lay, g in (("lptl", "stream", "open"), ("nptl", "collision", "open"),
                                  ("nptl", "stream", "porous"), ("lptl", "bundle", "porous"))]
    for k in a:
        for b in others:
            assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("precision", ["f32", "f16s", "f16c", "f64_strict"])
@pytest.mark.parametrize("alg,lay", [("nptl", "stream"), ("nptl", "bundle"), ("lptl", "collision")])
def test_gather_forms_agree(plbm, precision, alg, lay):
    """The open and the porous gather give bit-identical results on a porous channel; "auto"
    takes the porous gather there and the open one in a channel with a single disk (the FP64
    forms have one gather)."""
    w, h = 157, 53
    mask = plbm.porous_disks(w, h, 4, 0.7)
    a = run_gpu(plbm, alg, lay, "Hagen-Poiseuille", w, h, 250, precision=precision, mask=mask, gather="open")
    b = run_gpu(plbm, alg, lay, "Hagen-Poiseuille", w, h, 250, precision=precision, mask=mask, gather="porous")
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    props = plbm.Properties(alg, lay, False, 64, 10, 10, "Hagen-Poiseuille", h, w, 0.0, 0.0, 1.05, 0.0, 0.0, 1.0, 0.6)
    shifted = precision != "f64_strict"
    for m, g, want in ((mask, "auto", "porous" if shifted else "open"), (None, "auto", "open"),
                       (None, "porous", "porous" if shifted else "open")):
        hd = plbm.create_handler(props, precision=precision, mask=m, gather=g)
        assert hd.gather_form() == want
        hd.close()


# relative L2 of the momentum field / max |rho| difference against f64_strict after 600 steps, in the
# transient of a small channel (every algorithm x layout); the steady-state bars (FP16 <= 1e-3)
# are pinned by test_shifted_steady_state_against_converged_fp64
SHIFTED_TOL = {"f32": (1e-4, 2e-6), "f16s": (2e-3, 2e-4), "bf16s": (2e-2, 2e-3), "f16c": (1e-3, 1e-4)}


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("precision", ["f32", "f16s", "bf16s", "f16c"])
@pytest.mark.parametrize("lay,porous", [("stream", False), ("stream", True), ("collision", True), ("bundle", False)])
def test_shifted_forms_track_fp64(plbm, alg, precision, lay, porous):
    """Every algorithm and data layout in the FP32/FP16/BF16 storage forms stays within its storage
    precision of the FP64 drop-in (circle channel and a porous mask; nptl/lptl re-reference to the
    inlet-outlet profile, npol/nsol to rho0 = 1 and keep halo snapshots and swapped slots in that
    form)."""
    w, h = 203, 61
    mask = plbm.porous_disks(w, h, 9, 0.8) if porous else None
    scen = "Hagen-Poiseuille" if porous else "circle"
    ref = run_gpu(plbm, alg, lay, scen, w, h, 600, mask=mask)
    got = run_gpu(plbm, alg, lay, scen, w, h, 600, precision=precision, mask=mask)
    jr = np.concatenate([ref["jx"], ref["jy"]])
    jg = np.concatenate([got["jx"], got["jy"]])
    l2, drho = np.linalg.norm(jg - jr) / np.linalg.norm(jr), np.abs(got["rho"] - ref["rho"]).max()
    tl2, trho = SHIFTED_TOL[precision]
    assert l2 <= tl2 and drho <= trho, (l2, drho)


def test_q60_rejects_out_of_range_boundary(plbm):
    props = plbm.Properties("nptl", "stream", False, 64, 10, 10, "circle", 30, 62, 0.0, 0.0, 10.0, 0.0, 0.0, 1.0, 0.6)
    with pytest.raises(plbm.Exception, match="f64_q60"):
        plbm.create_handler(props, precision="f64_q60")


@pytest.mark.parametrize("alg,w,wg", [("npol", 65, 64), ("nsol", 61, 64), ("npol", 33, 16), ("nsol", 33, 16)])
def test_buffered_outlet_case(plbm, oracle_mod, alg, w, wg):
    ref = run_oracle(oracle_mod, alg, "stream", "Hagen-Poiseuille", w, 20, 300, wg=wg)
    got = run_gpu(plbm, alg, "stream", "Hagen-Poiseuille", w, 20, 300, wg=wg)
    assert maxdiff(got, ref) == 0.0


@pytest.mark.parametrize("scenario", ["walls", "square", "plate", "skyscraper", "wing"])
def test_scenarios_exact(plbm, oracle_mod, scenario):
    ref = run_oracle(oracle_mod, "nptl", "stream", scenario, 90, 48, 200)
    got = run_gpu(plbm, "nptl", "stream", scenario, 90, 48, 200)
    assert maxdiff(got, ref) == 0.0


def test_poiseuille_config_exact_10k_steps(plbm, oracle_mod):
    """Config: Hagen-Poiseuille 400x100, nptl + stream, tau 0.6, rho 1.2/1.0, 10^4 steps."""
    ref = run_oracle(oracle_mod, "nptl", "stream", "Hagen-Poiseuille", 400, 100, 10000, wg=1024, rho_in=1.2)
    got = run_gpu(plbm, "nptl", "stream", "Hagen-Poiseuille", 400, 100, 10000, wg=1024, rho_in=1.2)
    assert maxdiff(got, ref) == 0.0
    for prec in ("f64_fast", "f64_q60"):
        got = run_gpu(plbm, "nptl", "stream", "Hagen-Poiseuille", 400, 100, 10000, wg=1024, rho_in=1.2,
                      precision=prec)
        assert maxdiff(got, ref) <= 1e-12, prec


GOLDEN_CASES = None


def _golden():
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    cases = json.load(open(os.path.join(here, "golden", "cases.json")))
    return cases, np.load(os.path.join(here, "golden", "golden.npz"))


_CASES, _ARRAYS = _golden()


@pytest.mark.parametrize("case", _CASES, ids=[c["name"] for c in _CASES])
def test_gpu_matches_reference_golden(plbm, case):
    """GPU results equal the reference's own results (tests/golden, generated by running the
    reference's algorithm classes) exactly: f64_strict for double cases, f32_ref for USE_FLOAT."""
    import ctypes
    if case["scenario"] == "porous":
        ctypes.CDLL(None).srand(case["rand_seed"])
    precision = "f64_strict" if case["precision"] == "f64" else "f32_ref"
    got = run_gpu(plbm, case["algorithm"], case["data_layout"], case["scenario"], case["w"], case["h"],
                  case["steps"], wg=case["work_group_size"], precision=precision, rho_in=case["inlet_density"],
                  tau=case["relaxation_time"])
    for k in ("rho", "jx", "jy", "jabs"):
        ref = _ARRAYS[f"{case['name']}__{k}"]
        assert np.array_equal(got[k], ref), f"{k}: max abs {np.max(np.abs(got[k] - ref))}"


def test_residual_decreases_and_steady_state_is_reached(plbm):
    """run_to_residual: a 128x48 porous channel reaches residual 1e-6, and the momentum it reports
    equals the momentum of the last step."""
    mask = plbm.porous_disks(128, 48, 3, 0.7)
    props = plbm.Properties("nptl", "stream", False, 64, 10 ** 6, 10 ** 6, "Hagen-Poiseuille", 48, 128, 0.0, 0.0,
                            1.01, 0.0, 0.0, 1.0, 0.6)
    hd = plbm.create_handler(props, precision="f64_q60", mask=mask)
    steps, r = hd.run_to_residual(1e-6, 100, 200000)
    assert r < 1e-6 and steps < 200000
    jx = hd.get_x_velocities()
    assert np.all(np.isfinite(jx)) and jx[mask.reshape(-1) == 0].mean() > 0


@pytest.mark.parametrize("frame", [10, 7])
def test_frames_written_to_the_host_match_a_run_of_that_length(plbm, frame):
    """Frames inside the step loop's frame graphs are written by the step kernel straight into the
    host arrays: after a pause mid-run they equal a separate run of exactly that many steps."""
    import time
    props = plbm.Properties("nptl", "stream", False, 64, 10 ** 6, frame, "circle", 30, 62, 0.0, 0.0, 1.05, 0.0, 0.0,
                            1.0, 0.6)
    hd = plbm.create_handler(props, precision="f64_strict")
    hd.start()
    time.sleep(0.2)
    hd.pause()
    k = hd.get_current_iteration()
    assert k > 0 and k % frame == 0
    got = {"rho": hd.get_densities(), "jx": hd.get_x_velocities(), "jy": hd.get_y_velocities()}
    hd.close()
    ref = run_gpu(plbm, "nptl", "stream", "circle", 62, 30, k)
    for key, v in got.items():
        assert np.array_equal(v, ref[key]), key


def test_residual_windows_chain_across_calls(plbm):
    """The snapshot of one call is the baseline of the next: K-step calls report the same residuals
    as one call over the same steps."""
    mask = plbm.porous_disks(96, 40, 5, 0.7)
    props = plbm.Properties("nptl", "stream", False, 64, 10 ** 6, 10 ** 6, "Hagen-Poiseuille", 40, 96, 0.0, 0.0,
                            1.02, 0.0, 0.0, 1.0, 0.7)
    a = plbm.create_handler(props, precision="f64_q60", mask=mask)
    b = plbm.create_handler(props, precision="f64_q60", mask=mask)
    s1, r1 = a.run_to_residual(0.0, 50, 50)
    assert s1 == 50 and r1 == float("inf")          # no snapshot before the first window
    s2, r2 = a.run_to_residual(0.0, 50, 50)
    s3, r3 = b.run_to_residual(0.0, 50, 100)
    # same fields; the FP64 sums are accumulated with atomics, so the order (last bits) may differ
    assert s2 == 50 and s3 == 100 and np.isfinite(r2) and abs(r2 - r3) <= 1e-12 * r3
    a.close()
    b.close()


def _outlet_strip_mask(w, h):
    """Walls on the first/last rows and a block reaching column W-2, leaving a one-node strip of
    fluid in the outlet column beside it."""
    m = np.zeros((h, w), dtype=np.int8)
    m[0, :] = m[-1, :] = 1
    m[4:h - 5, w - 9:w - 1] = 1
    m[6:9, 10:14] = 1
    return m


@pytest.mark.parametrize("precision", ["f64_strict", "f64_q60", "f32"])
def test_set_equilibrium_ignores_solid_entries(plbm, precision):
    """Values at solid nodes, including column W-2 whose jy the outlet reads, do not reach the run."""
    w, h = 48, 24
    mask = _outlet_strip_mask(w, h)
    props = plbm.Properties("nptl", "stream", False, 64, 10 ** 6, 10 ** 6, "Hagen-Poiseuille", h, w, 0.0, 0.0,
                            1.02, 0.0, 0.0, 1.0, 0.8)
    rng = np.random.default_rng(0)
    x = np.arange(w)[None, :].repeat(h, 0)
    clean = [(1.02 - 0.02 * (x + 1) / (w + 1)).ravel(), np.full(w * h, 2e-3), 1e-4 * rng.standard_normal(w * h)]
    solid = mask.reshape(-1) == 1
    for f in clean:
        f[solid] = 0.0
    dirty = [f.copy() for f in clean]
    for f in dirty:
        f[solid] = rng.uniform(-0.5, 0.5, solid.sum())
    out = []
    for fields in (clean, dirty):
        hd = plbm.create_handler(props, precision=precision, mask=mask)
        hd.set_equilibrium(*fields)
        hd.run_steps(400)
        hd.sync_results()
        out.append([hd.get_densities().copy(), hd.get_x_velocities().copy(), hd.get_y_velocities().copy()])
        hd.close()
    for k in range(3):
        assert np.array_equal(out[0][k], out[1][k]), k


@pytest.mark.parametrize("fui", [60, 10])
def test_result_readers_agree_after_host_written_steps(plbm, fui):
    """The step loop's result steps write the observables straight into the mapped host arrays
    (fui = 60: the last step; fui = 10: frame graphs too), so the device copies are then older:
    mass_momentum must still sum the newest results, sync_results must leave the host arrays as
    they are, and after device-resident steps both must follow those."""
    w, h = 70, 33
    mask = plbm.porous_disks(w, h, 3, 0.8)
    fluid = mask.reshape(-1) == 0
    props = plbm.Properties("nptl", "stream", False, 64, 60, fui, "Hagen-Poiseuille", h, w, 0.0, 0.0,
                            1.03, 0.0, 0.0, 1.0, 0.7)
    hd = plbm.create_handler(props, precision="f64_strict", mask=mask)

    def host_sums():
        return [float(np.sum(a[fluid])) for a in (hd.get_densities(), hd.get_x_velocities(), hd.get_y_velocities())]

    hd.start()
    hd.block_until_finished()
    before = [hd.get_densities().copy(), hd.get_x_velocities().copy(), hd.get_y_velocities().copy()]
    assert abs(before[1][fluid]).max() > 0                        # the run produced results
    assert np.allclose(hd.mass_momentum(), host_sums(), rtol=1e-12, atol=1e-12)
    hd.sync_results()
    after = [hd.get_densities(), hd.get_x_velocities(), hd.get_y_velocities()]
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    hd.run_steps(7)
    hd.sync_results()
    assert not np.array_equal(before[0], hd.get_densities())
    assert np.allclose(hd.mass_momentum(), host_sums(), rtol=1e-12, atol=1e-12)
    hd.close()


@pytest.mark.parametrize("precision", ["f64_strict", "f64_q60"])
def test_set_equilibrium_of_rest_state_is_the_rest_start(plbm, precision):
    """Loading rho = 1, j = 0 gives the same run as the handler's own initialisation."""
    w, h = 48, 24
    mask = _outlet_strip_mask(w, h)
    props = plbm.Properties("nptl", "stream", False, 64, 10 ** 6, 10 ** 6, "Hagen-Poiseuille", h, w, 0.0, 0.0,
                            1.02, 0.0, 0.0, 1.0, 0.8)
    out = []
    for load in (False, True):
        hd = plbm.create_handler(props, precision=precision, mask=mask)
        if load:
            hd.set_equilibrium(np.ones(w * h), np.zeros(w * h), np.zeros(w * h))
        hd.run_steps(300)
        hd.sync_results()
        out.append([hd.get_densities().copy(), hd.get_x_velocities().copy()])
        hd.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def _batch_domains(plbm, n=5, seed=11, wmax=140):
    rng = np.random.default_rng(seed)
    doms = []
    for i in range(n):
        w, h = int(rng.integers(40, wmax)), int(rng.integers(24, 90))
        doms.append({"mask": plbm.porous_disks(w, h, seed + i, float(rng.uniform(0.6, 0.8))),
                     "relaxation_time": float(rng.uniform(0.55, 1.0)),
                     "inlet_density": float(rng.uniform(1.001, 1.05)), "outlet_density": 1.0})
    return doms


@pytest.mark.parametrize("precision", ["f32", "f16s", "bf16s", "f16c", "f64_q60"])
@pytest.mark.parametrize("mode", ["persistent", "persistent_graph", "per_domain"])
@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("vec_rows", [False, True])
def test_batch_equals_independent_handlers(plbm, precision, mode, wide, vec_rows):
    """Every domain of a batch ends bit-identical to the same channel run alone by a handler.
    `wide` draws widths up to 700, so a domain spans several tiles across (and several 256-node
    row segments with the vectorised rows of the 2-byte batches)."""
    if vec_rows and (precision in ("f32", "f64_q60") or mode == "per_domain"):
        pytest.skip("vectorised rows are a tile option of the persistent 2-byte batches")
    doms = _batch_domains(plbm, wmax=700 if wide else 140)
    b = plbm.Batch(doms, precision=precision)
    b.set_tile(32, 4 + 256 * (2 if wide else 1) + (plbm.BATCH_TILE_VEC if vec_rows else 0), 8)
    steps = 150
    b.run(steps, mode=mode)
    for i, d in enumerate(doms):
        h, w = d["mask"].shape
        props = plbm.Properties("nptl", "stream", False, 64, steps, steps, "Hagen-Poiseuille", h, w, 0.0, 0.0,
                                d["inlet_density"], 0.0, 0.0, 1.0, d["relaxation_time"])
        hd = plbm.create_handler(props, precision=precision, mask=d["mask"])
        hd.start()
        hd.block_until_finished()
        for k, get in enumerate((hd.get_densities, hd.get_x_velocities, hd.get_y_velocities)):
            assert np.array_equal(b.result(i, k), get()), (i, k)
        hd.close()
    b.close()


@pytest.mark.parametrize("precision", ["f16s", "bf16s", "f16c"])
def test_batch_vectorised_rows_across_row_ends(plbm, precision):
    """The vectorised batch walks each domain in row-major order, 256 nodes per warp, so a warp's
    lanes span rows: widths that are multiples of 32 end a row exactly at a lane (its neighbour lane
    starts the next row), and node counts that are not multiples of 256 leave a partial last
    segment.  Every domain still ends bit-identical to the channel run alone."""
    rng = np.random.default_rng(23)
    doms = []
    for i, (w, h) in enumerate(((32, 24), (64, 25), (96, 31), (256, 17), (40, 29), (72, 9), (288, 40))):
        doms.append({"mask": plbm.porous_disks(w, h, 40 + i, 0.75), "relaxation_time": float(rng.uniform(0.55, 1.0)),
                     "inlet_density": float(rng.uniform(1.001, 1.05)), "outlet_density": 1.0})
    b = plbm.Batch(doms, precision=precision)
    b.set_tile(32, 2 + 256 * 2 + plbm.BATCH_TILE_VEC, 4)
    steps = 120
    b.run(steps, mode="persistent_graph")
    for i, d in enumerate(doms):
        h, w = d["mask"].shape
        props = plbm.Properties("nptl", "stream", False, 64, steps, steps, "Hagen-Poiseuille", h, w, 0.0, 0.0,
                                d["inlet_density"], 0.0, 0.0, 1.0, d["relaxation_time"])
        hd = plbm.create_handler(props, precision=precision, mask=d["mask"])
        hd.start()
        hd.block_until_finished()
        for k, get in enumerate((hd.get_densities, hd.get_x_velocities, hd.get_y_velocities)):
            assert np.array_equal(b.result(i, k), get()), (i, k)
        hd.close()
    b.close()


@pytest.mark.parametrize("precision", ["f32", "f16s", "f16c"])
def test_batch_autotune_keeps_results(plbm, precision):
    """Autotuning times real steps (7 tile shapes x 3 occupancies x 2 steps, twice that for 2-byte
    storage, which also tries vectorised rows) and results do not depend on the tile it picks."""
    doms = _batch_domains(plbm, n=3, seed=5, wmax=600)
    a = plbm.Batch(doms, precision=precision)
    a.autotune(steps=2)
    a.run(58)
    tuned = 2 * 21 * (2 if precision in ("f16s", "f16c") else 1)
    ref = plbm.Batch(doms, precision=precision)
    ref.run(tuned + 58, mode="per_domain")
    for i in range(len(doms)):
        for k in range(3):
            assert np.array_equal(a.result(i, k), ref.result(i, k))
    na, _ = a.info()
    assert na == sum(d["mask"].size for d in doms)


def test_f16c_rejects_boundaries_beyond_its_range(plbm):
    """f16c stores deviations |f - w rho0| < 0.5: an inlet density of 3.5 puts the rest
    population's deviation beyond that and creation fails with a numeric error."""
    props = plbm.Properties("nptl", "stream", False, 64, 10, 10, "circle", 30, 62, 0.0, 0.0, 3.5, 0.0, 0.0, 1.0, 0.6)
    with pytest.raises(plbm.Exception, match="f16c"):
        plbm.create_handler(props, precision="f16c")


_STEADY = {}


def _steady_state(plbm, precision, target, cap):
    """Momentum of the 1024x256 porous channel (seed 12345, porosity 0.7, tau 0.6, rho 1.01/1.0)
    run to `target` (or `cap` steps) in `precision`; fluid nodes only."""
    w, h = 1024, 256
    mask = plbm.porous_disks(w, h, 12345, 0.7)
    props = plbm.Properties("nptl", "stream", False, 1024, 10 ** 9, 10 ** 9, "Hagen-Poiseuille", h, w, 0.0, 0.0,
                            1.01, 0.0, 0.0, 1.0, 0.6)
    hd = plbm.create_handler(props, precision=precision, mask=mask)
    steps, r = hd.run_to_residual(target, 100, cap)
    fl = mask.reshape(-1) == 0
    j = np.concatenate([hd.get_x_velocities()[fl], hd.get_y_velocities()[fl]])
    rho = hd.get_densities()[fl]
    hd.close()
    return j, rho, steps, r


@pytest.mark.parametrize("precision,bar", [("f16s", 1e-3), ("f16c", 5e-4), ("f32", 1e-4)])
def test_shifted_steady_state_against_converged_fp64(plbm, precision, bar):
    """The steady state of each storage form against the FP64 steady state: f64_q60 (<= 1e-12 from
    the drop-in) converged to residual 1e-9 is the reference; each form runs towards residual 1e-9
    as well, at most 60 000 steps (the 16-bit forms stop at their rounding plateau, ~1e-6; a run
    stopped at residual 1e-6 would still be ~2e-3 from its steady state).  FP16 must meet the 1e-3
    velocity bar, F16C (one more significand bit) half of it."""
    if "ref" not in _STEADY:
        _STEADY["ref"] = _steady_state(plbm, "f64_q60", 1e-9, 80000)
    jr, rr, n, r = _STEADY["ref"]
    assert r < 1e-9, (n, r)
    j, rho, _, _ = _steady_state(plbm, precision, 1e-9, 60000)
    l2 = float(np.linalg.norm(j - jr) / np.linalg.norm(jr))
    mass = abs(float(rho.sum() - rr.sum()) / float(rr.sum()))
    assert l2 <= bar, l2
    assert mass <= 1e-4, mass


@pytest.mark.parametrize("alg,lay", [("nptl", "stream"), ("lptl", "bundle"), ("npol", "collision"), ("nsol", "stream")])
def test_set_precision_continues_the_state_exactly(plbm, alg, lay):
    """f16s -> f32 re-encodes each stored deviation exactly (the FP16 form's values carry 2^12), and
    the FP16 form computes on scaled values with the same FP32 operations, so the step after the
    switch writes the same observables as one more FP16 step; f32 -> f16s -> f32 then continues."""
    w, h = 157, 53
    mask = plbm.porous_disks(w, h, 4, 0.7)
    props = plbm.Properties(alg, lay, False, 64, 10 ** 6, 10 ** 6, "Hagen-Poiseuille", h, w, 0.0, 0.0, 1.02, 0.0, 0.0,
                            1.0, 0.6)
    a = plbm.create_handler(props, precision="f16s", mask=mask)
    b = plbm.create_handler(props, precision="f16s", mask=mask)
    a.run_steps(301)
    b.run_steps(300)
    b.set_precision("f32")
    assert b.bytes_per_node() == 72.0
    b.run_steps(1)
    for get in ("get_densities", "get_x_velocities", "get_y_velocities"):
        assert np.array_equal(getattr(a, get)(), getattr(b, get)()), get
    b.set_precision("f16s")
    b.set_precision("f32")
    b.run_steps(200)
    assert np.all(np.isfinite(b.get_densities()))
    a.close()
    b.close()


def test_set_precision_rejects_forms_outside_the_shifted_ones(plbm):
    props = plbm.Properties("nptl", "stream", False, 64, 10, 10, "circle", 30, 62, 0.0, 0.0, 1.05, 0.0, 0.0, 1.0, 0.6)
    hd = plbm.create_handler(props, precision="f64_q60")
    with pytest.raises(plbm.Exception, match="shifted forms"):
        hd.set_precision("f32")
    hd.close()
    hd = plbm.create_handler(props, precision="f32")
    with pytest.raises(plbm.Exception, match="shifted forms"):
        hd.set_precision("f64_strict")
    hd.set_precision("f32")   # the same form: nothing to do
    hd.close()


def test_escalating_run_reaches_the_target_a_16_bit_form_stalls_above(plbm):
    """f16s stalls at its rounding floor above residual 1e-6 on this porous channel; finished in
    FP32 after the stall the same run reaches 1e-6.  Run on towards the steady state, it stays
    within 2e-3 (relative L2 of j) of the converged FP64 state: the 16-bit rounding left in the slow
    modes decays only over a long FP32 run (a run stopped at residual 1e-6 is itself ~2e-3 from
    the steady state), so this bar, not FP32's 3.5e-5, is what the switch guarantees."""
    w, h = 256, 64
    mask = plbm.porous_disks(w, h, 12345, 0.7)
    props = plbm.Properties("nptl", "stream", False, 1024, 10 ** 9, 10 ** 9, "Hagen-Poiseuille", h, w, 0.0, 0.0,
                            1.01, 0.0, 0.0, 1.0, 0.6)
    hd = plbm.create_handler(props, precision="f16s", mask=mask)
    n, r, switched = hd.run_to_residual_escalating(1e-6, 100, 200000)
    assert r < 1e-6 and switched is not None and switched < n, (n, r, switched)
    hd.run_to_residual(1e-9, 100, 200000)
    got = np.concatenate([hd.get_x_velocities(), hd.get_y_velocities()])
    hd.close()
    ref_h = plbm.create_handler(props, precision="f64_q60", mask=mask)
    ref_h.run_to_residual(1e-9, 100, 400000)
    ref = np.concatenate([ref_h.get_x_velocities(), ref_h.get_y_velocities()])
    ref_h.close()
    fl = np.concatenate([mask.reshape(-1) == 0] * 2)
    assert np.linalg.norm(got[fl] - ref[fl]) / np.linalg.norm(ref[fl]) < 2e-3

"""Parity of every algorithm x data layout at the FP64 sweep's 2000x500 size, against the oracle.

The workload is the sweep's circle channel: walls on the first and last inner rows, a disk of
radius floor(H/8) centred at (floor(W/4), floor(H/2)), inlet density 1.2, outlet 1.0, zero
boundary velocities, work-group size 1024 (the reference's default), relaxation times 0.55, 0.6
and 1.0.  Every GPU run is compared with the oracle's run of the same algorithm
(include/lbm/gpu/nptl/nptl_kernels.hpp:371-437 and its lptl/npol/nsol twins):

* f64_strict must be identical (1000 steps, every relaxation time);
* f64_fast (fused multiply-adds) and f64_q60 (64-bit fixed point) must agree within the drop-in
  tolerance, max |difference| <= 1e-12 in rho, jx and jy: after 1000 steps at tau 0.6 and 1.0,
  and after 200 steps at tau 0.55.

At tau 0.55 this channel amplifies rounding differences by about 10^4 every 250 steps: the
reference's own arithmetic compiled with fused multiply-adds (a legal compilation that rounds
differently) departs from its uncontracted build by ~1e-13 after 250 steps and ~1e-1 after 1000
(test_tau_055_amplifies_the_references_own_rounding).  Past that point only bit-identical
arithmetic can agree, which f64_strict is.

The oracle's values do not depend on the data layout (the golden cases pin all twelve
algorithm x layout variants to the reference bit for bit), so one oracle run per algorithm and
relaxation time serves the three layouts.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 2000, 500
TAUS = (0.55, 0.6, 1.0)
ALGS = ("nptl", "lptl", "npol", "nsol")
LAYOUTS = ("stream", "collision", "bundle")
TOL = {"f64_strict": 0.0, "f64_fast": 1e-12, "f64_q60": 1e-12}


def steps_for(tau, precision):
    return 200 if (tau == 0.55 and precision != "f64_strict") else 1000


def circle_channel_mask(w, h):
    yy, xx = np.mgrid[0:h, 0:w]
    r = h // 8
    m = ((xx - w // 4) ** 2 + (yy - h // 2) ** 2 <= r * r).astype(np.int8)
    m[0, :] = 1
    m[h - 1, :] = 1
    return m


MASK = circle_channel_mask(W, H)
_ORACLE = {}


def oracle_fields(oracle_mod, alg, tau, steps, precision="f64"):
    key = (alg, tau, steps, precision)
    if key not in _ORACLE:
        o = oracle_mod.Oracle(alg, "stream", 1024, "Hagen-Poiseuille", W, H, inlet_density=1.2,
                              relaxation_time=tau, mask=MASK, precision=precision)
        o.run(steps)
        _ORACLE[key] = {k: o.result(i) for i, k in enumerate(("rho", "jx", "jy"))}
    return _ORACLE[key]


def gpu_fields(plbm, alg, lay, tau, precision, steps):
    props = plbm.Properties(alg, lay, False, 1024, steps, steps, "Hagen-Poiseuille", H, W, 0.0, 0.0, 1.2, 0.0, 0.0,
                            1.0, tau)
    hd = plbm.create_handler(props, precision=precision, mask=MASK)
    hd.start()
    hd.block_until_finished()
    out = {"rho": hd.get_densities(), "jx": hd.get_x_velocities(), "jy": hd.get_y_velocities()}
    hd.close()
    return out


def maxdiff(a, b):
    return max(float(np.max(np.abs(a[k] - b[k]))) for k in b)


@pytest.mark.parametrize("precision", ["f64_strict", "f64_fast", "f64_q60"])
@pytest.mark.parametrize("tau", TAUS)
@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("lay", LAYOUTS)
def test_sweep_variant_matches_oracle(plbm, oracle_mod, alg, lay, tau, precision):
    steps = steps_for(tau, precision)
    ref = oracle_fields(oracle_mod, alg, tau, steps)
    got = gpu_fields(plbm, alg, lay, tau, precision, steps)
    err = maxdiff(got, ref)
    assert err <= TOL[precision], f"{alg}/{lay} tau {tau} {precision} {steps} steps: max abs {err:.3e}"
    # the run did something: the disk deflects the flow, so jy is nonzero somewhere
    assert float(np.max(np.abs(got["jy"]))) > 1e-6


def test_tau_055_amplifies_the_references_own_rounding(plbm, oracle_mod):
    """The oracle compiled with fused multiply-adds departs from the uncontracted oracle by far more
    than 1e-12 after 1000 steps at tau 0.55, while at tau 0.6 both builds agree to ~1e-13: the
    configuration, not the GPU arithmetic, limits non-bit-identical parity there.  The FP64-accuracy
    forms stay within a few times the reference's own spread."""
    strict = oracle_fields(oracle_mod, "nptl", 0.55, 1000)
    contracted = oracle_fields(oracle_mod, "nptl", 0.55, 1000, precision="f64_contracted")
    spread = maxdiff(contracted, strict)
    assert spread > 1e-9, spread
    calm = maxdiff(oracle_fields(oracle_mod, "nptl", 0.6, 1000, precision="f64_contracted"),
                   oracle_fields(oracle_mod, "nptl", 0.6, 1000))
    assert calm <= 1e-12, calm
    for precision in ("f64_fast", "f64_q60"):
        got = gpu_fields(plbm, "nptl", "stream", 0.55, precision, 1000)
        assert np.all(np.isfinite(got["jx"]))
        assert maxdiff(got, strict) <= 100 * spread, precision

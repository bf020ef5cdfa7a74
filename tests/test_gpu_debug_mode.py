"""debugMode: the reference's NPTLDebug / LPTLDebug drivers run the step as three kernels
(StreamKernel, MacroscopicObservablesKernel, CollideKernel; include/lbm/gpu/nptl/nptl_kernels.hpp:
49-295, include/lbm/gpu/lptl/lptl_kernels.hpp:51-278) instead of the fused StreamCollideKernel.
The unfused step gives the same results as the fused one, bit for bit, in the drop-in form and in
the USE_FLOAT form, and equals the oracle; npol / nsol keep the fused step in debug mode, as the
reference's NPOLDebug / NSOLDebug do."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(plbm, alg, lay, debug, precision, steps=250, fui=None, w=70, h=33, scenario="circle", tau=0.6, rho_in=1.05):
    props = plbm.Properties(alg, lay, debug, 64, steps, fui or steps, scenario, h, w, 0.0, 0.0, rho_in, 0.0, 0.0, 1.0,
                            tau)
    hd = plbm.create_handler(props, precision=precision)
    launches = hd.launches_per_step()
    hd.start()
    hd.block_until_finished()
    out = {"rho": hd.get_densities(), "jx": hd.get_x_velocities(), "jy": hd.get_y_velocities(),
           "jabs": hd.get_absolute_velocities()}
    hd.close()
    return out, launches


@pytest.mark.parametrize("precision", ["f64_strict", "f32_ref"])
@pytest.mark.parametrize("lay", ["stream", "collision", "bundle"])
@pytest.mark.parametrize("alg", ["nptl", "lptl"])
def test_unfused_debug_step_equals_fused_step(plbm, alg, lay, precision):
    fused, n_fused = run(plbm, alg, lay, False, precision)
    dbg, n_dbg = run(plbm, alg, lay, True, precision)
    assert n_fused == 1 and n_dbg == 3
    for k in fused:
        assert np.array_equal(fused[k], dbg[k]), k


@pytest.mark.parametrize("alg", ["nptl", "lptl"])
def test_debug_step_matches_oracle_with_frames(plbm, oracle_mod, alg):
    """Frame steps every 7 iterations (no frame graphs in debug mode), square obstacle, tau 0.55."""
    got, _ = run(plbm, alg, "bundle", True, "f64_strict", steps=300, fui=7, scenario="square", tau=0.55)
    o = oracle_mod.Oracle(alg, "bundle", 64, "square", 70, 33, inlet_density=1.05, relaxation_time=0.55)
    o.run(300)
    ref = o.results()
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k


@pytest.mark.parametrize("alg", ["npol", "nsol"])
def test_one_lattice_debug_mode_keeps_the_fused_step(plbm, alg):
    fused, _ = run(plbm, alg, "stream", False, "f64_strict")
    dbg, n = run(plbm, alg, "stream", True, "f64_strict")
    assert n == 1
    for k in fused:
        assert np.array_equal(fused[k], dbg[k]), k


def test_debug_mode_needs_a_literal_form(plbm):
    props = plbm.Properties("nptl", "stream", True, 64, 10, 10, "circle", 30, 62, 0.0, 0.0, 1.05, 0.0, 0.0, 1.0, 0.6)
    with pytest.raises(plbm.Exception, match="debugMode"):
        plbm.create_handler(props, precision="f64_q60")

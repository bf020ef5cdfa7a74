"""The CPU oracle (oracle/plbm_oracle.c) against golden vectors produced by the reference's own
code (tests/golden/make_golden.py runs the reference's algorithm classes): every case must match
exactly, including core::Domain.  This pins the oracle that the GPU parity tests rely on."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "cases.json")))


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(HERE, "golden", "golden.npz"))


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference_golden(oracle_mod, golden, case):
    o = oracle_mod.Oracle(case["algorithm"], case["data_layout"], case["work_group_size"], case["scenario"],
                          case["w"], case["h"], inlet_density=case["inlet_density"],
                          relaxation_time=case["relaxation_time"], outlet_density=case["outlet_density"],
                          precision=case["precision"])
    assert list(o.domain().values()) == case["domain"]
    o.run(case["steps"])
    res = o.results()
    for k in ("rho", "jx", "jy", "jabs"):
        ref = golden[f"{case['name']}__{k}"]
        assert np.array_equal(res[k], ref), f"{k}: max abs {np.max(np.abs(res[k] - ref))}"


def test_glibc_rand_sequence(oracle_mod):
    """porous_medium_mask (domain_initialization.hpp:277-278) draws from glibc's rand(); the
    restated generator reproduces its published sequence from seed 1."""
    lib = oracle_mod.load()
    lib.plbmo_rand_reset(1)
    assert [lib.plbmo_rand() for _ in range(5)] == [1804289383, 846930886, 1681692777, 1714636915, 1957747793]


def test_reference_regression_profile(golden):
    """tests/test_regression.cpp:121-181 of the reference, applied to its own output (golden):
    positive interior velocities, mirror symmetry < 1 % of u_max, peak at the centre row +-1,
    u_max / u_mean in (1.35, 1.55)."""
    w, h = 30, 14
    jx = golden["reference_regression__jx"].reshape(h, w)
    prof = jx[:, w // 2]
    fluid = prof[1:h - 1]
    assert np.all(fluid > 0)
    umax = fluid.max()
    for i in range(1, h // 2 + 1):
        assert abs(prof[i] - prof[h - 1 - i]) / umax < 0.01
    peak = int(np.argmax(fluid)) + 1
    assert (1 + h - 2) // 2 - 1 <= peak <= (1 + h - 2) // 2 + 1
    assert 1.35 < umax / fluid.mean() < 1.55


def test_reference_smoke_properties(golden):
    """tests/smoke_test.cpp:82-95 of the reference: finite, mean rho > 0.5, some |jx| > 1e-12."""
    rho, jx = golden["reference_smoke__rho"], golden["reference_smoke__jx"]
    assert np.all(np.isfinite(rho)) and np.all(np.isfinite(jx))
    assert rho.mean() > 0.5
    assert np.any(np.abs(jx) > 1e-12)


def test_all_variants_agree(golden):
    """All four algorithms and three layouts compute the same physics (no buffered-outlet case)."""
    base = golden["variant_nptl_stream__jx"]
    for alg in ("nptl", "lptl", "npol", "nsol"):
        for lay in ("collision", "stream", "bundle"):
            assert np.array_equal(golden[f"variant_{alg}_{lay}__jx"], base)


def test_nn_reference_adjoints():
    """The CPU conv reference is self-consistent: <conv(x), g> = <x, dgrad(g)> = <w, wgrad(x, g)>."""
    from oracle import nn_ref
    rng = np.random.default_rng(0)
    x, w, g = rng.standard_normal((2, 5, 6, 3)), rng.standard_normal((4, 27)), rng.standard_normal((2, 5, 6, 4))
    a = (nn_ref.conv_fwd(x, w) * g).sum()
    assert np.isclose(a, (x * nn_ref.conv_dgrad(g, w, 3)).sum())
    assert np.isclose(a, (w * nn_ref.conv_wgrad(x, g)[0]).sum())

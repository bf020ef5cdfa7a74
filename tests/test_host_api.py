"""Host-side logic of libplbm without a GPU: Properties validation (reference messages),
settings.json I/O, core::Domain arithmetic, scenario geometry, the exported C ABI, and the
failure mode when no GPU is present (no CPU fallback)."""
import json
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available


def P(plbm, alg="lptl", lay="stream", wg=64, steps=100, fui=100, sc="Hagen-Poiseuille", v=30, h=126,
      rho_in=1.3, rho_out=1.0, tau=0.6):
    return plbm.Properties(alg, lay, False, wg, steps, fui, sc, v, h, 0.0, 0.0, rho_in, 0.0, 0.0, rho_out, tau)


def test_library_exports_every_declared_symbol(plbm):
    lib = plbm.load_library()
    names = set()
    for hdr in os.listdir(os.path.join(ROOT, "include")):
        if hdr.endswith(".h"):
            text = open(os.path.join(ROOT, "include", hdr)).read()
            names |= set(re.findall(r"\b(plbm_[a-z0-9_]+)\s*\(", text))
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_constants_match_the_header(plbm):
    text = open(os.path.join(ROOT, "include", "plbm_c.h")).read()
    consts = {k: int(v, 0) for k, v in re.findall(r"\b(PLBM_[A-Z0-9_]+)\s*=\s*(0x[0-9a-fA-F]+|\d+)", text)}
    consts.update({k: int(v, 0) for k, v in re.findall(r"#define\s+(PLBM_[A-Z0-9_]+)\s+(0x[0-9a-fA-F]+|\d+)", text)})
    for name, code in plbm.PRECISIONS.items():
        assert consts["PLBM_" + name.upper()] == code, name
    for name, code in plbm.BATCH_MODES.items():
        assert consts["PLBM_BATCH_" + name.upper()] == code, name
    assert consts["PLBM_BATCH_TILE_VEC"] == plbm.BATCH_TILE_VEC
    for name, code in plbm.GATHER.items():
        assert consts["PLBM_GATHER_" + name.upper()] == code, name


def test_properties_ghost_accounting(plbm):
    """Properties ctor adds two ghost layers (simulation.cpp:45-48; test_properties.cpp:44-71)."""
    p = P(plbm, v=30, h=126)
    assert p.vertical_nodes == 32 and p.horizontal_nodes == 128
    assert p.total_unexpanded_node_count == 32 * 128 and p.domain_node_count == 30 * 126


@pytest.mark.parametrize("kw,msg", [
    (dict(v=1), "vertical_nodes must be >= 4"),
    (dict(h=1), "horizontal_nodes must be >= 4"),
    (dict(steps=0), "time_steps must be >= 1"),
    (dict(fui=0), "frame_update_interval must be >= 1"),
    (dict(wg=0), "work_group_size must be >= 1"),
    (dict(rho_in=0.0), "inlet_density must be > 0"),
    (dict(rho_out=-1.0), "outlet_density must be > 0"),
    (dict(tau=0.0), "relaxation_time must be > 0"),
    (dict(alg="xyz"), 'Unknown algorithm: "xyz"'),
    (dict(lay="soa"), 'Unknown data_layout: "soa"'),
    (dict(sc="cube"), 'Unknown scenario: "cube"'),
])
def test_validate_rejects(plbm, kw, msg):
    with pytest.raises(plbm.PropertyArgumentException, match=re.escape(msg)):
        P(plbm, **kw).validate()


def test_validate_accepts_large_frame_interval(plbm):
    P(plbm, steps=10000, fui=10001).validate()
    for alg in ("nptl", "lptl", "npol", "nsol"):
        for lay in ("collision", "stream", "bundle"):
            P(plbm, alg=alg, lay=lay).validate()


def _settings(path, **over):
    d = {"algorithmic": {"algorithm": "lptl", "dataLayout": "bundle", "debugMode": False, "frameUpdateInterval": 10,
                         "timeSteps": 1000000, "workGroupSize": 1024},
         "domain": {"horizontalNodes": 512, "verticalNodes": 128, "scenario": "circle"},
         "physical": {"inletDensity": 1.2, "inletVelocity": {"x": 0.0, "y": 0.0}, "outletDensity": 1.0,
                      "outletVelocity": {"x": 0.0, "y": 0.0}, "relaxationTime": 0.6}}
    for k, v in over.items():
        sec, key = k.split(".")
        d[sec][key] = v
    with open(path, "w") as f:
        json.dump(d, f, indent=4)


def test_json_to_properties(plbm, tmp_path):
    """json_to_properties (file_interaction.cpp:39-69): inner counts + offset, ghosts added."""
    path = str(tmp_path / "settings.json")
    _settings(path)
    p = plbm.json_to_properties(path)
    assert (p.algorithm, p.data_layout, p.scenario, p.work_group_size) == ("lptl", "bundle", "circle", 1024)
    assert (p.vertical_nodes, p.horizontal_nodes, p.frame_update_interval) == (130, 514, 10)
    assert p.settings_path == path
    q = plbm.json_to_properties(path, -2)
    assert (q.vertical_nodes, q.horizontal_nodes) == (128, 512)


def test_json_round_trip(plbm, tmp_path):
    path = str(tmp_path / "rt.json")
    p = P(plbm, alg="nsol", lay="collision", wg=256, sc="wing", v=77, h=301, tau=0.73)
    plbm.properties_to_json(p, path)
    q = plbm.json_to_properties(path)
    for k in ("algorithm", "data_layout", "work_group_size", "scenario", "vertical_nodes", "horizontal_nodes",
              "relaxation_time", "inlet_density", "time_steps", "frame_update_interval"):
        assert getattr(p, k) == getattr(q, k), k


def test_json_missing_key_and_bad_file(plbm, tmp_path):
    path = str(tmp_path / "bad.json")
    with open(path, "w") as f:
        f.write('{"algorithmic": {"algorithm": "nptl"}}')
    with pytest.raises(plbm.ParseException, match="not found"):
        plbm.json_to_properties(path)
    with open(path, "w") as f:
        f.write('{"algorithmic": ')
    with pytest.raises(plbm.ParseException):
        plbm.json_to_properties(path)
    with pytest.raises(plbm.ParseException):
        plbm.json_to_properties(str(tmp_path / "absent.json"))


def test_domain_reference_expectations(plbm):
    """tests/test_domain.cpp:40-160 of the reference."""
    d = plbm.compute_domain(P(plbm, alg="lptl", v=10, h=6, wg=64))
    assert (d["vertical_nodes"], d["horizontal_nodes"], d["total_node_count"]) == (12, 8, 96)
    assert (d["subdomain_count_vertical"], d["subdomain_count_horizontal"]) == (1, 1)
    assert (d["subdomain_vertical_nodes"], d["subdomain_horizontal_nodes"]) == (12, 8)
    d = plbm.compute_domain(P(plbm, alg="nptl", v=10, h=10, wg=4))
    assert d["subdomain_horizontal_nodes"] == 2 and d["subdomain_vertical_nodes"] == 2
    assert d["horizontal_nodes"] >= 12 and d["vertical_nodes"] >= 12
    d = plbm.compute_domain(P(plbm, alg="nptl", v=10, h=10, wg=8))
    assert d["subdomain_horizontal_nodes"] * d["subdomain_vertical_nodes"] == 8
    d = plbm.compute_domain(P(plbm, alg="nptl", v=10, h=10, wg=7))
    assert (d["subdomain_vertical_nodes"], d["subdomain_horizontal_nodes"]) == (1, 7)
    d = plbm.compute_domain(P(plbm, alg="npol", v=10, h=10, wg=4))
    assert d["subdomain_horizontal_nodes"] * d["subdomain_vertical_nodes"] == 4
    d = plbm.compute_domain(P(plbm, alg="npol", v=20, h=20, wg=16))
    assert (d["subdomain_horizontal_nodes"], d["subdomain_vertical_nodes"]) == (4, 4)
    for alg, v, h, wg in (("nsol", 10, 10, 8), ("nsol", 30, 30, 64)):
        d = plbm.compute_domain(P(plbm, alg=alg, v=v, h=h, wg=wg))
        assert d["total_node_count"] == d["horizontal_nodes"] * d["vertical_nodes"]
    with pytest.raises(plbm.PropertyArgumentException):
        plbm.compute_domain(P(plbm, alg="nsol", wg=4))


@pytest.mark.parametrize("alg", ["nptl", "lptl", "npol", "nsol"])
def test_domain_matches_oracle_sweep(plbm, oracle_mod, alg):
    """core::Domain for many work-group sizes (incl. the power-of-4 test's quirks, e.g. 20 and 80)
    equals the restated reference arithmetic."""
    for wg in (6, 7, 8, 12, 16, 20, 24, 48, 64, 80, 96, 100, 128, 255, 256, 512, 1000, 1024):
        for w, h in ((62, 30), (400, 100), (33, 17)):
            ref = oracle_mod.domain_for(alg, wg, w, h)
            if ref is None:   # nsol with 2x2 tiles: the reference would divide by zero
                with pytest.raises(plbm.PropertyArgumentException):
                    plbm.compute_domain(P(plbm, alg=alg, wg=wg, v=h, h=w))
                continue
            got = plbm.compute_domain(P(plbm, alg=alg, wg=wg, v=h, h=w))
            assert got == ref, (alg, wg, w, h)


@pytest.mark.parametrize("sc", ["Hagen-Poiseuille", "walls", "circle", "square", "plate", "skyscraper", "wing",
                                "porous"])
def test_flags_match_oracle(plbm, oracle_mod, sc):
    import ctypes
    w, h = 90, 48
    libc = ctypes.CDLL(None)
    libc.srand(1)   # the reference's porous mask reads the process-wide rand() sequence
    flags = plbm.make_flags(P(plbm, alg="lptl", sc=sc, v=h, h=w))
    o = oracle_mod.Oracle("lptl", "stream", 64, sc, w, h)
    of = o.flags().reshape(h + 2, w + 2)[1:h + 1, 1:w + 1]
    assert np.array_equal(flags, of)


@pytest.mark.skipif(gpu_available(), reason="checks the failure mode without a GPU")
def test_invalid_gather_option_is_rejected_before_any_device_work(plbm):
    import ctypes
    lib = plbm.load_library()
    opts = plbm._COpts()
    lib.plbm_default_options(ctypes.byref(opts))
    assert opts.gather == plbm.GATHER["auto"]
    opts.gather = 7
    c = P(plbm)._c()
    out = ctypes.c_void_p()
    rc = lib.plbm_create(ctypes.byref(c), ctypes.byref(opts), ctypes.byref(out))
    assert rc == -7 and not out.value   # PLBM_ERR_ARGUMENT
    assert "gather" in lib.plbm_last_error(None).decode()


@pytest.mark.skipif(gpu_available(), reason="checks the failure mode without a GPU")
def test_create_without_gpu_fails_loudly(plbm):
    with pytest.raises(plbm.NoDeviceException):
        plbm.create_handler(P(plbm))


@pytest.mark.skipif(gpu_available(), reason="checks the failure mode without a GPU")
def test_batch_without_gpu_fails_loudly(plbm):
    dom = {"mask": plbm.porous_disks(64, 32, 1, 0.8), "relaxation_time": 0.6, "inlet_density": 1.01}
    with pytest.raises(plbm.NoDeviceException):
        plbm.Batch([dom], precision="f16s")
    with pytest.raises(plbm.Exception, match="no domains"):
        plbm.Batch([], precision="f32")


def test_porous_disks_generator(plbm):
    m = plbm.porous_disks(300, 120, 5, 0.7)
    assert m.shape == (120, 300)
    assert np.all(m[0] == 1) and np.all(m[-1] == 1)
    assert abs((1 - m[1:-1].mean()) - 0.7) < 0.01
    assert np.array_equal(m, plbm.porous_disks(300, 120, 5, 0.7))      # seeded
    assert not np.array_equal(m, plbm.porous_disks(300, 120, 6, 0.7))


def test_checked_build_loads_and_exports_the_same_symbols(plbm):
    """libplbm_checked.so (PLBM_CHECKED) builds from the same sources, exports every entry point of
    libplbm.so and says which build it is; loading it needs no GPU."""
    import ctypes
    import subprocess
    from portlbm_gb300 import build as b
    lib = ctypes.CDLL(b.build(checked=True))
    lib.plbm_version.restype = ctypes.c_char_p
    assert b"checked" in lib.plbm_version()
    out = subprocess.run(["nm", "-D", "--defined-only", b.LIB_CHECKED], capture_output=True, text=True).stdout
    ref = subprocess.run(["nm", "-D", "--defined-only", b.LIB], capture_output=True, text=True).stdout
    names = lambda t: {ln.split()[-1] for ln in t.splitlines() if " T plbm_" in ln}  # noqa: E731
    assert names(ref) and names(ref) == names(out)

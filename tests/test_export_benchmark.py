"""Headless frame export and the benchmark driver (the reference's GUI frames and
src/lbm/benchmark/benchmark.cpp).  The CPU tests cover the .npy writer, the work-group sweep and
the driver's error path; the GPU tests run a handler with export on and a small benchmark."""
import glob
import json
import os

import numpy as np
import pytest
from conftest import gpu_available


def _which_power_of_4(x):
    # core::power_functions::which_power_of_4 (include/lbm/core/simulation.hpp), restated
    if x & 1 or x == 0:
        return 0
    p = 0
    while not x & 3:
        x >>= 2
        p += 1
    return 0 if x & 2 else p


def _which_power_of_2(x):
    if x & 1 or x == 0:
        return 0
    p = 0
    while not x & 1:
        x >>= 1
        p += 1
    return 0 if x >> 1 else p


def _reference_work_group_sizes(max_wg):
    """Benchmark::get_work_group_sizes (src/lbm/benchmark/benchmark.cpp:30-62), restated."""
    out = []
    for i in (4, 3, 2, 1):
        region = i * max_wg // 4
        even = odd = False
        for j in range(4):
            size = region - j
            if _which_power_of_4(size) or _which_power_of_2(size):
                out.append(size)
            elif size % 2 == 0 and not even:
                out.append(size)
                even = True
            elif size % 2 and not odd:
                out.append(size)
                odd = True
    return out


@pytest.mark.parametrize("max_wg", [1024, 512, 256, 1000, 64])
def test_benchmark_work_group_sizes(plbm, max_wg):
    assert plbm.benchmark_work_group_sizes(max_wg) == _reference_work_group_sizes(max_wg)
    if max_wg == 1024:
        assert plbm.benchmark_work_group_sizes(1024) == [1024, 1023, 1022, 768, 767, 512, 511, 510, 256, 255, 254]


@pytest.mark.parametrize("shape", [(1, 1), (7, 13), (30, 62), (3, 1000)])
def test_write_npy_round_trip(plbm, tmp_path, shape):
    a = np.random.default_rng(1).standard_normal(shape)
    a[0, 0] = -0.0
    path = tmp_path / "f.npy"
    plbm.write_npy(path, a)
    raw = path.read_bytes()
    assert raw[:8] == b"\x93NUMPY\x01\x00"
    header_len = raw[8] | raw[9] << 8
    assert (10 + header_len) % 64 == 0 and len(raw) == 10 + header_len + 8 * a.size
    b = np.load(path)
    assert b.dtype == np.float64 and b.shape == shape
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))   # bit-exact, including -0.0


def _project(tmp_path, plbm, w=64, h=32, steps=40, wg=64):
    """A project tree like the reference's: <root>/settings/{settings,benchmark}.json."""
    (tmp_path / "settings").mkdir()
    p = plbm.Properties("nptl", "stream", False, wg, steps, steps, "Hagen-Poiseuille", h, w, 0.0, 0.0, 1.05, 0.0, 0.0,
                        1.0, 0.7)
    settings = tmp_path / "settings" / "settings.json"
    plbm.properties_to_json(p, str(settings))
    # the driver reads node counts with offset -2, as the reference's Benchmark does
    d = json.loads(settings.read_text())
    d["domain"]["verticalNodes"] += 2
    d["domain"]["horizontalNodes"] += 2
    settings.write_text(json.dumps(d, indent=4))
    (tmp_path / "settings" / "benchmark.json").write_text(json.dumps({
        "testRunsPerConfig": 1, "testLinearTwoLattice": True, "dataLayouts": ["stream", "collision"],
        "algorithms": ["nptl", "nsol"], "phaseTwoScenarios": ["plate", "porous"]}, indent=4))
    return settings


@pytest.mark.skipif(gpu_available(), reason="checks the failure mode without a GPU")
def test_benchmark_without_gpu_reports_no_device(plbm, tmp_path):
    settings = _project(tmp_path, plbm)
    with pytest.raises(plbm.NoDeviceException):
        plbm.run_benchmark(settings)


@pytest.mark.gpu
def test_frame_export_writes_the_frame_results(plbm, tmp_path):
    props = plbm.Properties("nptl", "stream", False, 64, 100, 40, "circle", 30, 62, 0.0, 0.0, 1.05, 0.0, 0.0, 1.0, 0.6)
    hd = plbm.create_handler(props, precision="f64_strict")
    hd.set_frame_export(tmp_path / "frames", ("rho", "jx"))
    hd.start()
    hd.block_until_finished()
    files = sorted(os.path.basename(f) for f in glob.glob(str(tmp_path / "frames" / "*.npy")))
    assert files == [f"frame_{it:09d}_{f}.npy" for it in (40, 80, 100) for f in ("jx", "rho")]
    rho = np.load(tmp_path / "frames" / "frame_000000100_rho.npy")
    jx = np.load(tmp_path / "frames" / "frame_000000100_jx.npy")
    assert rho.shape == (30, 62)
    assert np.array_equal(rho.reshape(-1), hd.get_densities())
    assert np.array_equal(jx.reshape(-1), hd.get_x_velocities())
    early = np.load(tmp_path / "frames" / "frame_000000040_jx.npy")
    assert not np.array_equal(early, jx)            # frames are the states of their own steps
    hd.set_frame_export(None)
    hd.close()


@pytest.mark.gpu
def test_benchmark_driver_writes_the_reference_files(plbm, tmp_path):
    settings = _project(tmp_path, plbm)
    plbm.run_benchmark(settings, precision="f64_q60", hbm_gbs=6800.0)
    wgs = plbm.benchmark_work_group_sizes(1024)
    for phase in (0, 1):
        for alg in ("nptl", "nsol"):
            (f,) = glob.glob(str(tmp_path / "benchmarks" / f"phase{phase}" / f"results_phase{phase}_{alg}_*.json"))
            d = json.loads(open(f).read())
            assert d["algorithm"] == alg and d["verticalNodes"] == 34 and d["horizontalNodes"] == 66
            for lay in ("stream", "collision"):
                assert [e["workGroupSize"] for e in d[lay]] == wgs
                for e in d[lay]:
                    assert len(e["runtimes"]) == len(e["initializationTimes"]) == len(e["mlups"]) == 1
                    assert e["runtimes"][0] > 0 and e["mlups"][0] > 0 and 0 < e["hbmFraction"][0] < 2
        (f,) = glob.glob(str(tmp_path / "benchmarks" / f"phase{phase}" / f"results_phase{phase}_lptl_*.json"))
        d = json.loads(open(f).read())
        assert d["algorithm"] == "lptl" and d["stream"][0]["workGroupSize"] == "auto"
    for alg in ("nptl", "nsol", "lptl"):
        for scn in ("plate", "porous"):
            (f,) = glob.glob(str(tmp_path / "benchmarks" / "phase2" / f"phase2_{alg}_{scn}_*.json"))
            d = json.loads(open(f).read())
            assert d["scenario"] == scn and d["dataLayout"] in ("stream", "collision")
            assert (d["workGroupSize"] == "auto") == (alg == "lptl")
            if alg != "lptl":
                assert d["workGroupSize"] in wgs          # the phase-1 choice
            assert len(d["runtimes"]) == 1 and d["mlups"][0] > 0

"""Host-side pieces of bench.py that need no GPU: the clock record keeps only the samples taken
while the timed steps ran."""
import datetime
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _line(t, sm, reasons=("Not Active",) * 4):
    ts = datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    return ", ".join([ts, str(sm), "2070", "900.5", "0x0000000000000000", *reasons])


def test_clock_summary_keeps_the_timed_window():
    c = bench.ClockSampler(0)
    t0 = 1_790_000_000.0
    # set-up at low clock, timed steps at full clock, a throttle flag only during set-up
    c.lines = ([_line(t0 + 0.1 * k, 1000, ("Active", "Not Active", "Not Active", "Not Active")) for k in range(10)]
               + [_line(t0 + 1.0 + 0.1 * k, 1995 + k) for k in range(8)] + ["garbage line"])
    whole = c.summary()
    assert whole["samples"] == 18 and whole["reasons"] == ["hw_slowdown"]
    timed = c.summary((t0 + 0.95, t0 + 1.75))
    assert timed["samples"] == 8 and timed["reasons"] == [] and timed["sm_mhz"] == 1998.5
    assert timed["sm_max_mhz"] == 2070 and timed["window_s"] == 0.8
    # a window shorter than the sampling interval takes its neighbours within 0.3 s
    short = c.summary((t0 + 1.72, t0 + 1.74))
    assert short["samples"] == 3 and short["reasons"] == []


def test_reference_arm_samples_a_band_when_the_run_would_be_long(capsys):
    """The reference arm (the CPU oracle) keeps each step a bounded sample: with a run that would
    exceed its time budget it steps a centred band of the channel and says so in `sample`."""
    import argparse
    import json
    args = argparse.Namespace(width=256, height=160, steps=3, warmup=1, algorithm="nptl", layout="stream",
                              precision="f64_q60")
    bench.run_reference(args, 1, 0, budget_s=1e-6)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 3 and line["value"] > 0
    assert "band" in line["cpu_baseline"]["sample"] and "256x64" in line["cpu_baseline"]["sample"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
    bench.run_reference(args, 1, 0, budget_s=1e6)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["cpu_baseline"]["sample"].startswith("3 full 256x160 timesteps")
    # the reference arm reports the same config as the measured arm
    assert line["config"] == bench.line_config(args, 1) and line["metric"] == bench.METRIC


def test_clock_summary_from_nvml_samples():
    """The NVML sampler's (time, MHz, max MHz, reason bits) samples go through the same window and
    reason names as nvidia-smi's lines: bit 0x4 is sw_power_cap, 0x8 hw_slowdown."""
    c = bench.ClockSampler(0)
    t0 = 1_790_000_000.0
    c.nvml_samples = [(t0 + 0.001 * k, 2070.0, 2070.0, 0x4 if k == 5 else 0x1) for k in range(40)]
    s = c.summary((t0 + 0.0005, t0 + 0.0305))
    assert s["samples"] == 30 and s["sm_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"]
    c.nvml_samples.append((t0 + 0.02, 1500.0, 2070.0, 0x8))
    assert "hw_slowdown" in c.summary((t0, t0 + 0.05))["reasons"]


def test_batch_tile_argument_and_sampler_period():
    """--batch-tile W,THREADS_Y,ROWS,BLOCKS[,vec] becomes Batch.set_tile's (tile_w, tile_h, blocks)
    with the rows in tile_h's second byte and the vectorised-rows flag above; the clock sampler
    queries every millisecond until relax() slows it after the device-timed steps."""
    class Lib:
        BATCH_TILE_VEC = 0x10000
    assert bench.parse_batch_tile("32,4,2,4,vec", Lib) == (32, 4 + 256 * 2 + 0x10000, 4)
    assert bench.parse_batch_tile("32,8,4,16", Lib) == (32, 8 + 256 * 4, 16)
    c = bench.ClockSampler(0)
    assert c.period_s == 0.001
    c.relax()
    assert c.period_s == 0.05

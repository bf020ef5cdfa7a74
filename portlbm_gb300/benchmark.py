"""Command line for the benchmark driver (the reference's ``main_gpu --benchmark``,
src/main_gpu.cpp:160-174, src/lbm/benchmark/benchmark.cpp).

    python -m portlbm_gb300.benchmark settings/settings.json [--precision f64_q60] [--phases 0 1 2]

Reads settings/benchmark.json next to the settings file (or --benchmark-json) and writes
benchmarks/phase<N>/*.json under the project root (or --output-root), in the reference's shape
with per-run MLUPS and, given --hbm-gbs, the fraction of that copy bandwidth.
"""
from __future__ import annotations

import argparse
import json
import os

from . import PRECISIONS, run_benchmark


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("settings")
    ap.add_argument("--benchmark-json", default=None)
    ap.add_argument("--output-root", default=None)
    ap.add_argument("--precision", default="f64_strict", choices=list(PRECISIONS))
    ap.add_argument("--phases", type=int, nargs="+", default=[0, 1, 2])
    ap.add_argument("--hbm-gbs", type=float, default=None,
                    help="copy bandwidth for hbmFraction (default: MEASURED_PEAKS.json beside the package, if any)")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    hbm = a.hbm_gbs
    if hbm is None:
        peaks = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")
        try:
            with open(peaks) as f:
                hbm = float(json.load(f)["hbm_gbs"])
        except (OSError, KeyError, ValueError):
            hbm = 0.0
    run_benchmark(a.settings, a.benchmark_json, a.output_root, a.precision, a.phases, hbm, a.device)


if __name__ == "__main__":
    main()

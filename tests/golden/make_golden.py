"""Generates tests/golden/*.npz from the reference's own code (oracle/_ref, built from the
reference tree by oracle/build_ref.py).  Run in the development container, naming the tree:

    PORTLBM_REFERENCE=<reference tree> python tests/golden/make_golden.py

Each case records the reference's rho, jx, jy, |j| after N steps (float64; the USE_FLOAT build's
values converted exactly) and its core::Domain.  cases.json lists the parameters.  The cases cover
every algorithm x data layout, the buffered-outlet configurations, all eight scenarios (porous
with the glibc rand() sequence from seed 1), the reference's own smoke and regression test
configurations, the 400x100 Hagen-Poiseuille parity configuration (10^4 steps), tau variants,
and the USE_FLOAT build.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import reference  # noqa: E402


def cases():
    out = []
    for alg in ("nptl", "lptl", "npol", "nsol"):
        for lay in ("collision", "stream", "bundle"):
            out.append(dict(name=f"variant_{alg}_{lay}", algorithm=alg, data_layout=lay,
                            work_group_size=64 if alg == "nsol" else 16, scenario="circle", w=40, h=24, steps=100,
                            inlet_density=1.05, relaxation_time=0.6))
    for alg, w, wg in (("npol", 65, 64), ("nsol", 61, 64), ("npol", 33, 16), ("nsol", 33, 16)):
        out.append(dict(name=f"bufferedoutlet_{alg}_{w}_{wg}", algorithm=alg, data_layout="stream",
                        work_group_size=wg, scenario="Hagen-Poiseuille", w=w, h=20, steps=300, inlet_density=1.05,
                        relaxation_time=0.6))
    for sc in ("Hagen-Poiseuille", "walls", "circle", "square", "plate", "skyscraper", "wing", "porous"):
        out.append(dict(name=f"scenario_{sc}", algorithm="nptl", data_layout="stream", work_group_size=64,
                        scenario=sc, w=90, h=48, steps=200, inlet_density=1.05, relaxation_time=0.6))
    for tau in (0.55, 1.0):
        out.append(dict(name=f"tau_{tau}", algorithm="nptl", data_layout="stream", work_group_size=1024,
                        scenario="circle", w=62, h=30, steps=300, inlet_density=1.2, relaxation_time=tau))
    # tests/smoke_test.cpp:46-63 and tests/test_regression.cpp:71-88 of the reference
    out.append(dict(name="reference_smoke", algorithm="lptl", data_layout="stream", work_group_size=64,
                    scenario="Hagen-Poiseuille", w=126, h=30, steps=100, inlet_density=1.3, relaxation_time=0.6))
    out.append(dict(name="reference_regression", algorithm="lptl", data_layout="stream", work_group_size=16,
                    scenario="Hagen-Poiseuille", w=30, h=14, steps=8000, inlet_density=1.01, relaxation_time=1.0))
    out.append(dict(name="poiseuille_400x100_10k", algorithm="nptl", data_layout="stream", work_group_size=1024,
                    scenario="Hagen-Poiseuille", w=400, h=100, steps=10000, inlet_density=1.2, relaxation_time=0.6))
    for alg in ("nptl", "lptl", "npol", "nsol"):
        out.append(dict(name=f"usefloat_{alg}", algorithm=alg, data_layout="stream",
                        work_group_size=64 if alg == "nsol" else 16, scenario="circle", w=40, h=24, steps=200,
                        inlet_density=1.05, relaxation_time=0.6, precision="f32"))
    return out


def main():
    arrays, index = {}, []
    for c in cases():
        prec = c.get("precision", "f64")
        r = reference.run(c["algorithm"], c["data_layout"], c["work_group_size"], c["scenario"], c["w"], c["h"],
                          c["steps"], inlet_density=c["inlet_density"], relaxation_time=c["relaxation_time"],
                          precision=prec)
        for k in ("rho", "jx", "jy", "jabs"):
            arrays[f"{c['name']}__{k}"] = r[k]
        c = dict(c, precision=prec, domain=r["domain"], outlet_density=1.0, rand_seed=1)
        index.append(c)
        print(c["name"], "done", flush=True)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(index, f, indent=1)


if __name__ == "__main__":
    main()

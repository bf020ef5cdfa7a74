"""Recipe that compiles the reference's own sources into oracle/_ref/ — TEST INFRASTRUCTURE.

The reference (SC-SGS/PortLBM) needs AdaptiveCpp (SYCL), LLVM and nlohmann/json/fmt, none of which
exist here; its kernels and drivers are header-only SYCL functors, so they are compiled unchanged,
from their place in the reference tree, against the host SYCL subset in oracle/ref_shim:

    include/lbm/**                         (kernels, drivers, core)
    src/lbm/core/simulation.cpp            (Properties, Domain, Simulation)
    src/lbm/exceptions/exceptions.cpp
    src/lbm/core/timer.cpp

plus oracle/ref_driver.cpp (a C entry point).  Outputs go to oracle/_ref/ only (git-ignored):
libplbm_ref.so (real_type = double, WITH_NAN_PROTECTION as the CMake default) and
libplbm_ref_f32.so (USE_FLOAT).  Needs the reference tree, so it runs in the development
container only; the GPU host uses the committed fixtures in tests/golden instead.

The reference tree's location has no default: pass it to build(root) or set PORTLBM_REFERENCE
(`PORTLBM_REFERENCE=<tree> python -m oracle.build_ref`).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SOURCES = ["src/lbm/core/simulation.cpp", "src/lbm/exceptions/exceptions.cpp", "src/lbm/core/timer.cpp"]


def reference_root(root: str | None = None) -> str | None:
    """The reference tree: `root`, else $PORTLBM_REFERENCE, else None."""
    return root or os.environ.get("PORTLBM_REFERENCE") or None


def available(root: str | None = None) -> bool:
    ref = reference_root(root)
    return bool(ref) and os.path.isdir(os.path.join(ref, "include", "lbm"))


def lib_path(precision: str = "f64") -> str:
    return os.path.join(OUT, "libplbm_ref.so" if precision == "f64" else "libplbm_ref_f32.so")


def build(root: str | None = None, force: bool = False) -> bool:
    """Compiles oracle/_ref from the reference tree at `root` (or $PORTLBM_REFERENCE); False when
    no tree is given or it is absent."""
    if not available(root):
        return False
    REF = reference_root(root)
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "ref_shim", "sycl", "sycl.hpp")]
    for prec, extra in (("f64", []), ("f32", ["-DUSE_FLOAT"])):
        out = lib_path(prec)
        if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
            continue
        cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               "-DWITH_NAN_PROTECTION", *extra, "-I", os.path.join(HERE, "ref_shim"), "-I", os.path.join(REF, "include"),
               "-o", out + ".tmp", os.path.join(HERE, "ref_driver.cpp"), *[os.path.join(REF, s) for s in SOURCES]]
        subprocess.run(cmd, check=True)
        os.replace(out + ".tmp", out)
    return True


if __name__ == "__main__":
    print("built" if build(force="--force" in sys.argv) else "reference tree not given or not available "
                                                             "(set PORTLBM_REFERENCE)")

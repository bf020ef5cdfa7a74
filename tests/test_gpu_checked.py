"""The bounds-checked build (PLBM_CHECKED): every lattice, link, result, jy-column and halo index
of the step kernels is compared with its buffer's extent; an index outside it is skipped and the
host reports PLBM_ERR_CUDA after the steps.  This runs the batch tests (the persistent tile queue,
vectorised rows, every precision and mode), the vectorised-row and gather tests, the exact parity
of every algorithm x layout and the debug-mode tests against libplbm_checked.so in a child process
(the library is chosen when the package loads it), so a passing run means no kernel index left its
buffer on those workloads."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SELECTION = ("batch or vectorised or strict_matches_oracle_exactly or gather_forms or buffered_outlet or "
             "unfused or one_lattice")


def test_checked_build_runs_the_kernel_tests_without_out_of_range_accesses():
    from portlbm_gb300 import build as b
    b.build(checked=True)
    env = dict(os.environ, PLBM_CHECKED="1")
    probe = subprocess.run([sys.executable, "-c", "import portlbm_gb300 as p; print(p.load_library().plbm_version()"
                                                  ".decode())"], cwd=ROOT, env=env, capture_output=True, text=True)
    assert probe.returncode == 0 and "checked" in probe.stdout, probe.stdout + probe.stderr
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
                        os.path.join("tests", "test_gpu_parity.py"), os.path.join("tests", "test_gpu_debug_mode.py"),
                        "-k", SELECTION], cwd=ROOT, env=env, capture_output=True, text=True, timeout=1500)
    tail = "\n".join((r.stdout + r.stderr).splitlines()[-30:])
    assert r.returncode == 0, tail
    assert " passed" in tail, tail

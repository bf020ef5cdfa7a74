"""The C++ drop-in header (include/portlbm_gb300.hpp): compiles against libplbm.so on any host;
on a GPU its test program runs the reference's smoke and regression checks through it."""
import os
import subprocess

import pytest

from conftest import ROOT


def _compile(tmp_path):
    exe = str(tmp_path / "api_test")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "api_test.cpp"), "-o", exe,
           "-L", os.path.join(ROOT, "portlbm_gb300"), "-lplbm", "-Wl,-rpath," + os.path.join(ROOT, "portlbm_gb300")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_header_compiles_and_links(plbm, tmp_path):
    _compile(tmp_path)


@pytest.mark.gpu
def test_cpp_reference_style_checks(plbm, tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr

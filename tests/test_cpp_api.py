"""The C++ drop-in header (include/portlbm_gb300.hpp): compiles against libplbm.so on any host;
core::Domain(Properties&) matches the oracle's domain arithmetic without a GPU; on a GPU its test
program runs the reference's smoke and regression checks and the AlgorithmHandler interface
(get_properties, get_domain) through it."""
import os
import subprocess

import pytest

from conftest import ROOT


def _compile(tmp_path, name="api_test"):
    exe = str(tmp_path / name)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-o", exe,
           "-L", os.path.join(ROOT, "portlbm_gb300"), "-lplbm", "-Wl,-rpath," + os.path.join(ROOT, "portlbm_gb300")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_header_compiles_and_links(plbm, tmp_path):
    _compile(tmp_path)


@pytest.mark.parametrize("w,h,wg", [(91, 37, 64), (400, 100, 1024), (126, 30, 16), (2000, 500, 1024), (33, 20, 8)])
def test_cpp_domain_matches_oracle(plbm, oracle_mod, tmp_path, w, h, wg):
    exe = _compile(tmp_path, "domain_test")
    r = subprocess.run([exe, str(w), str(h), str(wg)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    keys = ("total_node_count", "horizontal_nodes", "vertical_nodes", "subdomain_vertical_nodes",
            "subdomain_horizontal_nodes", "subdomain_count_vertical", "subdomain_count_horizontal")
    for line in r.stdout.splitlines():
        alg, *vals = line.split()
        want = oracle_mod.domain_for(alg, wg, w, h)
        assert dict(zip(keys, map(int, vals))) == want, alg


@pytest.mark.gpu
def test_cpp_reference_style_checks(plbm, tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr

"""Host-side logic without a GPU: the miniFE.x driver's parameter scan (the
reference's parse_parameter semantics, ref/utils/param_utils.hpp:116-155, and
defaults of ref/utils/utils.cpp:66-68), the C++ shim header compiling against
reference-style code, and the committed reference YAML key tree."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "minife_gb300", "miniFE.x")


@pytest.fixture(scope="module")
def driver():
    from minife_gb300 import build
    build.build()
    return DRIVER


def params(driver, *args, cwd=None):
    out = subprocess.run([driver, *args, "print_params=1"], capture_output=True, text=True,
                         check=True, cwd=cwd).stdout
    d = {}
    for line in out.splitlines():
        k, _, v = line.partition(" ")
        d[k] = v
    return d


def test_defaults(driver):
    p = params(driver)
    assert (p["nx"], p["ny"], p["nz"]) == ("10", "10", "10")
    assert p["max_iters"] == "200" and p["precision"] == "f64"


def test_ny_nz_default_to_previous(driver):
    p = params(driver, "nx=7")
    assert (p["nx"], p["ny"], p["nz"]) == ("7", "7", "7")
    p = params(driver, "nx=7", "ny=5")
    assert (p["nx"], p["ny"], p["nz"]) == ("7", "5", "5")


@pytest.mark.parametrize("form", [["nx=12"], ["-nx", "12"], ["nx:12"], ["nx", "12"], ["nx", "=", "12"]])
def test_separators(driver, form):
    assert params(driver, *form)["nx"] == "12"


def test_input_file(driver, tmp_path):
    f = tmp_path / "params.yaml"
    f.write_text("nx: 9\nny: 8\nnz: 7\nverify_solution: 1\n")
    p = params(driver, "input_file=%s" % f)
    assert (p["nx"], p["ny"], p["nz"], p["verify_solution"]) == ("9", "8", "7", "1")


def test_gb300_keys(driver):
    p = params(driver, "precision=mixed", "rel_tol=1e-8", "max_iters=5000", "refine_k=30")
    assert p["precision"] == "mixed" and float(p["rel_tol"]) == 1e-8
    assert p["max_iters"] == "5000" and p["refine_k"] == "30"
    assert float(p["inner_tol"]) == 0.0 and p["max_refine"] == "0"  # library defaults
    p = params(driver, "precision=mixed", "inner_tol=1e-3", "max_refine=4")
    assert float(p["inner_tol"]) == 1e-3 and p["max_refine"] == "4"


def test_zero_equations_exit(driver):
    r = subprocess.run([driver, "nx=0"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "0 equations" in r.stdout


def test_shim_header_compiles(tmp_path):
    src = os.path.join(ROOT, "tests", "cpp", "shim_solve.cpp")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_reference_yaml_keys_fixture():
    keys = open(os.path.join(ROOT, "tests", "golden", "ref_yaml_keys.txt")).read().split()
    assert "0:Matrix" in " ".join(keys) or any(k.startswith("0:Matrix") for k in keys)
    assert len(keys) > 40

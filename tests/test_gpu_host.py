"""GPU tests of the host-side drop-in: miniFE.x (the reference's CLI, phases
and YAML report) and the C++ shim header (reference types and signatures)."""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "minife_gb300", "miniFE.x")


def yaml_keys(path):
    keys = []
    for line in open(path):
        if ":" not in line:
            continue
        indent = len(line) - len(line.lstrip(" "))
        keys.append("%d:%s" % (indent, line.strip().split(":")[0]))
    return keys


def yaml_value(path, key):
    for line in open(path):
        if line.strip().startswith(key + ":"):
            return line.split(":", 1)[1].strip()
    return None


def run_driver(tmp_path, *args):
    from minife_gb300 import build
    build.build()
    r = subprocess.run([DRIVER, *args], cwd=tmp_path, capture_output=True, text=True)
    ymls = [f for f in os.listdir(tmp_path) if f.endswith(".yaml")]
    return r, (os.path.join(tmp_path, ymls[0]) if ymls else None)


def test_minife_x_reference_run(tmp_path):
    """./miniFE.x nx=10 verify_solution=1 (ref/src/run_test:3): exit 0, the
    reference's YAML key tree, iterations and residual like the reference."""
    r, yml = run_driver(tmp_path, "nx=10", "verify_solution=1")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "solution matches analytic solution" in r.stdout
    ref = open(os.path.join(ROOT, "tests", "golden", "ref_yaml_keys.txt")).read().split("\n")
    ref = [k for k in ref if k]
    ours = yaml_keys(yml)
    missing = [k for k in ref if k not in ours]
    assert not missing, missing
    assert os.path.basename(yml).startswith("miniFE.10x10x10.")
    it = int(yaml_value(yml, "Iterations"))
    assert abs(it - 31) <= 2  # reference: 31 iterations (tests/golden, 10x10x10)
    assert float(yaml_value(yml, "Final Resid Norm")) < 1e-14
    assert int(yaml_value(yml, "Global NNZ")) == 29791


def test_minife_x_ell_matrix(tmp_path):
    """./miniFE.x nx=10 verify_solution=1 matrix=ell against the reference
    built with MINIFE_ELL_MATRIX (tests/golden/ref_ell_nx10.json, written by
    that build): the same key tree, the ELL's padded nonzeros (27 per row) in
    Matrix attributes and in the matvec flop count, the reference's
    iterations and an absolute DBL_EPSILON stop, the analytic check passed.
    Then kernels=1 times the ELL matvec."""
    import json
    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "ref_ell_nx10.json")))
    r, yml = run_driver(tmp_path, "nx=10", "verify_solution=1", "matrix=ell")
    assert r.returncode == 0, r.stdout + r.stderr
    assert ref["verified"] and "solution matches analytic solution" in r.stdout
    keys = [k for k in open(os.path.join(ROOT, "tests", "golden", "ref_yaml_keys.txt")).read().split("\n") if k]
    missing = [k for k in keys if k not in yaml_keys(yml)]
    assert not missing, missing
    for k in ("Global Nrows", "Global NNZ", "NNZ per proc MAX"):
        assert yaml_value(yml, k) == ref["Matrix attributes/" + k], k
    assert abs(float(yaml_value(yml, "Global Memory (GB)")) -
               float(ref["Matrix attributes/Global Memory (GB)"])) <= 1e-9
    it = int(yaml_value(yml, "Iterations"))
    assert abs(it - int(ref["CG solve/Iterations"])) <= 1
    assert float(yaml_value(yml, "Final Resid Norm")) <= 2.220446049250313e-16
    # the report prints six significant digits
    assert abs(float(yaml_value(yml, "MATVEC Flops")) / (35937 * 2.0 * (it + 1)) - 1) <= 1e-5
    assert yaml_value(yml, "matrix") == "ELL"
    kdir = tmp_path / "kernels"
    kdir.mkdir()
    r2, yml2 = run_driver(kdir, "nx=10", "matrix=ell", "kernels=1")
    assert r2.returncode == 0, r2.stdout + r2.stderr
    assert abs(float(yaml_value(yml2, "MATVEC Flops")) / (35937 * 2.0 * 500) - 1) <= 1e-5


def test_minife_x_mixed_relative(tmp_path):
    r, yml = run_driver(tmp_path, "-nx", "24", "-ny", "20", "-nz", "16", "precision=mixed",
                        "rel_tol=1e-8", "max_iters=3000", "verify_solution=1", "name=mx")
    assert r.returncode == 0, r.stdout + r.stderr
    assert os.path.basename(yml).startswith("miniFE.24x20x16.mx.")
    true_res = float(yaml_value(yml, "True Final Resid Norm"))
    r0 = float(yaml_value(yml, "Initial Resid Norm"))
    assert true_res <= 1e-8 * r0
    assert yaml_value(yml, "inner operator") == "FP32 stencil (verified)"


def test_minife_x_kernel_timing_mode(tmp_path):
    """kernels=1: the reference's MINIFE_KERNELS loops (time_kernels.hpp):
    500 of each operation with x = 0.9 e_0, so every dot is p.A p = 0.81 A_00
    (row 0 is a Dirichlet row: A_00 = 1) and the reported norm is their sum."""
    r, yml = run_driver(tmp_path, "nx=12", "ny=10", "nz=8", "kernels=1")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Starting kernel timing loops" in r.stdout
    keys = yaml_keys(yml)
    for k in ("0:Kernel timings", "2:Iterations", "2:WAXPY Time", "2:DOT Time",
              "2:MATVEC Time", "2:MATVEC Mflops"):
        assert k in keys, k
    assert "0:CG solve" not in keys
    assert int(yaml_value(yml, "Iterations")) == 500
    assert abs(float(yaml_value(yml, "Final Resid Norm")) - 500 * (0.9 * 0.9)) <= 1e-9
    nnz = int(yaml_value(yml, "Global NNZ"))
    assert float(yaml_value(yml, "MATVEC Flops")) == 2.0 * nnz * 500


def test_minife_x_dump_files_match_reference(tmp_path):
    """dump=1 writes the reference's MINIFE_DEBUG files; for the 2x3x2 box the
    system files are byte-identical to the ones the reference wrote
    (tests/golden/dumps_2x3x2) and x agrees to the printed digits."""
    r, yml = run_driver(tmp_path, "nx=2", "ny=3", "nz=2", "dump=1")
    assert r.returncode == 0, r.stdout + r.stderr
    ref = os.path.join(ROOT, "tests", "golden", "dumps_2x3x2")
    for name in ("A_prebc.mtx", "b_prebc.vec", "A.mtx", "b.vec"):
        ours = open(os.path.join(tmp_path, name + ".1.0")).read()
        assert ours == open(os.path.join(ref, name + ".1.0")).read(), name
    assert open(os.path.join(tmp_path, "A_local.mtx.1.0")).read() == \
        open(os.path.join(ref, "A.mtx.1.0")).read()
    xo = [float(l.split()[1]) for l in open(os.path.join(ref, "x.vec.1.0")).read().splitlines()[1:]]
    xs = [float(l.split()[1]) for l in open(os.path.join(tmp_path, "x.vec.1.0")).read().splitlines()[1:]]
    assert np.allclose(xs, xo, rtol=1e-5, atol=1e-12)


def test_cpp_shim_dump_files(tmp_path):
    """The shim's write_matrix / write_vector on the 2x3x2 box after both
    Dirichlet passes: byte for byte the files the reference itself wrote
    (tests/golden/dumps_2x3x2).  The ELLMatrix's file is the same rows under
    the header the reference's ELL build writes, its padded nonzero count
    (36 rows x 27)."""
    exe = os.path.join(tmp_path, "shim_solve")
    from minife_gb300 import build
    build.build()
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "shim_solve.cpp"), "-L",
                    os.path.join(ROOT, "minife_gb300"), "-lminife_gb300",
                    "-Wl,-rpath," + os.path.join(ROOT, "minife_gb300"), "-o", exe], check=True)
    subprocess.run([exe, "2", "3", "2", "dump"], cwd=tmp_path, capture_output=True, text=True,
                   check=True)
    gold = os.path.join(ROOT, "tests", "golden", "dumps_2x3x2")
    for name in ("A.mtx.1.0", "b.vec.1.0"):
        assert open(os.path.join(tmp_path, name), "rb").read() == \
            open(os.path.join(gold, name), "rb").read(), name
    ell = open(os.path.join(tmp_path, "A_ell.mtx.1.0")).read().split("\n")
    csr = open(os.path.join(gold, "A.mtx.1.0")).read().split("\n")
    assert ell[0] == "36 %d" % (36 * 27)
    assert ell[1:] == csr[1:]


def test_cpp_shim_matches_oracle(tmp_path):
    exe = os.path.join(tmp_path, "shim_solve")
    from minife_gb300 import build
    build.build()
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "shim_solve.cpp"), "-L",
                    os.path.join(ROOT, "minife_gb300"), "-lminife_gb300",
                    "-Wl,-rpath," + os.path.join(ROOT, "minife_gb300"), "-o", exe], check=True)
    out = subprocess.run([exe, "10", "9", "8"], capture_output=True, text=True, check=True).stdout
    v = {k: float(x) for k, x in (ln.split() for ln in out.splitlines())}
    ro, cols, vals, b = O.build_system(10, 9, 8)
    s = 0.0
    for a in vals:  # same summation order as the shim program
        s += a
    assert v["vals_sum"] == s
    # the mesh's Dirichlet sets (faces x=0, y=0, z=0, y=1, z=1; face x=1)
    Nx, Ny, Nz = 11, 10, 9
    n0 = sum(1 for iz in range(Nz) for iy in range(Ny) for ix in range(Nx)
             if ix == 0 or iy == 0 or iz == 0 or iy == Ny - 1 or iz == Nz - 1)
    assert int(v["bc_rows_0"]) == n0 and int(v["bc_rows_1"]) == Ny * Nz
    xw = 1.0 / (1.0 + np.arange(ro.size - 1))
    yw = O.matvec(ro, cols, vals, xw)
    assert v["fused_waxpby_diff"] == 0.0
    w2 = 1.5 * yw + 0.25 * xw
    assert abs(v["fused_waxpby_sum2"] - w2 @ w2) <= 1e-12 * (w2 @ w2)
    x = 1.0 / (1.0 + np.arange(ro.size - 1))
    y = O.matvec(ro, cols, vals, x)
    assert abs(v["matvec_dot"] - O.dot(x, y)) <= 1e-13 * abs(O.dot(np.abs(x), np.abs(y)))
    xo, it, nr, st = O.cg_solve(ro, cols, vals, b)
    assert abs(int(v["num_iters"]) - it) <= 2
    assert abs(v["x_sum"] - xo.sum()) <= 1e-11 * np.abs(xo).sum()
    # the ELLMatrix run: rows (padding left out) and b bit for bit the CSR's,
    # the same matvec (the padding adds exact zeros), the CG of the
    # reference's ELL build within one iteration and rounding of the CSR's
    assert int(v["ell_same_as_csr"]) == 1
    assert v["ell_matvec_diff"] == 0.0
    assert abs(int(v["ell_num_iters"]) - int(v["num_iters"])) <= 1
    assert v["ell_normr"] <= 2.220446049250313e-16
    assert v["ell_x_rel_diff"] <= 1e-12

"""Generate the golden fixtures that pin the oracle to the reference.

Run with REF set to a miniFE checkout (the directory holding ref/src), after
`make -C oracle ref REF=...`, which compiles the unmodified reference sources
(ref/ variant) with oracle/ref_harness.cpp into oracle/_ref/ref_harness.
Writes:

  tests/golden/minife_golden.npz   full arrays for small boxes
  tests/golden/golden_hashes.json  sha256 of every array for larger boxes

With --ell it only writes tests/golden/ref_ell_nx10.json (also written by the
full run): the report of the reference built with MINIFE_ELL_MATRIX at
nx=10 (oracle/_ref/miniFE_ell.x).

With --big N (run separately: the serial reference takes about 7 minutes at
N = 256) it instead runs the N^3 box to a 1e-8 relative residual and writes
  tests/golden/golden_<N>.json     sha256 of every array, iteration count,
                                   final residual, analytic check, ||x||
  tests/golden/x<N>_strided.npy    x[::997] (the solution, sampled)
--workdir DIR keeps the harness's raw outputs there and reuses them when a
run with the same arguments already left them (DIR/args.txt).

The legacy unit test's known-answer element matrix (ref/basic/utest_cases.hpp,
get_test_elem_mat) is read from the reference source as text and stored too.
The GPU machine never runs this script; tests only read its outputs.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("REF", "")
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
EPS = 2.220446049250313e-16

FULL_CASES = [  # (nx, ny, nz, max_iter, tol_mode, tol)
    (1, 1, 2, 200, 0, EPS),
    (2, 2, 2, 200, 0, EPS),
    (4, 5, 6, 200, 0, EPS),
    (17, 3, 5, 200, 0, EPS),
    (10, 10, 10, 200, 0, EPS),
    (10, 10, 10, 200, 1, 1e-8),
    (7, 9, 4, 200, 1, 1e-8),
]
HASH_CASES = [
    (20, 30, 40, 200, 0, EPS),
    (30, 30, 30, 200, 0, EPS),
    (30, 30, 30, 200, 1, 1e-8),
    (24, 16, 8, 200, 1, 1e-8),
]
ARRAYS = [("row_offsets", "i32", np.int32), ("cols", "i32", np.int32),
          ("vals_prebc", "f64", np.float64), ("b_prebc", "f64", np.float64),
          ("vals", "f64", np.float64), ("b", "f64", np.float64), ("x", "f64", np.float64)]


def run_case(case, tmp):
    nx, ny, nz, mi, mode, tol = case
    d = os.path.join(tmp, "c_%d_%d_%d_%d" % (nx, ny, nz, mode))
    os.makedirs(d, exist_ok=True)
    subprocess.run([HARNESS, str(nx), str(ny), str(nz), str(mi), str(mode), repr(tol), d],
                   check=True, capture_output=True)
    arrs = {name: np.fromfile(os.path.join(d, "%s.%s" % (name, ext)), dt)
            for name, ext, dt in ARRAYS}
    meta = {}
    for line in open(os.path.join(d, "meta.txt")):
        k, v = line.split()
        meta[k] = float(v) if "." in v or "e" in v else int(v)
    return arrs, meta


def key(case):
    nx, ny, nz, mi, mode, tol = case
    return "%dx%dx%d_mode%d" % (nx, ny, nz, mode)


def utest_known_answer():
    path = os.path.join(REF, "ref", "basic", "utest_cases.hpp")
    text = open(path).read()
    body = text[text.index("void get_test_elem_mat"):]
    body = body[: body.index("}")]
    vals = np.zeros(36)
    for idx, val in re.findall(r"elem_mat\[(\d+)\]\s*=\s*([-0-9.e]+);", body):
        vals[int(idx)] = float(val)
    return vals


X_STRIDE = 997


def big_case(n, workdir=None):
    """The N^3 box to 1e-8 relative (max 2000 iterations): hashes and a
    strided sample of the solution."""
    case = (n, n, n, 2000, 1, 1e-8)
    args = [str(v) for v in case[:5]] + [repr(case[5])]
    own = workdir is None
    d = workdir or tempfile.mkdtemp()
    os.makedirs(d, exist_ok=True)
    stamp = os.path.join(d, "args.txt")
    if not (os.path.exists(stamp) and open(stamp).read().split() == args and
            os.path.exists(os.path.join(d, "meta.txt"))):
        subprocess.run([HARNESS, *args, d], check=True)
        with open(stamp, "w") as f:
            f.write(" ".join(args) + "\n")
    meta = {}
    for line in open(os.path.join(d, "meta.txt")):
        k, v = line.split()
        meta[k] = float(v) if "." in v or "e" in v else int(v)
    out = {"dims": [n, n, n], "max_iter": case[3], "tol_mode": 1, "tol": case[5],
           "num_iters": meta["num_iters"], "normr": meta["normr"], "abs_tol": meta["abs_tol"],
           "verify": meta["verify"], "nrows": meta["nrows"], "nnz": meta["nnz"],
           "x_stride": X_STRIDE, "sha256": {}}
    for name, ext, dt in ARRAYS:
        a = np.fromfile(os.path.join(d, "%s.%s" % (name, ext)), dt)
        out["sha256"][name] = hashlib.sha256(a.tobytes()).hexdigest()
        if name == "x":
            out["x_l2"] = float(np.linalg.norm(a))
            np.save(os.path.join(HERE, "x%d_strided.npy" % n), a[::X_STRIDE].copy())
        del a
    with open(os.path.join(HERE, "golden_%d.json" % n), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    if own:
        shutil.rmtree(d)
    print("wrote golden_%d.json and x%d_strided.npy (%d iterations)" % (n, n, meta["num_iters"]))


def ell_report():
    """The reference built with MINIFE_ELL_MATRIX (oracle/_ref/miniFE_ell.x)
    at nx=10 with verify_solution=1: the report's values that the ELL layout
    changes or must keep (Matrix attributes, the CG's iterations and final
    residual, the flop counts) and its verification line, to
    tests/golden/ref_ell_nx10.json."""
    exe = os.path.join(ROOT, "oracle", "_ref", "miniFE_ell.x")
    if not os.path.exists(exe):
        sys.exit("build the reference first: make -C oracle ref REF=$REF")
    with tempfile.TemporaryDirectory() as tmp:
        run = subprocess.run([exe, "nx=10", "verify_solution=1"], cwd=tmp, capture_output=True,
                             text=True, check=True)
        yml = [f for f in os.listdir(tmp) if f.endswith(".yaml")][0]
        section, vals = None, {}
        for line in open(os.path.join(tmp, yml)):
            if ":" not in line:
                continue
            indent = len(line) - len(line.lstrip(" "))
            key, _, val = line.strip().partition(":")
            if indent == 0:
                section = key
            elif section in ("Matrix attributes", "CG solve") and indent == 2 and val.strip():
                vals["%s/%s" % (section, key)] = val.strip()
    keep = ["Matrix attributes/Global Nrows", "Matrix attributes/Global NNZ",
            "Matrix attributes/Global Memory (GB)", "Matrix attributes/NNZ per proc MAX",
            "CG solve/Iterations", "CG solve/Final Resid Norm", "CG solve/MATVEC Flops",
            "CG solve/DOT Flops", "CG solve/WAXPY Flops"]
    out = {k: vals[k] for k in keep}
    out["verified"] = "solution matches analytic solution" in run.stdout
    with open(os.path.join(HERE, "ref_ell_nx10.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote ref_ell_nx10.json")


def main():
    if "--ell" in sys.argv:
        return ell_report()
    if "--big" in sys.argv:
        if not os.path.exists(HARNESS):
            sys.exit("build the reference harness first: make -C oracle ref REF=$REF")
        n = int(sys.argv[sys.argv.index("--big") + 1])
        wd = sys.argv[sys.argv.index("--workdir") + 1] if "--workdir" in sys.argv else None
        return big_case(n, wd)
    if not REF or not os.path.isdir(os.path.join(REF, "ref", "src")):
        sys.exit("set REF to the miniFE checkout (the directory holding ref/src)")
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: make -C oracle ref REF=$REF")
    out = {}
    hashes = {}
    with tempfile.TemporaryDirectory() as tmp:
        for case in FULL_CASES:
            arrs, meta = run_case(case, tmp)
            k = key(case)
            for name, arr in arrs.items():
                out["%s/%s" % (k, name)] = arr
            out["%s/meta" % k] = np.array([meta["num_iters"], meta["normr"], meta["verify"],
                                           meta["abs_tol"], case[3], case[4], case[5]])
        for case in HASH_CASES:
            arrs, meta = run_case(case, tmp)
            hashes[key(case)] = {
                "dims": list(case[:3]), "max_iter": case[3], "tol_mode": case[4], "tol": case[5],
                "num_iters": meta["num_iters"], "normr": meta["normr"], "verify": meta["verify"],
                "nrows": meta["nrows"], "nnz": meta["nnz"],
                "sha256": {n: hashlib.sha256(a.tobytes()).hexdigest() for n, a in arrs.items()},
                "x_l2": float(np.linalg.norm(arrs["x"])),
            }
        d = os.path.join(tmp, "elem")
        os.makedirs(d)
        subprocess.run([HARNESS, "element", d], check=True)
        out["element/ref_elem_mat"] = np.fromfile(os.path.join(d, "elem_mat.f64"), np.float64)
        out["element/ref_elem_vec"] = np.fromfile(os.path.join(d, "elem_vec.f64"), np.float64)
        out["element/ref_grad_vals"] = np.fromfile(os.path.join(d, "grad_vals.f64"), np.float64)
    out["element/utest_elem_mat"] = utest_known_answer()
    # the reference's own YAML report (oracle/_ref/miniFE.x nx=10
    # verify_solution=1): its key tree, one "indent:key" line per entry
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(ROOT, "oracle", "_ref", "miniFE.x")
        run = subprocess.run([exe, "nx=10", "verify_solution=1"], cwd=tmp, capture_output=True,
                             text=True, check=True)
        yml = [f for f in os.listdir(tmp) if f.endswith(".yaml")][0]
        keys = []
        for line in open(os.path.join(tmp, yml)):
            if ":" not in line:
                continue
            indent = len(line) - len(line.lstrip(" "))
            keys.append("%d:%s" % (indent, line.strip().split(":")[0]))
        with open(os.path.join(HERE, "ref_yaml_keys.txt"), "w") as f:
            f.write("\n".join(keys) + "\n")
        with open(os.path.join(HERE, "ref_stdout_nx10.txt"), "w") as f:
            f.write(run.stdout)
    # the reference's own MINIFE_DEBUG dump files (write_matrix /
    # write_vector) for the 2x3x2 box, reference defaults
    ddir = os.path.join(HERE, "dumps_2x3x2")
    os.makedirs(ddir, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([HARNESS, "2", "3", "2", "200", "0", repr(2.220446049250313e-16), tmp,
                        "dump"], cwd=tmp, check=True)
        for name in ("A_prebc.mtx", "b_prebc.vec", "A.mtx", "b.vec", "x.vec"):
            shutil.copy(os.path.join(tmp, name + ".1.0"), os.path.join(ddir, name + ".1.0"))
    ell_report()
    np.savez_compressed(os.path.join(HERE, "minife_golden.npz"), **out)
    with open(os.path.join(HERE, "golden_hashes.json"), "w") as f:
        json.dump(hashes, f, indent=1, sort_keys=True)
    print("wrote", len(out), "arrays and", len(hashes), "hashed cases")


if __name__ == "__main__":
    main()

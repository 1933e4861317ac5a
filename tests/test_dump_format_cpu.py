"""The reference's MINIFE_DEBUG dump files (write_matrix / write_vector,
ref/src/SparseMatrix_functions.hpp:98-140, Vector_functions.hpp:49-82),
written by the reference itself for the 2x3x2 box (tests/golden/dumps_2x3x2,
made by gen_golden.py), against the oracle's system in the same format."""
import os

import numpy as np

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
DUMPS = os.path.join(HERE, "golden", "dumps_2x3x2")


def fmt(v):
    """std::ostream's default double format: 6 significant digits, %g style."""
    return "%.6g" % v


def mtx_text(ro, cols, vals):
    lines = ["%d %d" % (ro.size - 1, cols.size)]
    for i in range(ro.size - 1):
        for k in range(ro[i], ro[i + 1]):
            lines.append("%d %d %s" % (i, cols[k], fmt(vals[k])))
    return "\n".join(lines) + "\n"


def vec_text(v):
    return "\n".join(["%d" % v.size] + ["%d %s" % (i, fmt(x)) for i, x in enumerate(v)]) + "\n"


def read(name):
    return open(os.path.join(DUMPS, name + ".1.0")).read()


def test_oracle_system_matches_reference_dumps():
    ro, cols, vals_pre, b_pre = O.assemble(2, 3, 2)
    assert read("A_prebc.mtx") == mtx_text(ro, cols, vals_pre)
    assert read("b_prebc.vec") == vec_text(b_pre)
    ro, cols, vals, b = O.build_system(2, 3, 2)
    assert read("A.mtx") == mtx_text(ro, cols, vals)
    assert read("b.vec") == vec_text(b)
    x, it, nr, st = O.cg_solve(ro, cols, vals, b)
    xs = np.array([float(l.split()[1]) for l in read("x.vec").splitlines()[1:]])
    assert np.allclose(xs, x, rtol=1e-5, atol=1e-12)

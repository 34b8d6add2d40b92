"""CPU tests of the oracle's block-tridiagonal solvers (the second-order
implicit path, src/nsolve{1,2}{bc,p}.f90): bit-for-bit against the outputs
of the reference's own sources (tests/golden, and the translated reference
where it is built), and known answers."""
import os

import numpy as np
import pytest

import oracle
import tricase
from tricase import SOLVERS

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("solver", SOLVERS)
def test_tri_oracle_reproduces_reference_golden(solver):
    d = np.load(os.path.join(GOLDEN, "tri_%s.npz" % solver))
    case = tricase.make_case(solver, int(d["rows"]), int(d["nsys"]))
    case["mat"] = np.asfortranarray(d["mat_in"])
    case["rhs"] = np.asfortranarray(d["rhs_in"])
    if "bc_in" in d:
        case["bc"] = np.asfortranarray(d["bc_in"])
    assert np.array_equal(tricase.run_oracle(case), d["rhs_out"])


@pytest.mark.parametrize("solver", SOLVERS)
@pytest.mark.parametrize("rows,nsys", [(9, 1), (12, 4), (31, 3)])
def test_tri_oracle_matches_translated_reference(solver, rows, nsys):
    if oracle.ref() is None:
        pytest.skip("translated reference not built")
    case = tricase.make_case(solver, rows, nsys, seed=rows * 10 + nsys)
    assert np.array_equal(tricase.run_oracle(case), tricase.run_ref(case))


@pytest.mark.parametrize("solver", SOLVERS)
@pytest.mark.parametrize("rows", [9, 16])
def test_tri_oracle_known_answer(solver, rows):
    """A x = b with the line's dense matrix built from the block table."""
    case = tricase.make_case(solver, rows, 3, seed=rows)
    x = tricase.run_oracle(case)
    for iv in range(3):
        A = tricase.dense_line(case, iv)
        b = tricase.line_rhs(case, case["rhs"], iv)
        assert np.allclose(A @ tricase.line_rhs(case, x, iv), b, rtol=0, atol=1e-12 * np.abs(b).max())
    if tricase.info(solver)["periodic"]:  # row np repeats row 1
        first = x[:, 0, :] if tricase.info(solver)["layout"] == 2 else x[:, :, 0]
        last = x[:, rows - 1, :] if tricase.info(solver)["layout"] == 2 else x[:, :, rows - 1]
        assert np.array_equal(first, last)

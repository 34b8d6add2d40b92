"""CPU tests of the oracle (the restated reference line solvers)."""
import glob
import os

import numpy as np
import pytest

import oracle
import pentacase
from pentacase import SOLVERS, info

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(solver):
    d = np.load(os.path.join(GOLDEN, "penta_%s.npz" % solver))
    case = pentacase.make_case(solver, int(d["rows"]), int(d["nsys"]), seed=0)
    case["mat"] = np.asfortranarray(d["mat_in"])
    case["rhs"] = np.asfortranarray(d["rhs_in"])
    return case, d


@pytest.mark.parametrize("solver", SOLVERS)
def test_oracle_reproduces_reference_golden(solver):
    """Bit-for-bit: the oracle with the reference-compatible options gives the
    outputs the reference's own sources produced (tests/golden)."""
    case, d = golden(solver)
    c = info(solver)
    flags = oracle.COMPAT_PERIODIC_SLOT | oracle.COMPAT_CBC_RHS
    if c["complex"]:
        fac = pentacase.run_oracle(case, code=0, flags=flags)
        assert np.array_equal(fac["mat"], d["mat_factored"])
        if c["periodic"]:
            assert np.array_equal(fac["per"], d["per_factored"])
            assert np.array_equal(fac["per2"], d["per2_factored"])
    out = pentacase.run_oracle(case, code=2, flags=flags)
    assert np.array_equal(out["rhs"], d["rhs_out"])


@pytest.mark.parametrize("solver", SOLVERS)
@pytest.mark.parametrize("rows,nsys", [(7, 1), (8, 5), (13, 4), (40, 3)])
def test_oracle_matches_translated_reference(solver, rows, nsys):
    """Bit-for-bit against the translated reference on fresh seeded cases
    (skipped where the reference tree was not available to translate)."""
    if oracle.ref() is None:
        pytest.skip("translated reference not built")
    c = info(solver)
    if c["periodic"] and rows < 8:
        rows = 8
    case = pentacase.make_case(solver, rows, nsys, seed=rows * 100 + nsys)
    if c["complex"] and not c["periodic"]:
        # the reference solve phase is mis-indexed; compare its bug-free factor phase
        a, b = pentacase.run_ref(case, code=0), pentacase.run_oracle(case, code=0)
        assert np.array_equal(a["mat"], b["mat"])
        return
    a = pentacase.run_ref(case)
    b = pentacase.run_oracle(case)
    assert np.array_equal(a["rhs"], b["rhs"])
    if c["complex"]:
        assert np.array_equal(a["mat"], b["mat"])


# ---------------------------------------------------------------- known answers

def col_bc(i, k, n):
    """Column (1-based) of slot k in row i, boundary-closure layout."""
    if i == 1:
        return {3: 1, 4: 2, 5: 3, 1: 4, 2: 5}[k]
    if i == 2:
        return {2: 1, 3: 2, 4: 3, 5: 4, 1: 5}[k]
    if i == n - 1:
        return {5: n - 4, 1: n - 3, 2: n - 2, 3: n - 1, 4: n}[k]
    if i == n:
        return {4: n - 4, 5: n - 3, 1: n - 2, 2: n - 1, 3: n}[k]
    return i + k - 3


def dense(case, iv):
    """Dense matrix of line iv assembled directly from the slot layout."""
    c = info(case["solver"])
    rows = case["rows"]
    n = rows - 1 if c["periodic"] else rows
    mat = case["mat"]
    A = np.zeros((5 * n, 5 * n), dtype=mat.dtype)
    for i in range(1, n + 1):
        blk = mat[:, :, :, i - 1, iv] if c["layout"] == 2 else mat[:, :, :, iv, i - 1]
        for k in range(1, 6):
            col = (i + k - 4) % n + 1 if c["periodic"] else col_bc(i, k, n)
            A[5 * (i - 1):5 * i, 5 * (col - 1):5 * col] += blk[k - 1]
    return A, n


def line_rhs(case, arr, iv, n):
    c = info(case["solver"])
    v = arr[:, :n, iv] if c["layout"] == 2 else arr[:, iv, :n]
    return v.T.reshape(-1)


@pytest.mark.parametrize("solver", SOLVERS)
@pytest.mark.parametrize("rows", [8, 9, 16, 33])
def test_oracle_known_answer(solver, rows):
    """The exact (corrected) oracle solves the assembled dense system."""
    case = pentacase.make_case(solver, rows, 3, seed=rows)
    out = pentacase.run_oracle(case, code=2, flags=0)
    for iv in range(3):
        A, n = dense(case, iv)
        b = line_rhs(case, case["rhs"], iv, n)
        x = line_rhs(case, out["rhs"], iv, n)
        assert np.abs(A @ x - b).max() < 1e-12 * np.abs(b).max()
        if info(solver)["periodic"]:
            xs = out["rhs"][:, -1, iv] if info(solver)["layout"] == 2 else out["rhs"][:, iv, -1]
            assert np.array_equal(xs, x[:5])  # row np duplicates row 1


@pytest.mark.parametrize("solver", ["penta2p", "cpenta1p"])
def test_reference_periodic_slot_quirk(solver):
    """The reference periodic solvers place one fill block in the wrong slot
    at row n-5: their solution misses A^-1 b by an amount that decays with
    the line length; the corrected oracle does not."""
    for rows, lo, hi in [(8, 1e-6, 1e-1), (21, 1e-12, 1e-5)]:
        case = pentacase.make_case(solver, rows, 1, seed=5)
        A, n = dense(case, 0)
        b = line_rhs(case, case["rhs"], 0, n)
        xc = line_rhs(case, pentacase.run_oracle(case, flags=oracle.COMPAT_PERIODIC_SLOT)["rhs"], 0, n)
        xe = line_rhs(case, pentacase.run_oracle(case, flags=0)["rhs"], 0, n)
        ec = np.abs(xc - xe).max() / np.abs(xe).max()
        assert lo < ec < hi
        assert np.abs(A @ xe - b).max() < 1e-12 * np.abs(b).max()


def test_oracle_rejects_short_lines():
    O = oracle.orc()
    a = np.zeros(125 * 6, dtype=np.float64)
    r = np.zeros(5 * 6, dtype=np.float64)
    assert O.orc_penta_bc(2, 6, 1, oracle.ptr(a), oracle.ptr(r)) != 0

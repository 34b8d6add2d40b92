"""GPU parity of the line solvers against the oracle and the reference
golden outputs.  Tolerance: 1e-13 in the max norm relative to the largest
entry (the isolated-solve workload's bar); the GPU fuses multiply-adds and
multiplies by reciprocals where the reference divides, so agreement is to
rounding, not bit-for-bit."""
import os

import numpy as np
import pytest

import pentacase
from pentacase import info, relerr

pytestmark = pytest.mark.gpu
TOL = 1e-13
BC = ["penta2bc", "penta1bc", "cpenta2bc", "cpenta1bc"]
PER = ["penta2p", "penta1p", "cpenta2p", "cpenta1p"]
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("solver", BC)
@pytest.mark.parametrize("rows,nsys", [(7, 1), (8, 3), (9, 5), (12, 33), (64, 17), (130, 9)])
@pytest.mark.parametrize("where", ["host", "device"])
def test_bc_solve_matches_oracle(cuda, solver, rows, nsys, where):
    case = pentacase.make_case(solver, rows, nsys, seed=rows * 31 + nsys)
    ref = pentacase.run_oracle(case, code=2, flags=0)
    got = pentacase.run_gpu(case, code=2, device=cuda if where == "device" else None)
    assert relerr(got["rhs"], ref["rhs"]) < TOL
    if info(solver)["complex"]:
        assert relerr(got["mat"], ref["mat"]) < TOL


@pytest.mark.parametrize("solver", ["cpenta2bc", "cpenta1bc"])
@pytest.mark.parametrize("rows,nsys", [(7, 2), (11, 6), (96, 13)])
def test_complex_factor_then_solve(cuda, solver, rows, nsys):
    """code 0 then code 1 (the impdrv3d pattern: factor once, solve per step)."""
    case = pentacase.make_case(solver, rows, nsys, seed=rows + 7 * nsys)
    fac_ref = pentacase.run_oracle(case, code=0)
    fac = pentacase.run_gpu(case, code=0, device=cuda)
    assert relerr(fac["mat"], fac_ref["mat"]) < TOL
    assert np.array_equal(fac["rhs"], case["rhs"])  # code 0 leaves rhs alone
    for step in range(3):
        rhs = pentacase.make_case(solver, rows, nsys, seed=500 + step)["rhs"]
        a = dict(fac, rhs=rhs)
        b = dict(fac_ref, rhs=rhs)
        got = pentacase.run_gpu(a, code=1, device=cuda)
        want = pentacase.run_oracle(b, code=1, flags=0)
        assert relerr(got["rhs"], want["rhs"]) < TOL
        assert np.array_equal(got["mat"], fac["mat"])  # code 1 leaves mat alone


@pytest.mark.parametrize("solver", PER)
@pytest.mark.parametrize("rows,nsys", [(8, 1), (9, 3), (10, 5), (13, 17), (64, 9), (129, 6)])
@pytest.mark.parametrize("where", ["host", "device"])
def test_periodic_solve_matches_oracle(cuda, solver, rows, nsys, where):
    """Default mode reproduces the reference (fill placement at row n-5)."""
    case = pentacase.make_case(solver, rows, nsys, seed=rows * 17 + nsys)
    ref = pentacase.run_oracle(case, code=2)
    got = pentacase.run_gpu(case, code=2, device=cuda if where == "device" else None)
    assert relerr(got["rhs"], ref["rhs"]) < TOL
    if info(solver)["complex"]:
        for k in ("mat", "per", "per2"):
            assert relerr(got[k], ref[k]) < TOL, k


@pytest.mark.parametrize("solver", PER)
@pytest.mark.parametrize("rows,nsys", [(8, 2), (12, 7), (100, 5)])
def test_periodic_exact_mode(cuda, solver, rows, nsys):
    import lns3d_gb300 as g

    case = pentacase.make_case(solver, rows, nsys, seed=rows + 3 * nsys)
    ref = pentacase.run_oracle(case, code=2, flags=0)
    g.set_periodic_exact(True)
    try:
        got = pentacase.run_gpu(case, code=2, device=cuda)
    finally:
        g.set_periodic_exact(False)
    assert relerr(got["rhs"], ref["rhs"]) < TOL


@pytest.mark.parametrize("solver", ["cpenta2p", "cpenta1p"])
@pytest.mark.parametrize("rows,nsys", [(8, 2), (11, 6), (96, 13)])
def test_periodic_factor_then_solve(cuda, solver, rows, nsys):
    case = pentacase.make_case(solver, rows, nsys, seed=rows + 11 * nsys)
    fac_ref = pentacase.run_oracle(case, code=0)
    fac = pentacase.run_gpu(case, code=0, device=cuda)
    for k in ("mat", "per", "per2"):
        assert relerr(fac[k], fac_ref[k]) < TOL, k
    for step in range(2):
        rhs = pentacase.make_case(solver, rows, nsys, seed=900 + step)["rhs"]
        got = pentacase.run_gpu(dict(fac, rhs=rhs), code=1, device=cuda)
        want = pentacase.run_oracle(dict(fac_ref, rhs=rhs), code=1)
        assert relerr(got["rhs"], want["rhs"]) < TOL
        assert np.array_equal(got["mat"], fac["mat"])


@pytest.mark.parametrize("solver", BC + PER)
def test_matches_reference_golden(cuda, solver):
    """Against outputs of the reference's own sources (tests/golden)."""
    d = np.load(os.path.join(GOLDEN, "penta_%s.npz" % solver))
    case = pentacase.make_case(solver, int(d["rows"]), int(d["nsys"]), seed=0)
    case["mat"], case["rhs"] = np.asfortranarray(d["mat_in"]), np.asfortranarray(d["rhs_in"])
    c = info(solver)
    if c["complex"]:
        fac = pentacase.run_gpu(case, code=0)
        assert relerr(fac["mat"], d["mat_factored"]) < TOL
        if c["periodic"]:
            assert relerr(fac["per"], d["per_factored"]) < TOL
            assert relerr(fac["per2"], d["per2_factored"]) < TOL
    if not (c["complex"] and not c["periodic"]):  # the reference's complex bc solve is mis-indexed
        got = pentacase.run_gpu(case)
        assert relerr(got["rhs"], d["rhs_out"]) < TOL


def test_zero_lines_device(cuda):
    import torch

    import lns3d_gb300 as g

    m = torch.zeros(1, dtype=torch.complex128, device=cuda)
    g.cpenta2bc(8, 0, 5, m, m.clone(), 2)
    torch.cuda.synchronize()


def test_zero_pivot_reports_error(cuda):
    import lns3d_gb300 as g

    case = pentacase.make_case("penta2bc", 9, 2, seed=3)
    case["mat"][:, :, :, :, 1] = 0.0  # line 2 is singular: its first pivot is zero
    with pytest.raises(g.LnsError) as e:
        g.penta2bc(9, 2, 5, case["mat"], case["rhs"])
    assert e.value.code == 3


def test_full_size_periodic_solve(cuda):
    """512 complex periodic lines of 257 rows (256 unknowns)."""
    case = pentacase.make_case("cpenta1p", 257, 512, seed=77, normal_rhs=True)
    ref = pentacase.run_oracle(case, code=2)
    got = pentacase.run_gpu(case, code=2, device=cuda)
    assert relerr(got["rhs"], ref["rhs"]) < TOL


def test_full_size_isolated_solve(cuda):
    """512 complex lines of 256 rows (the isolated batched solve): every line
    against the oracle, and the device result equals the host-staged one."""
    case = pentacase.make_case("cpenta2bc", 256, 512, seed=2024, normal_rhs=True)
    ref = pentacase.run_oracle(case, code=2, flags=0)
    got = pentacase.run_gpu(case, code=2, device=cuda)
    assert relerr(got["rhs"], ref["rhs"]) < TOL
    assert relerr(got["mat"], ref["mat"]) < TOL
    host = pentacase.run_gpu(case, code=2)
    assert np.array_equal(host["rhs"], got["rhs"])

"""GPU tests of the mixed-precision solves (FP32 LU + FP64 refinement)
against the exact FP64 oracle.  Tolerances: 1e-13 relative (max norm) with
two refinement steps, 1e-5 for the bare FP32 solve."""
import numpy as np
import pytest

import pentacase
from pentacase import info, relerr

pytestmark = pytest.mark.gpu


def run_mixed(case, cuda, refine, code=2, work=None):
    import torch

    from lns3d_gb300 import mixed

    c = info(case["solver"])
    d = pentacase.dims(case)
    mat = torch.from_numpy(case["mat"].ravel(order="F")).to(cuda)
    rhs = torch.from_numpy(case["rhs"].ravel(order="F")).to(cuda)
    mat0 = mat.clone()
    fn = getattr(mixed, case["solver"] + "_mixed")
    if c["complex"]:
        work = fn(d[0], d[1], 5, mat, rhs, code=code, refine=refine, work=work)
    else:
        work = fn(d[0], d[1], 5, mat, rhs, refine=refine, work=work)
    assert torch.equal(mat, mat0)  # mat is read only
    return rhs.cpu().numpy().reshape(case["rhs"].shape, order="F"), work


SOLVERS = ["cpenta2bc", "cpenta1bc", "cpenta2p", "cpenta1p", "penta2bc", "penta1bc"]


@pytest.mark.parametrize("solver", SOLVERS)
@pytest.mark.parametrize("rows,nsys", [(8, 3), (33, 7), (256, 20)])
def test_mixed_refined_matches_fp64(cuda, solver, rows, nsys):
    case = pentacase.make_case(solver, rows, nsys, seed=rows * 3 + nsys, normal_rhs=True)
    want = pentacase.run_oracle(case, code=2, flags=0)["rhs"]
    got, _ = run_mixed(case, cuda, refine=2)
    assert relerr(got, want) < 1e-13


@pytest.mark.parametrize("solver", ["cpenta2bc", "cpenta1p"])
def test_mixed_fp32_only(cuda, solver):
    case = pentacase.make_case(solver, 64, 9, seed=4, normal_rhs=True)
    want = pentacase.run_oracle(case, code=2, flags=0)["rhs"]
    got, _ = run_mixed(case, cuda, refine=0)
    e = relerr(got, want)
    assert 1e-12 < e < 1e-5  # FP32 accuracy, and genuinely FP32
    got1, _ = run_mixed(case, cuda, refine=1)
    assert relerr(got1, want) < e * 1e-3  # each refinement step gains ~cond * 2^-24


@pytest.mark.parametrize("solver", ["cpenta2bc", "cpenta2p"])
def test_mixed_factor_once_solve_many(cuda, solver):
    case = pentacase.make_case(solver, 40, 6, seed=8)
    _, work = run_mixed(case, cuda, refine=2, code=0)
    for step in range(3):
        rhs = pentacase.make_case(solver, 40, 6, seed=100 + step, normal_rhs=True)["rhs"]
        c2 = dict(case, rhs=rhs)
        want = pentacase.run_oracle(c2, code=2, flags=0)["rhs"]
        got, _ = run_mixed(c2, cuda, refine=2, code=1, work=work)
        assert relerr(got, want) < 1e-13


def test_mixed_full_size(cuda):
    """The isolated batched solve workload, 512 complex lines x 256 rows."""
    case = pentacase.make_case("cpenta2bc", 256, 512, seed=2024, normal_rhs=True)
    want = pentacase.run_oracle(case, code=2, flags=0)["rhs"]
    got, _ = run_mixed(case, cuda, refine=2)
    assert relerr(got, want) < 1e-13


def test_mixed_host_entry_point(cuda):
    import lns3d_gb300 as g

    case = pentacase.make_case("cpenta2bc", 50, 4, seed=9, normal_rhs=True)
    want = pentacase.run_oracle(case, code=2, flags=0)["rhs"]
    rhs = case["rhs"].copy(order="F")
    g.lib().lns_cpenta2bc_mixed(50, 4, 5, case["mat"].ctypes.data, rhs.ctypes.data, 2)
    assert relerr(rhs, want) < 1e-13

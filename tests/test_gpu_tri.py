"""GPU tests of the block-tridiagonal line solvers of the second-order
implicit path (lns_solve{1,2}{bc,p}, through the C ABI): host and device
forms against the oracle (oracle/tri_oracle.c, bit-for-bit with the
reference's own sources), within 1e-13 of the largest solution entry."""
import numpy as np
import pytest

import tricase
from tricase import SOLVERS

pytestmark = pytest.mark.gpu
TOL = 1e-13


def gpu_solve(case, device):
    import torch

    import lns3d_gb300 as g

    s, rows, nsys = case["solver"], case["rows"], case["nsys"]
    mat, rhs = case["mat"].copy(order="F"), case["rhs"].copy(order="F")
    bc = case["bc"].copy(order="F") if "bc" in case else None
    dims = (rows, nsys) if tricase.info(s)["layout"] == 2 else (nsys, rows)
    fn = getattr(g, s)
    if device:
        tm = torch.from_numpy(mat.ravel(order="F")).cuda()
        tr = torch.from_numpy(rhs.ravel(order="F")).cuda()
        tb = torch.from_numpy(bc.ravel(order="F")).cuda() if bc is not None else None
        if bc is None:
            fn(dims[0], dims[1], 5, tm, tr)
        else:
            fn(dims[0], dims[1], 5, tm, tr, tb)
        torch.cuda.synchronize()
        return tr.cpu().numpy().reshape(rhs.shape, order="F"), None
    if bc is None:
        fn(dims[0], dims[1], 5, mat, rhs)
    else:
        fn(dims[0], dims[1], 5, mat, rhs, bc)
    return rhs, (mat, bc)


@pytest.mark.parametrize("solver", SOLVERS)
@pytest.mark.parametrize("rows,nsys", [(8, 1), (9, 3), (17, 5), (64, 130), (40, 700)])
@pytest.mark.parametrize("device", [False, True])
def test_tri_matches_oracle(cuda, solver, rows, nsys, device):
    if tricase.info(solver)["periodic"]:
        rows = max(rows, 9)
    case = tricase.make_case(solver, rows, nsys, seed=rows + 7 * nsys)
    want = tricase.run_oracle(case)
    got, kept = gpu_solve(case, device)
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()
    if kept is not None:  # host form: mat and bc are read only
        assert np.array_equal(kept[0], case["mat"])
        if kept[1] is not None:
            assert np.array_equal(kept[1], case["bc"])


def test_tri_known_answer(cuda):
    case = tricase.make_case("solve2bc", 12, 2, seed=5)
    got, _ = gpu_solve(case, False)
    for iv in range(2):
        A = tricase.dense_line(case, iv)
        b = tricase.line_rhs(case, case["rhs"], iv)
        assert np.allclose(A @ tricase.line_rhs(case, got, iv), b, rtol=0, atol=1e-12 * np.abs(b).max())


def test_tri_rejects_short_lines(cuda):
    import lns3d_gb300 as g

    case = tricase.make_case("solve2bc", 7, 1)
    with pytest.raises(g.LnsError):
        g.solve2bc(7, 1, 5, case["mat"], case["rhs"], case["bc"])
    case = tricase.make_case("solve2p", 8, 1)
    with pytest.raises(g.LnsError):
        g.solve2p(8, 1, 5, case["mat"], case["rhs"])

"""GPU test of lns_cpenta2bc_mixed_static_dev, the mixed complex boundary
solve whose scratch is a fixed array in the library's device image.

It is for callers that cannot allocate device memory during a solve: the
entry point takes no workspace and must not allocate.  It is called through
the C ABI twice in a row on the same inputs; each result is compared with
lns_cpenta2bc_mixed_dev (caller-owned workspace, code 2, the same refinement
count: the same kernels, so the expected difference is zero) and with the
oracle's FP64 direct solve, both at 1e-13 of the largest entry, the
isolated-solve parity bar.  The device's free memory (cudaMemGetInfo) is the
same before and after the second call: the call allocated nothing.  Problems
whose scratch exceeds the fixed array must be rejected before any device
work.
"""
import ctypes

import numpy as np
import pytest

from pentacase import make_case, run_oracle

pytestmark = pytest.mark.gpu

TOL = 1e-13
N, NSYS, REFINE = 200, 96, 2   # 19 200 rows x lines: inside the fixed scratch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()


def test_static_workspace_solve_matches_caller_workspace(cuda):
    import torch
    from lns3d_gb300 import lib

    L = lib()
    case = make_case("cpenta2bc", N, NSYS, seed=21, normal_rhs=True)
    mat = _dev(torch, case["mat"])
    rhs0 = _dev(torch, case["rhs"])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    nbytes = L.lns_mixed_workspace_bytes(N, NSYS, 1, 0)
    assert 0 < nbytes <= 32 << 20
    work = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    want = rhs0.clone()
    rc = L.lns_cpenta2bc_mixed_dev(N, NSYS, 5, ctypes.c_void_p(mat.data_ptr()), ctypes.c_void_p(want.data_ptr()),
                                   2, REFINE, ctypes.c_void_p(work.data_ptr()), stream)
    assert rc == 0, L.lns_last_error()

    oracle = run_oracle(case, code=2, flags=0)["rhs"]   # FP64 direct solve, row n-3 corrected
    want_orc = torch.from_numpy(np.ascontiguousarray(oracle.ravel(order="F")))

    for call in range(2):
        got = rhs0.clone()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = L.lns_cpenta2bc_mixed_static_dev(N, NSYS, 5, ctypes.c_void_p(mat.data_ptr()),
                                              ctypes.c_void_p(got.data_ptr()), REFINE, stream)
        assert rc == 0, L.lns_last_error()
        torch.cuda.synchronize()
        if call == 1:   # the first call on a device may load the module; the second must not allocate
            assert torch.cuda.mem_get_info()[0] == free_before
        err = float((got - want).abs().max() / want.abs().max())
        assert err <= TOL, (call, err)
        err_orc = float((got.cpu() - want_orc).abs().max() / want_orc.abs().max())
        assert err_orc <= TOL, (call, err_orc)
    # mat is read only in the mixed solves
    assert torch.equal(mat, _dev(torch, case["mat"]))


def test_static_workspace_rejects_oversize_problem(cuda):
    from lns3d_gb300 import lib

    L = lib()
    # 256 rows x 512 lines needs ~147 MB of scratch: rejected before any device work
    rc = L.lns_cpenta2bc_mixed_static_dev(256, 512, 5, None, None, 2, None)
    assert rc == 1
    msg = L.lns_last_error().decode()
    assert "static workspace" in msg and str(32 << 20) in msg

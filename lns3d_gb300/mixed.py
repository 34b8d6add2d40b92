"""Mixed-precision line solves (FP32 LU, FP64 residual refinement).

Device tensors only (torch CUDA complex128 / float64 flat buffers in the
reference layouts, as for :mod:`lns3d_gb300.penta`).  ``mat`` is read only.
The FP32 factors live in a workspace tensor returned by the factor call
(code 0 or 2) and passed back to later solve calls (code 1).
"""
import ctypes

from ._lib import check, lib
from .penta import _buf, _stream

__all__ = ["workspace", "cpenta2bc_mixed", "cpenta1bc_mixed", "cpenta2p_mixed", "cpenta1p_mixed",
           "penta2bc_mixed", "penta1bc_mixed"]


def workspace(rows, nsys, is_complex, periodic, device):
    import torch

    nbytes = lib().lns_mixed_workspace_bytes(rows, nsys, 1 if is_complex else 0, 1 if periodic else 0)
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


def _run(name, d0, d1, rows, nsys, nblk, mat, rhs, complex_, periodic, code, refine, work):
    pm, dm = _buf(mat, complex_, 125 * rows * nsys, "mat")
    pr, dr = _buf(rhs, complex_, 5 * rows * nsys, "rhs")
    if not (dm and dr):
        raise ValueError("mixed solves take CUDA tensors")
    if work is None:
        work = workspace(rows, nsys, complex_, periodic, mat.device)
    args = [d0, d1, nblk, pm, pr]
    if code is not None:
        args.append(int(code))
    args += [int(refine), ctypes.c_void_p(work.data_ptr()), _stream()]
    check(getattr(lib(), "lns_%s_dev" % name)(*args), name)
    return work


def cpenta2bc_mixed(n, nsys, nblk, mat, rhs, code=2, refine=2, work=None):
    return _run("cpenta2bc_mixed", n, nsys, n, nsys, nblk, mat, rhs, True, False, code, refine, work)


def cpenta1bc_mixed(nsys, n, nblk, mat, rhs, code=2, refine=2, work=None):
    return _run("cpenta1bc_mixed", nsys, n, n, nsys, nblk, mat, rhs, True, False, code, refine, work)


def cpenta2p_mixed(np_, nsys, nblk, mat, rhs, code=2, refine=2, work=None):
    return _run("cpenta2p_mixed", np_, nsys, np_, nsys, nblk, mat, rhs, True, True, code, refine, work)


def cpenta1p_mixed(nsys, np_, nblk, mat, rhs, code=2, refine=2, work=None):
    return _run("cpenta1p_mixed", nsys, np_, np_, nsys, nblk, mat, rhs, True, True, code, refine, work)


def penta2bc_mixed(n, nsys, nblk, mat, rhs, refine=2, work=None):
    return _run("penta2bc_mixed", n, nsys, n, nsys, nblk, mat, rhs, False, False, None, refine, work)


def penta1bc_mixed(nsys, n, nblk, mat, rhs, refine=2, work=None):
    return _run("penta1bc_mixed", nsys, n, n, nsys, nblk, mat, rhs, False, False, None, refine, work)

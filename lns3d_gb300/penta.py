"""Host-side mirror of the reference line-solver interface.

The functions keep the Fortran names, argument order and array layouts of
the LNS3D solvers (src/penta2bc.f:2, src/penta1bc.f:2, src/cpenta2bc.f:2,
src/cpenta1bc.f:2): ``mat`` and ``rhs`` are flat buffers holding the Fortran
column-major arrays ``mat(5,nblk,nblk,n,nsys)`` / ``rhs(nblk,n,nsys)`` (the
"2" solvers) or ``mat(5,nblk,nblk,nsys,n)`` / ``rhs(nblk,nsys,n)`` (the "1"
solvers), real float64 or complex128.  They are updated in place, like the
Fortran INOUT arguments.

``mat``/``rhs`` may be numpy arrays (host memory: the call stages them to the
GPU and back, synchronously) or CUDA torch tensors (device memory: the solve
is enqueued on torch's current stream).  Every call runs the sm_103a kernels
of ``lib/liblns3d_gb300.so``; errors raise :class:`LnsError` (the reference
has no error return and leaves Inf/NaN on a zero pivot).
"""
import ctypes

import numpy as np

from ._lib import LnsError, check, lib

__all__ = ["penta2bc", "penta1bc", "cpenta2bc", "cpenta1bc", "penta2p", "penta1p", "cpenta2p", "cpenta1p",
           "set_periodic_exact", "LnsError"]


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _buf(a, complex_, count, name):
    """Pointer to a contiguous buffer of `count` elements; (ptr, is_device)."""
    if _is_torch(a):
        import torch

        want = torch.complex128 if complex_ else torch.float64
        if a.dtype != want:
            raise TypeError("%s must be %s, got %s" % (name, want, a.dtype))
        if not a.is_contiguous():
            raise ValueError("%s must be contiguous" % name)
        if a.numel() < count:
            raise ValueError("%s holds %d elements, needs %d" % (name, a.numel(), count))
        return ctypes.c_void_p(a.data_ptr()), a.is_cuda
    want = np.complex128 if complex_ else np.float64
    if not isinstance(a, np.ndarray) or a.dtype != want:
        raise TypeError("%s must be a numpy %s array" % (name, np.dtype(want).name))
    if not (a.flags.c_contiguous or a.flags.f_contiguous):
        raise ValueError("%s must be contiguous" % name)
    if a.size < count:
        raise ValueError("%s holds %d elements, needs %d" % (name, a.size, count))
    if not a.flags.writeable:
        raise ValueError("%s must be writeable" % name)
    return ctypes.c_void_p(a.ctypes.data), False


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _call(name, dims, nblk, mat, rhs, complex_, code=None, per=None, per2=None):
    n_rows = dims[0] * dims[1]
    pm, dev_m = _buf(mat, complex_, 125 * n_rows, "mat")
    pr, dev_r = _buf(rhs, complex_, 5 * n_rows, "rhs")
    bufs = [pm, pr]
    devs = {dev_m, dev_r}
    if per is not None:
        pp, dev_p = _buf(per, complex_, 50 * n_rows, "per")
        bufs.append(pp)
        devs.add(dev_p)
        if complex_:
            pp2, dev_p2 = _buf(per2, complex_, 50 * n_rows, "per2")
            devs.add(dev_p2)
        else:  # real per2 is reference scratch, unused here
            pp2 = ctypes.c_void_p(0)
        bufs.append(pp2)
    if len(devs) != 1:
        raise ValueError("arrays must all be host arrays or all CUDA tensors")
    L = lib()
    extra = [] if code is None else [int(code)]
    if dev_m:
        rc = getattr(L, "lns_%s_dev" % name)(dims[0], dims[1], nblk, *bufs, *extra, _stream())
    else:
        rc = getattr(L, "lns_%s" % name)(dims[0], dims[1], nblk, *bufs, *extra)
    check(rc, name)


def penta2bc(n, nsys, nblk, mat, rhs):
    """Real boundary-closure solve, lines along the first spatial index."""
    _call("penta2bc", (n, nsys), nblk, mat, rhs, False)


def penta1bc(nsys, n, nblk, mat, rhs):
    """Real boundary-closure solve, lines along the second spatial index."""
    _call("penta1bc", (nsys, n), nblk, mat, rhs, False)


def cpenta2bc(n, nsys, nblk, mat, rhs, code):
    """Complex boundary-closure solve; code 0 factor, 1 solve, 2 both."""
    _call("cpenta2bc", (n, nsys), nblk, mat, rhs, True, code)


def cpenta1bc(nsys, n, nblk, mat, rhs, code):
    """Complex boundary-closure solve (lines batched over the first index)."""
    _call("cpenta1bc", (nsys, n), nblk, mat, rhs, True, code)


def penta2p(np_, nsys, nblk, mat, rhs, per, per2=None):
    """Real periodic solve (np_ rows, the last repeating the first)."""
    _call("penta2p", (np_, nsys), nblk, mat, rhs, False, per=per, per2=per2)


def penta1p(nsys, np_, nblk, mat, rhs, per, per2=None):
    """Real periodic solve, lines batched over the first index."""
    _call("penta1p", (nsys, np_), nblk, mat, rhs, False, per=per, per2=per2)


def cpenta2p(np_, nsys, nblk, mat, rhs, per, per2, code):
    """Complex periodic solve; code 0 factor, 1 solve, 2 both."""
    _call("cpenta2p", (np_, nsys), nblk, mat, rhs, True, code, per=per, per2=per2)


def cpenta1p(nsys, np_, nblk, mat, rhs, per, per2, code):
    """Complex periodic solve, lines batched over the first index."""
    _call("cpenta1p", (nsys, np_), nblk, mat, rhs, True, code, per=per, per2=per2)


def set_periodic_exact(on):
    """True: later periodic factorisations are the exact LU; False (default):
    they reproduce the reference's fill placement at row n-5."""
    check(lib().lns_set_periodic_exact(1 if on else 0), "set_periodic_exact")


# ---------------------------------------------------------------------------
# Block-tridiagonal solves of the second-order implicit path (iLHS = 0):
# src/nsolve{1,2}{bc,p}.f90, same argument order.  Host numpy arrays or
# CUDA torch tensors (float64); the device form allocates its workspace
# with torch.


def _tri(name, dims, rows, nsys, nblk, mat, rhs, bc=None):
    n_rows = rows * nsys
    pm, dev_m = _buf(mat, False, 75 * n_rows, "mat")
    pr, dev_r = _buf(rhs, False, 5 * n_rows, "rhs")
    bufs, devs = [pm, pr], {dev_m, dev_r}
    if bc is not None:
        pb, dev_b = _buf(bc, False, 350 * nsys, "bc")
        bufs.append(pb)
        devs.add(dev_b)
    if len(devs) != 1:
        raise ValueError("arrays must all be host arrays or all CUDA tensors")
    L = lib()
    if dev_m:
        import torch

        wb = L.lns_tri_workspace_bytes(rows, nsys, 0 if bc is not None else 1)
        work = torch.empty(max(wb, 8), dtype=torch.uint8, device=mat.device)
        rc = getattr(L, "lns_%s_dev" % name)(dims[0], dims[1], nblk, *bufs, ctypes.c_void_p(work.data_ptr()),
                                             _stream())
    else:
        if bc is None:
            bufs += [ctypes.c_void_p(0), ctypes.c_void_p(0)]
        rc = getattr(L, "lns_%s" % name)(dims[0], dims[1], nblk, *bufs)
    check(rc, name)


def solve2bc(n, nsys, nblk, mat, rhs, bc):
    """Block-tridiagonal boundary-closure solve, lines along the first index."""
    _tri("solve2bc", (n, nsys), n, nsys, nblk, mat, rhs, bc)


def solve1bc(nsys, n, nblk, mat, rhs, bc):
    """Block-tridiagonal boundary-closure solve, lines batched over the first index."""
    _tri("solve1bc", (nsys, n), n, nsys, nblk, mat, rhs, bc)


def solve2p(np_, nsys, nblk, mat, rhs):
    """Periodic block-tridiagonal solve (np_ rows, the last repeating the first)."""
    _tri("solve2p", (np_, nsys), np_, nsys, nblk, mat, rhs)


def solve1p(nsys, np_, nblk, mat, rhs):
    """Periodic block-tridiagonal solve, lines batched over the first index."""
    _tri("solve1p", (nsys, np_), np_, nsys, nblk, mat, rhs)


"""Host-side mirror of the nonlinear two-dimensional driver (src/impdrv.f90).

:class:`ImpDrv2D` owns one device context of the C ABI (``lns_ctx2d_*`` in
``include/lns3d_gb300.h``): the deck values, the metrics and the far field
of the top boundary (``bnt``, ``top.pot``).  The state ``v`` is the Fortran
array ``v(5,nx,ny)`` (rho, u, v, w, T): a numpy float64 array (host memory,
staged like the Fortran call) or a CUDA torch float64 tensor (device
memory, enqueued on torch's current stream).  Every call runs the sm_103a
kernels of ``lib/liblns3d_gb300.so``; there is no CPU fallback.
"""
import ctypes

import numpy as np

from ._lib import Params2D, check, lib

FIELDS = {"Ah": 0, "Bh": 1, "Dh": 2, "Vh11": 3, "Vh12": 4, "Vh22": 5, "dtl": 6}
METRICS = ("m1", "m2", "n1", "n2", "m11", "m12", "m22", "n11", "n12", "n22")


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class ImpDrv2D:
    """One nonlinear 2D problem resident on the current GPU.

    params: dict with nx, ny, dxi, deta, Ma, Re, Pr, gamma, alfa, xper, yper,
    navier, wall, wallt, top, optx, opty (and left, right with xper = 0);
    metrics: the ten (nx, ny) arrays; bnt: (nx, 2) unit normal of the top
    boundary; pot: (5, nx) top.pot rows.
    """

    def __init__(self, params, metrics, bnt, pot, cflmax=1.0, dtmax=1e30, loctime=0, theta=0.0,
                 ilhs=1, impl=1, ispg=0, spg=None, spg2=None, eps_e=0.0, buff=None, left_far=None,
                 right_far=None, extrap=-1, nbl=0, update_nbl=False):
        """ilhs: the reference's iLHS switch, 1 = fourth-order LHS with
        pentadiagonal solves, 0 = second-order LHS with block-tridiagonal
        solves (src/impdrv.f90:307-344).  impl: time scheme, 1 backward
        Euler, 2 two-step backward, 3 midpoint (src/impdrv.f90:186-279).
        ispg (0 or 2), spg, spg2: the sponge towards the free stream; eps_e,
        buff: the explicit smoother and implicit damping (buff ones when
        None).  With a non-periodic xi direction: left_far, right_far the
        (bn (ny, 2), pot (5, ny)) far fields of Riemann planes (bnl / bnr of
        src/gengrid.f90, left.pot / right.pot); extrap, nbl, update_nbl the
        extrapolation of the right plane over the viscous layer (the deck's
        extrap and the &extras namelist's nbl and update_nbl)."""
        if ilhs not in (0, 1):
            raise ValueError("ilhs must be 0 or 1")
        if impl not in (1, 2, 3):
            raise ValueError("impl must be 1, 2 or 3")
        p = params
        self.nx, self.ny = int(p["nx"]), int(p["ny"])
        prm = Params2D(nx=self.nx, ny=self.ny, dxi=p["dxi"], deta=p["deta"], Ma=p["Ma"], Re=p["Re"], Pr=p["Pr"],
                       gamma=p["gamma"], gamma1=p.get("gamma1", 0.0), alfa=p["alfa"], cflmax=cflmax, dtmax=dtmax,
                       theta=theta, loctime=loctime, xper=p["xper"], yper=p["yper"], navier=p["navier"],
                       wall=p["wall"], wallt=p["wallt"], top=p["top"], optx=p["optx"], opty=p["opty"],
                       lhs_order=2 if ilhs == 0 else 4, impl=impl, ispg=ispg, eps_e=eps_e,
                       left=p.get("left", -1), right=p.get("right", -1), extrap=extrap, nbl=nbl,
                       update_nbl=int(bool(update_nbl)))
        self._ctx = ctypes.c_void_p()
        check(lib().lns_ctx2d_create(ctypes.byref(prm), ctypes.byref(self._ctx)), "lns_ctx2d_create")
        m = np.empty((self.nx, self.ny, 10), order="F")
        for k, name in enumerate(METRICS):
            m[:, :, k] = metrics[name]
        check(lib().lns_upload_metrics2d(self._ctx, ctypes.c_void_p(m.ctypes.data)), "lns_upload_metrics2d")
        b = np.asfortranarray(bnt, dtype=np.float64)
        q = np.asfortranarray(pot, dtype=np.float64)
        assert b.shape == (self.nx, 2) and q.shape == (5, self.nx)
        check(lib().lns_upload_top2d(self._ctx, ctypes.c_void_p(b.ctypes.data), ctypes.c_void_p(q.ctypes.data)),
              "lns_upload_top2d")
        for side, far in ((1, left_far), (2, right_far)):
            if far is None:
                continue
            fb = np.asfortranarray(far[0], dtype=np.float64)
            fq = np.asfortranarray(far[1], dtype=np.float64)
            assert fb.shape == (self.ny, 2) and fq.shape == (5, self.ny)
            check(lib().lns_upload_side2d(self._ctx, side, ctypes.c_void_p(fb.ctypes.data),
                                          ctypes.c_void_p(fq.ctypes.data)), "lns_upload_side2d")
        if ispg:
            s1 = np.asfortranarray(spg, dtype=np.float64)
            s2 = np.asfortranarray(spg2, dtype=np.float64)
            check(lib().lns_upload_sponge2d(self._ctx, ctypes.c_void_p(s1.ctypes.data),
                                            ctypes.c_void_p(s2.ctypes.data)), "lns_upload_sponge2d")
        if eps_e and buff is not None:
            bb = np.asfortranarray(buff, dtype=np.float64)
            check(lib().lns_upload_buffer2d(self._ctx, ctypes.c_void_p(bb.ctypes.data)), "lns_upload_buffer2d")

    @property
    def device_bytes(self):
        return lib().lns_ctx2d_bytes(self._ctx)

    def _dev(self, a, name):
        import torch

        n = 5 * self.nx * self.ny
        if not (_is_torch(a) and a.is_cuda and a.dtype == torch.float64 and a.is_contiguous() and a.numel() == n):
            raise ValueError("%s must be a contiguous CUDA float64 tensor of %d elements" % (name, n))
        return ctypes.c_void_p(a.data_ptr())

    def itrbc(self, v):
        """itrBC on v in place (src/itrbc.f90): the reference applies it once
        before the step loop (src/impdrv.f90:160).  A host v is staged
        through the device."""
        if _is_torch(v):
            check(lib().lns_itrbc2d_dev(self._ctx, self._dev(v, "v"), _stream()), "lns_itrbc2d_dev")
            return
        import torch

        t = torch.from_numpy(np.asarray(v).ravel(order="F")).cuda()
        check(lib().lns_itrbc2d_dev(self._ctx, self._dev(t, "v"), _stream()), "lns_itrbc2d_dev")
        v[...] = t.cpu().numpy().reshape(v.shape, order="F")

    def step(self, v, nsteps=1, niter=1, totres=None):
        """Advance v in place by nsteps implicit steps of niter correctors;
        host v returns the per-step residuals."""
        if _is_torch(v):
            pt = ctypes.c_void_p(totres.data_ptr()) if totres is not None else None
            check(lib().lns_step2d_dev(self._ctx, self._dev(v, "v"), nsteps, niter, pt, _stream()), "lns_step2d_dev")
            return None
        if not isinstance(v, np.ndarray) or v.dtype != np.float64 or v.size != 5 * self.nx * self.ny \
                or not v.flags.f_contiguous:
            raise ValueError("v must be a Fortran-ordered float64 array of shape (5, nx, ny)")
        res = np.zeros(max(nsteps, 1))
        check(lib().lns_step2d(self._ctx, ctypes.c_void_p(v.ctypes.data), nsteps, niter,
                               ctypes.c_void_p(res.ctypes.data)), "lns_step2d")
        return res[:nsteps]

    def rhs(self, v, vold, r, totres=None):
        """set_time_step(v), r = rhsBC(rbe(genmtrx(v))) on device tensors."""
        pt = ctypes.c_void_p(totres.data_ptr()) if totres is not None else None
        check(lib().lns_rhs2d_dev(self._ctx, self._dev(v, "v"), self._dev(vold, "vold"), self._dev(r, "r"), pt,
                                  _stream()), "lns_rhs2d_dev")

    def lhs(self, direction, v, mat):
        if mat.numel() != 125 * self.nx * self.ny or not mat.is_cuda:
            raise ValueError("mat must be a CUDA tensor of 125*nx*ny float64 entries")
        check(lib().lns_lhs2d_dev(self._ctx, direction, self._dev(v, "v"), ctypes.c_void_p(mat.data_ptr()),
                                  _stream()), "lns_lhs2d_dev")

    def field(self, name):
        shape = {0: (5, 5), 1: (5, 5), 2: (5, 5), 6: ()}.get(FIELDS[name], (6,))
        out = np.zeros(shape + (self.nx, self.ny), order="F")
        check(lib().lns_get_field2d(self._ctx, FIELDS[name], ctypes.c_void_p(out.ctypes.data)), "lns_get_field2d")
        return out

    def close(self):
        if self._ctx:
            lib().lns_ctx2d_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

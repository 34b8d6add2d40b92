"""ctypes harness of the nonlinear 2D step oracle (oracle/impdrv2d_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/ as the checker and by bench.py's
CPU-baseline leg (with the OpenMP build, liborc_omp.so)."""
import ctypes

import numpy as np

from . import orc
from .adi3d import A3Grid, A3Ops, _lib as _lib3

D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p


class A2Grid(ctypes.Structure):
    _fields_ = [("g", A3Grid), ("theta", D), ("bnt", P), ("rhobt", P), ("ubt", P), ("vbt", P), ("wbt", P),
                ("tbt", P)]


def _lib(L=None):
    L = _lib3(L if L is not None else orc())
    if not hasattr(L, "_a2_setup"):
        G = ctypes.POINTER(A2Grid)
        L.a2_genmtrx.argtypes = [G, P, ctypes.POINTER(A3Ops), P]
        L.a2_rbe.argtypes = [G, P, P, P, P]
        L.a2_rhsbc.argtypes = [G, P, P]
        L.a2_itrbc.argtypes = [G, P]
        L.a2_resstat.argtypes = [G, P, P]
        L.a2_resstat.restype = D
        L.a2_lhs.argtypes = [G, ctypes.POINTER(A3Ops), P, P, I, P]
        L.a2_step.argtypes = [G, I, P, P, P, ctypes.POINTER(A3Ops), P, P, P, P]
        L.a2_step.restype = D
        L.a2_lhs2.argtypes = [G, ctypes.POINTER(A3Ops), P, P, I, P, P]
        L.a2_step2.argtypes = [G, I, P, P, P, ctypes.POINTER(A3Ops), P, P, P, P]
        L.a2_step2.restype = D
        L.a2_step_impl.argtypes = [G, I, I, ctypes.c_long, I, P, P, P, P, P, ctypes.POINTER(A3Ops), P, P, P, P, P,
                                   P]
        L.a2_step_impl.restype = D
        L._a2_setup = True
    return L


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class Oracle2D:
    """Grid struct, operator storage and scratch of the oracle for one case."""

    def __init__(self, case, cflmax=1.0, loctime=0, dtmax=1e30, lib=None, ilhs=1, impl=1,
                 ispg=0, spg=None, spg2=None, eps_e=0.0, buff=None):
        """ilhs = 1: fourth-order LHS, pentadiagonal solves; ilhs = 0:
        second-order LHS, block-tridiagonal solves (src/impdrv.f90:307-344).
        impl: time scheme 1 (backward Euler), 2 (two-step backward), 3
        (midpoint), src/impdrv.f90:186-279; steps are counted from creation.
        ispg = 2, spg, spg2: the sponge towards the free stream
        (src/genmtrx.f90:436-446); eps_e, buff: the explicit smoother and
        implicit damping (buff ones when None)."""
        if ispg not in (0, 2):
            raise ValueError("the nonlinear 2D step supports ispg 0 or 2")
        self.L = _lib(lib)
        self.ilhs, self.impl, self.lstep = ilhs, impl, 0
        p = case["params"]
        self.nx, self.ny = nx, ny = p["nx"], p["ny"]
        self.keep = {k: np.asfortranarray(v, dtype=np.float64) for k, v in case["metrics"].items()}
        pot = np.asfortranarray(case["pot"], dtype=np.float64)
        self.pot = {k: np.ascontiguousarray(pot[i]) for i, k in enumerate(("rhobt", "ubt", "vbt", "wbt", "tbt"))}
        self.bnt = np.asfortranarray(case["bnt"], dtype=np.float64)
        g3 = A3Grid(cflmax=cflmax, dtmax=dtmax, loctime=loctime,
                    **{k: p[k] for k in ("nx", "ny", "dxi", "deta", "Ma", "Re", "Pr", "gamma", "gamma1", "omega",
                                         "kz", "alfa", "xper", "yper", "navier", "wall", "wallt", "top", "optx",
                                         "opty")},
                    **{k: ptr(v).value for k, v in self.keep.items()})
        if ispg:
            self.spg = np.asfortranarray(spg, dtype=np.float64).reshape((nx, ny), order="F")
            self.spg2 = np.asfortranarray(spg2, dtype=np.float64).reshape((nx, ny), order="F")
            g3.ispg, g3.spg, g3.spg2 = ispg, ptr(self.spg).value, ptr(self.spg2).value
        if eps_e:
            self.buff = np.asfortranarray(buff if buff is not None else np.ones((nx, ny)),
                                          dtype=np.float64).reshape((nx, ny), order="F")
            g3.eps_e, g3.buff = eps_e, ptr(self.buff).value
        self.g = A2Grid(g=g3, theta=case.get("theta", 0.0), bnt=ptr(self.bnt).value,
                        **{k: ptr(v).value for k, v in self.pot.items()})
        self.ops = {k: np.zeros((5, 5, nx, ny), order="F") for k in ("Ah", "Bh", "Dh", "Dhi")}
        self.ops.update({k: np.zeros((6, nx, ny), order="F") for k in ("Vh11", "Vh12", "Vh22", "ABhi")})
        self.o = A3Ops(**{k: ptr(v).value for k, v in self.ops.items()})
        self.dtl = np.zeros((nx, ny), order="F")
        self.r = np.zeros((5, nx, ny), order="F")
        self.vold = np.zeros((5, nx, ny), order="F")
        self.mat = np.zeros((5, 5, 5, nx, ny), order="F")
        self.per = np.zeros((2, 5, 5, nx, ny), order="F")
        self.v2old = np.zeros((5, nx, ny), order="F")
        self.w = np.zeros((5, nx, ny), order="F")
        self.mat3 = np.zeros((3, 5, 5, nx, ny), order="F")
        self.bc = np.zeros((14, 5, 5, nx), order="F")
        self.cfl = ctypes.c_double(0.0)

    def itrbc(self, v):
        self.L.a2_itrbc(ctypes.byref(self.g), ptr(v))

    def step(self, v, niter=1):
        if self.impl != 1:
            res = self.L.a2_step_impl(ctypes.byref(self.g), self.ilhs, self.impl, self.lstep, niter, ptr(v),
                                      ptr(self.vold), ptr(self.v2old), ptr(self.w), ptr(self.r),
                                      ctypes.byref(self.o), ptr(self.dtl), ptr(self.mat), ptr(self.per),
                                      ptr(self.mat3), ptr(self.bc), ctypes.byref(self.cfl))
            self.lstep += 1
            return res
        if self.ilhs == 0:
            return self.L.a2_step2(ctypes.byref(self.g), niter, ptr(v), ptr(self.vold), ptr(self.r),
                                   ctypes.byref(self.o), ptr(self.dtl), ptr(self.mat3), ptr(self.bc),
                                   ctypes.byref(self.cfl))
        return self.L.a2_step(ctypes.byref(self.g), niter, ptr(v), ptr(self.vold), ptr(self.r), ctypes.byref(self.o),
                              ptr(self.dtl), ptr(self.mat), ptr(self.per), ctypes.byref(self.cfl))

    def genmtrx(self, v):
        r = np.zeros_like(v)
        assert self.L.a2_genmtrx(ctypes.byref(self.g), ptr(v), ctypes.byref(self.o), ptr(r)) == 0
        return r

    def rhs(self, v, vold, dtl):
        """r = rhsBC(rbe(genmtrx(v))) and its resstat value."""
        r = self.genmtrx(v)
        self.L.a2_rbe(ctypes.byref(self.g), ptr(r), ptr(v), ptr(vold), ptr(dtl))
        self.L.a2_rhsbc(ctypes.byref(self.g), ptr(r), ptr(v))
        return r, self.L.a2_resstat(ctypes.byref(self.g), ptr(r), ptr(dtl))

    def lhs(self, v, dtl, direction):
        """LHS of a sweep for the operators of the last genmtrx call."""
        mat = np.zeros((5, 5, 5, self.nx, self.ny), order="F")
        assert self.L.a2_lhs(ctypes.byref(self.g), ctypes.byref(self.o), ptr(dtl), ptr(v), direction, ptr(mat)) == 0
        return mat

    def lhs2(self, v, dtl, direction):
        """Second-order LHS of a sweep: (mat(3,5,5,nx,ny), bc(14,5,5,nlines))."""
        mat = np.zeros((3, 5, 5, self.nx, self.ny), order="F")
        bc = np.zeros((14, 5, 5, self.ny if direction == 1 else self.nx), order="F")
        assert self.L.a2_lhs2(ctypes.byref(self.g), ctypes.byref(self.o), ptr(dtl), ptr(v), direction, ptr(mat),
                              ptr(bc)) == 0
        return mat, bc

"""ctypes harness of the linear ADI step oracle (oracle/adi3d_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/ as the checker and by bench.py's
CPU-baseline leg (with the OpenMP build, liborc_omp.so)."""
import ctypes

import numpy as np

from . import orc

D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p


class A3Grid(ctypes.Structure):
    _fields_ = [("nx", I), ("ny", I), ("dxi", D), ("deta", D), ("Ma", D), ("Re", D), ("Pr", D), ("gamma", D),
                ("gamma1", D), ("omega", D), ("kz", D), ("alfa", D), ("cflmax", D), ("dtmax", D),
                ("loctime", I), ("xper", I), ("yper", I), ("navier", I), ("wall", I), ("wallt", I), ("top", I),
                ("optx", I), ("opty", I)] + [(k, P) for k in
                                             ("m1", "m2", "n1", "n2", "m11", "m12", "m22", "n11", "n12", "n22")] + \
        [("ispg", I), ("spg", P), ("spg2", P), ("eps_e", D), ("buff", P), ("vm", P), ("xc", P),
         ("wamp", P), ("x0", D), ("cvic", P), ("bump", P)]


class A3Ops(ctypes.Structure):
    _fields_ = [(k, P) for k in ("Ah", "Bh", "Dh", "Dhi", "Vh11", "Vh12", "Vh22", "ABhi")]


def _lib(L=None):
    L = L if L is not None else orc()
    if not hasattr(L, "_a3_setup"):
        L.a3_genmtrx.argtypes = [ctypes.POINTER(A3Grid), P, ctypes.POINTER(A3Ops)]
        L.a3_set_time_step.argtypes = [ctypes.POINTER(A3Grid), P, P]
        L.a3_set_time_step.restype = D
        L.a3_deriv1.argtypes = [ctypes.POINTER(A3Grid), I, P, P, P]
        L.a3_deriv2.argtypes = [ctypes.POINTER(A3Grid), I, P, P, P, P, P]
        L.a3_lrhs.argtypes = [ctypes.POINTER(A3Grid), ctypes.POINTER(A3Ops), P, P]
        L.a3_rbe.argtypes = [ctypes.POINTER(A3Grid), P, P, P, P]
        L.a3_rhsbc.argtypes = [ctypes.POINTER(A3Grid), P, P]
        L.a3_resstat.argtypes = [ctypes.POINTER(A3Grid), P, P]
        L.a3_resstat.restype = D
        L.a3_itrbc.argtypes = [ctypes.POINTER(A3Grid), P]
        L.a3_lhs.argtypes = [ctypes.POINTER(A3Grid), ctypes.POINTER(A3Ops), P, I, P]
        L.a3_step.argtypes = [ctypes.POINTER(A3Grid), ctypes.POINTER(A3Ops), P, I, P, P, P, P, P, P, P, P, P,
                              ctypes.POINTER(I)]
        L.a3_step.restype = D
        L.a3_step_impl.argtypes = [ctypes.POINTER(A3Grid), ctypes.POINTER(A3Ops), P, I, I, I, P, P, P, P, P, P, P, P,
                                   P, P, P, ctypes.POINTER(D)]
        L.a3_step_impl.restype = D
        L._a3_setup = True
    return L


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class Oracle3D:
    """Holds the oracle's grid struct, operators and factor arrays for one case."""

    def __init__(self, case, cflmax=1.0, loctime=1, dtmax=1e30, lib=None, ispg=0, spg=None,
                 spg2=None, eps_e=0.0, buff=None, x0=0.0, wamp=None, cvic=None, bump=None):
        """ispg, spg, spg2: the sponge (0 none, 1 spg, > 4 spg + spg2), spg
        and spg2 (nx, ny) as the reference's sponge setup leaves them.
        eps_e, buff: the explicit smoother and implicit damping, buff (nx, ny)
        (ones, the reference's ibuff = 0, when None).  The inflow sponges
        (ispg 2, 3) use the case's x coordinates, x0 and (ispg 3) wamp (nx);
        the eigenfunction sponge (ispg 4) its target cvic, complex (5, nx, ny)."""
        self.L = _lib(lib)
        self.case = case
        p = case["params"]
        self.nx, self.ny = p["nx"], p["ny"]
        self.keep = {k: np.asfortranarray(v, dtype=np.float64) for k, v in case["metrics"].items()}
        self.g = A3Grid(cflmax=cflmax, dtmax=dtmax, loctime=loctime,
                        **{k: p[k] for k in ("nx", "ny", "dxi", "deta", "Ma", "Re", "Pr", "gamma", "gamma1",
                                             "omega", "kz", "alfa", "xper", "yper", "navier", "wall", "wallt",
                                             "top", "optx", "opty")},
                        **{k: ptr(v).value for k, v in self.keep.items()})
        nx, ny = self.nx, self.ny
        if ispg:
            self.spg = np.asfortranarray(spg, dtype=np.float64).reshape((nx, ny), order="F")
            self.spg2 = np.asfortranarray(spg2 if spg2 is not None else np.zeros((nx, ny)),
                                          dtype=np.float64).reshape((nx, ny), order="F")
            self.g.ispg, self.g.spg, self.g.spg2 = ispg, ptr(self.spg).value, ptr(self.spg2).value
        if ispg or p["top"] == 1:
            self._vm = np.asfortranarray(case["vm"], dtype=np.float64)
            self._xc = np.asfortranarray(case["x"], dtype=np.float64)
            self._wamp = np.ascontiguousarray(wamp if wamp is not None else np.ones(nx), dtype=np.float64)
            self._cvic = np.asfortranarray(cvic if cvic is not None else np.zeros((5, nx, ny)), dtype=np.complex128)
            self.g.vm, self.g.xc, self.g.wamp = ptr(self._vm).value, ptr(self._xc).value, ptr(self._wamp).value
            self.g.x0, self.g.cvic = x0, ptr(self._cvic).value
        if p["wall"] == 3:  # the bump wall's u1w, u2w, u3w, tw, twp, complex (5, nx)
            self._bump = np.asfortranarray(bump, dtype=np.complex128).reshape((5, nx), order="F")
            self.g.bump = ptr(self._bump).value
        if eps_e:
            self.buff = np.asfortranarray(buff if buff is not None else np.ones((nx, ny)),
                                          dtype=np.float64).reshape((nx, ny), order="F")
            self.g.eps_e, self.g.buff = eps_e, ptr(self.buff).value
        self.ops = {k: np.zeros((5, 5, nx, ny), order="F") for k in ("Ah", "Bh", "Dh", "Dhi")}
        self.ops.update({k: np.zeros((6, nx, ny), order="F") for k in ("Vh11", "Vh12", "Vh22", "ABhi")})
        self.o = A3Ops(**{k: ptr(v).value for k, v in self.ops.items()})
        self.vm = np.asfortranarray(case["vm"], dtype=np.float64)
        L = self.L
        assert L.a3_genmtrx(ctypes.byref(self.g), ptr(self.vm), ctypes.byref(self.o)) == 0
        self.dtl = np.zeros((nx, ny), order="F")
        self.cfl = L.a3_set_time_step(ctypes.byref(self.g), ptr(self.vm), ptr(self.dtl))
        self.matx = np.zeros((5, 5, 5, nx, ny), np.complex128, order="F")
        self.maty = np.zeros((5, 5, 5, nx, ny), np.complex128, order="F")
        self.perx = np.zeros((2, 5, 5, nx, ny), np.complex128, order="F")
        self.per2x = np.zeros((2, 5, 5, nx, ny), np.complex128, order="F")
        self.pery = np.zeros((2, 5, 5, nx, ny), np.complex128, order="F")
        self.per2y = np.zeros((2, 5, 5, nx, ny), np.complex128, order="F")
        self.r = np.zeros((5, nx, ny), np.complex128, order="F")
        self.factored = I(0)

    def itrbc(self, v):
        """itrBC3D on v in place (src/itrbc3d.f90)."""
        self.L.a3_itrbc(ctypes.byref(self.g), ptr(v))

    def step_impl(self, v, impl, niter=1):
        """One step of time scheme impl (1, 2, 3) on v in place; vold,
        v2old and the step count carry over between calls (src/impdrv3d.f90)"""
        if not hasattr(self, "_lstep"):
            self._lstep = 0
            self._vold = np.zeros_like(v)
            self._v2old = np.zeros_like(v)
            self._w = np.zeros_like(v)
            self._alfa_fac = D(-1.0)
        res = self.L.a3_step_impl(ctypes.byref(self.g), ctypes.byref(self.o), ptr(self.dtl), niter, impl,
                                  self._lstep, ptr(v), ptr(self._vold), ptr(self._v2old), ptr(self._w), ptr(self.r),
                                  ptr(self.matx), ptr(self.maty), ptr(self.perx), ptr(self.per2x),
                                  ptr(self.pery), ptr(self.per2y), ctypes.byref(self._alfa_fac))
        self._lstep += 1
        return res

    def step(self, v, niter=1):
        vold = np.zeros_like(v)
        return self.L.a3_step(ctypes.byref(self.g), ctypes.byref(self.o), ptr(self.dtl), niter, ptr(v), ptr(vold),
                              ptr(self.r), ptr(self.matx), ptr(self.maty), ptr(self.perx), ptr(self.per2x),
                              ptr(self.pery), ptr(self.per2y), ctypes.byref(self.factored))

    def lrhs(self, v):
        r = np.zeros_like(v)
        assert self.L.a3_lrhs(ctypes.byref(self.g), ctypes.byref(self.o), ptr(v), ptr(r)) == 0
        return r

    def lhs(self, direction):
        mat = np.zeros((5, 5, 5, self.nx, self.ny), np.complex128, order="F")
        assert self.L.a3_lhs(ctypes.byref(self.g), ctypes.byref(self.o), ptr(self.dtl), direction, ptr(mat)) == 0
        return mat

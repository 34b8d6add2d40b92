"""CPU checker libraries (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package.  It loads ``liborc_penta.so`` (the restatement of the
reference line solvers and of the linear 3D step), ``liborc_omp.so`` (the
same sources built for speed with OpenMP) and, where built, ``_ref/libref_penta.so`` (the
reference's own solver sources translated by f77sub2c.py).
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_PATH = os.path.join(HERE, "liborc_penta.so")
ORC_OMP_PATH = os.path.join(HERE, "liborc_omp.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_penta.so")
REF_FAST_PATH = os.path.join(HERE, "_ref", "libref_penta_fast.so")

COMPAT_PERIODIC_SLOT = 1
COMPAT_CBC_RHS = 2

_orc = {}
_ref = {}


def _load(path):
    if path not in _orc:
        if not os.path.exists(path):
            raise ImportError("oracle not built: make -C oracle")
        L = ctypes.CDLL(path)
        i, p = ctypes.c_int, ctypes.c_void_p
        L.orc_penta_bc.argtypes = [i, i, i, p, p]
        L.orc_penta_p.argtypes = [i, i, i, p, p, p, i]
        L.orc_cpenta_bc.argtypes = [i, i, i, p, p, i, i]
        L.orc_cpenta_p.argtypes = [i, i, i, p, p, p, p, i, i]
        L.orc_oob_count.restype = ctypes.c_long
        L.orc_tri_bc.argtypes = [i, i, i, p, p, p]
        L.orc_tri_p.argtypes = [i, i, i, p, p]
        _orc[path] = L
    return _orc[path]


def orc():
    """The parity build of the restatement (serial, no contraction)."""
    return _load(ORC_PATH)


def orc_omp():
    """The same restatement built -O3 -fopenmp: the timed CPU baseline."""
    return _load(ORC_OMP_PATH)


def ref(fast=False):
    """The translated reference solvers, or None where they were not built."""
    path = REF_FAST_PATH if fast else REF_PATH
    if path not in _ref:
        if not os.path.exists(path):
            _ref[path] = None
        else:
            L = ctypes.CDLL(path)
            i, p = ctypes.c_int, ctypes.c_void_p
            for nm in ("penta1bc", "penta2bc"):
                getattr(L, "ref_" + nm).argtypes = [i, i, i, p, p]
            for nm in ("penta1p", "penta2p"):
                getattr(L, "ref_" + nm).argtypes = [i, i, i, p, p, p, p]
            for nm in ("cpenta1bc", "cpenta2bc"):
                getattr(L, "ref_" + nm).argtypes = [i, i, i, p, p, i]
            for nm in ("cpenta1p", "cpenta2p"):
                getattr(L, "ref_" + nm).argtypes = [i, i, i, p, p, p, p, i]
            if hasattr(L, "ref_solve2bc"):  # the block-tridiagonal solvers
                for nm in ("solve1bc", "solve2bc"):
                    getattr(L, "ref_" + nm).argtypes = [i, i, i, p, p, p]
                for nm in ("solve1p", "solve2p"):
                    getattr(L, "ref_" + nm).argtypes = [i, i, i, p, p, p, p]
            _ref[path] = L
    return _ref[path]


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data)

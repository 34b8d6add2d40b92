"""ctypes driver of the translated reference (oracle/_ref/libref_step.so).

TEST INFRASTRUCTURE ONLY: the reference's own Fortran step routines and main
program, translated to C by oracle/f90sub2c.py and linked with
oracle/ref_harness.c, run here as the checker of the hand restatements and,
through committed golden files, of the GPU path.

Two ways to use it:

* ``RefProgram.run(rundir, deck)`` runs the reference program (src/lns3d.f90)
  as ``lns3d < deck`` in ``rundir``: it reads grid.dat, metric.dat, mean.dat,
  output.R.N and *.pot there and writes the history (output.h.N, the numeric
  items at full precision) and the restart files, exactly as the reference.
* ``RefProgram.call(name, *args)`` calls one translated routine; module
  variables are read and set with ``get``/``set``/``array``.

The reference keeps its state in module variables and SAVEd locals, so every
RefProgram loads its own copy of the library: instances never share state.
"""
import ctypes
import os
import shutil
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libref_step.so")
# the same program without the correction of the complex boundary solvers'
# row n-3 index fault (src/cpenta1bc.f:675, src/cpenta2bc.f:676)
LIB_ASIS = os.path.join(HERE, "_ref", "libref_step_asis.so")

# the reference's metric pre-processor (pre/src_ij/pre.f90 and its grad,
# grad2, stencil, wdata), translated the same way
LIB_PRE = os.path.join(HERE, "_ref", "libref_pre.so")

TYPES = {0: ctypes.c_int, 1: ctypes.c_double, 4: ctypes.c_float}


class FDesc(ctypes.Structure):
    _fields_ = [("p", ctypes.c_void_p), ("rank", ctypes.c_int), ("owned", ctypes.c_int),
                ("lb", ctypes.c_long * 7), ("n", ctypes.c_long * 7), ("st", ctypes.c_long * 7)]


class RefProc(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("fn", ctypes.c_void_p), ("nargs", ctypes.c_int),
                ("sig", ctypes.c_char_p)]


def available(asis=False):
    return os.path.exists(LIB_ASIS if asis else LIB)


class RefError(RuntimeError):
    pass


class RefProgram:
    def __init__(self, asis=False, lib=None):
        """asis: the reference exactly as written, without the correction of
        the complex boundary solvers' row n-3 index fault.  lib: another
        translated program (e.g. LIB_PRE) instead of the step program."""
        src = lib or (LIB_ASIS if asis else LIB)
        if not os.path.exists(src):
            raise RefError("%s is not built (the reference sources are needed to translate it)"
                           % os.path.relpath(src, os.path.dirname(HERE)))
        self._tmp = tempfile.mkdtemp(prefix="refstep_")
        path = os.path.join(self._tmp, "libref.so")
        shutil.copy(src, path)   # a private copy: its own module state
        self.L = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
        L = self.L
        L.ref_call.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        L.ref_call.restype = ctypes.c_int
        L.ref_last_message.restype = ctypes.c_char_p
        L.ref_scalar.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        L.ref_scalar.restype = ctypes.c_void_p
        L.ref_array.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        L.ref_array.restype = ctypes.POINTER(FDesc)
        L.ref_proc_find.argtypes = [ctypes.c_char_p]
        L.ref_proc_find.restype = ctypes.POINTER(RefProc)
        L.ref_set_dir.argtypes = [ctypes.c_char_p]
        L.ref_set_stdin.argtypes = [ctypes.c_char_p]
        L.ref_set_swap.argtypes = [ctypes.c_int]
        L.ref_get_oob.restype = ctypes.c_long
        L.ref_get_dim.restype = ctypes.c_long
        L.ref_init()
        self._keep = []

    def close(self):
        shutil.rmtree(self._tmp, ignore_errors=True)

    # ---- module variables --------------------------------------------------

    def _scalar(self, name):
        t = ctypes.c_int()
        addr = self.L.ref_scalar(name.lower().encode(), ctypes.byref(t))
        if not addr:
            raise KeyError(name)
        return addr, t.value

    def get(self, name):
        addr, t = self._scalar(name)
        if t == 2:
            c = (ctypes.c_double * 2).from_address(addr)
            return complex(c[0], c[1])
        if t == 3:
            return ctypes.string_at(addr).decode().rstrip()
        return TYPES[t].from_address(addr).value

    def set(self, name, value):
        addr, t = self._scalar(name)
        if t == 2:
            c = (ctypes.c_double * 2).from_address(addr)
            c[0], c[1] = value.real, value.imag
        elif t == 3:
            raise KeyError("character variables are not set from Python")
        else:
            TYPES[t].from_address(addr).value = value

    def array(self, name):
        """A numpy view (Fortran order) of an allocated module array."""
        t = ctypes.c_int()
        d = self.L.ref_array(name.lower().encode(), ctypes.byref(t))
        if not d:
            raise KeyError(name)
        d = d.contents
        if not d.p:
            return None
        shape = tuple(d.n[k] for k in range(d.rank))
        dt = {0: np.int32, 1: np.float64, 2: np.complex128, 4: np.float32}[t.value]
        n = int(np.prod(shape))
        buf = (ctypes.c_char * (n * np.dtype(dt).itemsize)).from_address(d.p)
        return np.frombuffer(buf, dtype=dt).reshape(shape, order="F")

    def bind(self, name, arr):
        """Point a module allocatable at a caller array (kept alive here)."""
        t = ctypes.c_int()
        d = self.L.ref_array(name.lower().encode(), ctypes.byref(t)).contents
        arr = np.asfortranarray(arr)
        self._keep.append(arr)
        d.p = arr.ctypes.data
        d.rank = arr.ndim
        d.owned = 0
        st = 1
        for k in range(arr.ndim):
            d.lb[k] = 1
            d.n[k] = arr.shape[k]
            d.st[k] = st
            st *= arr.shape[k]
        return arr

    # ---- procedures ----------------------------------------------------------

    def call(self, name, *args):
        """Call a translated routine.  Arrays are passed by address (they must
        be Fortran-ordered numpy arrays of the dummy's type); Python scalars
        are converted to the dummy's type and passed by reference, and the
        values they hold after the call are returned in a list."""
        p = self.L.ref_proc_find(name.lower().encode())
        if not p:
            raise KeyError(name)
        p = p.contents
        sig = p.sig.decode()
        if len(args) != p.nargs:
            raise TypeError("%s takes %d arguments" % (name, p.nargs))
        ptrs = (ctypes.c_void_p * max(1, len(args)))()
        cells = []
        for k, (a, ch) in enumerate(zip(args, sig)):
            if ch in "ILDFZ":
                if not (isinstance(a, np.ndarray) and a.flags.f_contiguous):
                    raise TypeError("argument %d of %s must be a Fortran-ordered array" % (k + 1, name))
                ptrs[k] = a.ctypes.data
                cells.append(None)
            elif ch in "il":
                c = ctypes.c_int(int(a))
                cells.append(c)
                ptrs[k] = ctypes.addressof(c)
            elif ch == "d":
                c = ctypes.c_double(float(a))
                cells.append(c)
                ptrs[k] = ctypes.addressof(c)
            elif ch == "z":
                c = (ctypes.c_double * 2)(complex(a).real, complex(a).imag)
                cells.append(c)
                ptrs[k] = ctypes.addressof(c)
            elif ch == "c":
                c = ctypes.create_string_buffer(str(a).encode(), 256)
                cells.append(c)
                ptrs[k] = ctypes.addressof(c)
            else:
                raise TypeError("argument kind %s of %s is not supported from Python" % (ch, name))
        st = self.L.ref_call(p.fn, len(args), ptrs)
        if st != 0:
            raise RefError("%s: %s" % (name, self.L.ref_last_message().decode()))
        out = []
        for c, ch in zip(cells, sig):
            if c is None:
                out.append(None)
            elif ch in "il":
                out.append(c.value)
            elif ch == "d":
                out.append(c.value)
            elif ch == "z":
                out.append(complex(c[0], c[1]))
            else:
                out.append(c.value.decode())
        return out

    def oob(self):
        """Accesses outside an array's storage made so far (skipped)."""
        return self.L.ref_get_oob()

    def transposed(self):
        """Accesses with a subscript outside its dimension that still fell
        inside the array's storage (performed, as compiled Fortran does)."""
        return self.L.ref_get_dim()

    # ---- the program -------------------------------------------------------

    def run(self, rundir, deck, swap=False, program="lns3d"):
        """Run the reference program as ``lns3d < deck`` in rundir."""
        self.L.ref_set_dir(os.path.abspath(rundir).encode())
        self.L.ref_set_stdin(deck.encode())
        self.L.ref_set_swap(1 if swap else 0)
        p = self.L.ref_proc_find(program.encode()).contents
        st = self.L.ref_call(p.fn, 0, (ctypes.c_void_p * 1)())
        msg = self.L.ref_last_message().decode()
        if st not in (0, 2):        # 2: the program's own STOP
            raise RefError(program + ": " + msg)
        return msg

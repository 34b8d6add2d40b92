"""ctypes binding of lib/liblns3d_gb300.so (the C ABI in include/lns3d_gb300.h).

The library is the only compute path: importing this module fails loudly
when it has not been built, and nothing here falls back to CPU code.
"""
import ctypes
import os

from ._build import LIBDIR, LIBNAME

LNS_OK, LNS_ERR_ARG, LNS_ERR_CUDA, LNS_ERR_PIVOT, LNS_ERR_NOMEM = 0, 1, 2, 3, 4
_NAMES = {1: "LNS_ERR_ARG", 2: "LNS_ERR_CUDA", 3: "LNS_ERR_PIVOT", 4: "LNS_ERR_NOMEM"}


class LnsError(RuntimeError):
    """A non-zero status returned by the C ABI."""

    def __init__(self, code, where, message):
        self.code = code
        super().__init__("%s failed with %s: %s" % (where, _NAMES.get(code, code), message))


def library_path():
    return os.path.join(LIBDIR, LIBNAME)


_lib = None
I32, P, DP = ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p

# name -> argument types (all return int)
SIGNATURES = {
    "lns_penta2bc": [I32, I32, I32, DP, DP],
    "lns_penta2bc_dev": [I32, I32, I32, DP, DP, P],
    "lns_penta1bc": [I32, I32, I32, DP, DP],
    "lns_penta1bc_dev": [I32, I32, I32, DP, DP, P],
    "lns_cpenta2bc": [I32, I32, I32, DP, DP, I32],
    "lns_cpenta2bc_dev": [I32, I32, I32, DP, DP, I32, P],
    "lns_cpenta1bc": [I32, I32, I32, DP, DP, I32],
    "lns_cpenta1bc_dev": [I32, I32, I32, DP, DP, I32, P],
    "lns_set_periodic_exact": [I32],
    "lns_solve2bc": [I32, I32, I32, DP, DP, DP],
    "lns_solve1bc": [I32, I32, I32, DP, DP, DP],
    "lns_solve2p": [I32, I32, I32, DP, DP, DP, DP],
    "lns_solve1p": [I32, I32, I32, DP, DP, DP, DP],
    "lns_solve2bc_dev": [I32, I32, I32, DP, DP, DP, P, P],
    "lns_solve1bc_dev": [I32, I32, I32, DP, DP, DP, P, P],
    "lns_solve2p_dev": [I32, I32, I32, DP, DP, P, P],
    "lns_solve1p_dev": [I32, I32, I32, DP, DP, P, P],
    "lns_penta2p": [I32, I32, I32, DP, DP, DP, DP],
    "lns_penta2p_dev": [I32, I32, I32, DP, DP, DP, DP, P],
    "lns_penta1p": [I32, I32, I32, DP, DP, DP, DP],
    "lns_penta1p_dev": [I32, I32, I32, DP, DP, DP, DP, P],
    "lns_cpenta2p": [I32, I32, I32, DP, DP, DP, DP, I32],
    "lns_cpenta2p_dev": [I32, I32, I32, DP, DP, DP, DP, I32, P],
    "lns_cpenta1p": [I32, I32, I32, DP, DP, DP, DP, I32],
    "lns_cpenta1p_dev": [I32, I32, I32, DP, DP, DP, DP, I32, P],
    "lns_cpenta2bc_mixed_dev": [I32, I32, I32, DP, DP, I32, I32, P, P],
    "lns_cpenta1bc_mixed_dev": [I32, I32, I32, DP, DP, I32, I32, P, P],
    "lns_cpenta2p_mixed_dev": [I32, I32, I32, DP, DP, I32, I32, P, P],
    "lns_cpenta1p_mixed_dev": [I32, I32, I32, DP, DP, I32, I32, P, P],
    "lns_penta2bc_mixed_dev": [I32, I32, I32, DP, DP, I32, P, P],
    "lns_penta1bc_mixed_dev": [I32, I32, I32, DP, DP, I32, P, P],
    "lns_cpenta2bc_mixed": [I32, I32, I32, DP, DP, I32],
    "lns_cpenta2bc_mixed_static_dev": [I32, I32, I32, DP, DP, I32, P],
    "lns_ctx3d_create": [P, P],
    "lns_ctx3d_destroy": [P],
    "lns_upload_metrics3d": [P, DP],
    "lns_upload_sponge3d": [P, DP, DP],
    "lns_upload_inflow3d": [P, DP, DP, ctypes.c_double],
    "lns_upload_sponge_target3d": [P, DP],
    "lns_upload_bump3d": [P, DP],
    "lns_upload_profile3d": [P, DP, DP, ctypes.c_double, ctypes.c_double],
    "lns_upload_buffer3d": [P, DP],
    "lns_upload_sponge2d": [P, DP, DP],
    "lns_upload_buffer2d": [P, DP],
    "lns_upload_mean3d": [P, DP, DP],
    "lns_step3d": [P, DP, I32, I32, DP],
    "lns_step3d_dev": [P, DP, I32, I32, DP, P],
    "lns_itrbc3d_dev": [P, DP, P],
    "lns_rhs3d_dev": [P, DP, DP, DP, DP, P],
    "lns_lhs3d_dev": [P, I32, DP, P],
    "lns_get_field3d": [P, I32, DP],
    "lns_lin2d_create": [P, P],
    "lns_lin2d_destroy": [P],
    "lns_lin2d_set_nbl": [P, I32],
    "lns_upload_metrics_lin2d": [P, DP],
    "lns_upload_mean_lin2d": [P, DP, DP],
    "lns_itrbc_lin2d_dev": [P, DP, P],
    "lns_get_dtl_lin2d": [P, DP],
    "lns_step_lin2d": [P, DP, I32, I32, DP],
    "lns_step_lin2d_dev": [P, DP, I32, I32, DP, P],
    "lns_ctx3d_profile": [P, I32],
    "lns_ctx3d_set_row_pairs": [P, I32],
    "lns_server3d_graph_captures": [P],
    "lns_ctx3d_profile_read": [P, DP, P],
    "lns_batch3d_create": [I32, P, P],
    "lns_batch3d_destroy": [P],
    "lns_batch3d_upload": [P, I32, DP, DP, DP],
    "lns_batch3d_tune": [P, I32, P],
    "lns_batch3d_run": [P, I32, I32, ctypes.c_double, I32, P, P],
    "lns_batch3d_get_state": [P, I32, DP],
    "lns_server3d_create": [ctypes.c_size_t, I32, I32, I32, P],
    "lns_server3d_destroy": [P],
    "lns_server3d_submit": [P, P, DP, DP, DP, ctypes.c_double, I32, P],
    "lns_server3d_tick": [P, I32, P, P],
    "lns_server3d_poll": [P, ctypes.c_int64, P, P, P, P],
    "lns_server3d_fetch": [P, ctypes.c_int64, DP],
    "lns_ctx2d_create": [P, P],
    "lns_ctx2d_destroy": [P],
    "lns_upload_metrics2d": [P, DP],
    "lns_upload_top2d": [P, DP, DP],
    "lns_upload_side2d": [P, I32, DP, DP],
    "lns_itrbc2d_dev": [P, DP, P],
    "lns_step2d": [P, DP, I32, I32, DP],
    "lns_step2d_dev": [P, DP, I32, I32, DP, P],
    "lns_rhs2d_dev": [P, DP, DP, DP, DP, P],
    "lns_lhs2d_dev": [P, I32, DP, DP, P],
    "lns_get_field2d": [P, I32, DP],
}


class Params2D(ctypes.Structure):
    """lns_params2d of include/lns3d_gb300.h."""
    _fields_ = [("nx", I32), ("ny", I32), ("dxi", ctypes.c_double), ("deta", ctypes.c_double),
                ("Ma", ctypes.c_double), ("Re", ctypes.c_double), ("Pr", ctypes.c_double),
                ("gamma", ctypes.c_double), ("gamma1", ctypes.c_double), ("alfa", ctypes.c_double),
                ("cflmax", ctypes.c_double), ("dtmax", ctypes.c_double), ("theta", ctypes.c_double), ("loctime", I32), ("xper", I32),
                ("yper", I32), ("navier", I32), ("wall", I32), ("wallt", I32), ("top", I32), ("optx", I32),
                ("opty", I32), ("lhs_order", I32), ("impl", I32), ("ispg", I32),
                ("eps_e", ctypes.c_double), ("left", I32), ("right", I32), ("extrap", I32), ("nbl", I32),
                ("update_nbl", I32)]


class Params3D(ctypes.Structure):
    """lns_params3d of include/lns3d_gb300.h."""
    _fields_ = [("nx", I32), ("ny", I32), ("dxi", ctypes.c_double), ("deta", ctypes.c_double),
                ("Ma", ctypes.c_double), ("Re", ctypes.c_double), ("Pr", ctypes.c_double),
                ("gamma", ctypes.c_double), ("gamma1", ctypes.c_double), ("omega", ctypes.c_double),
                ("beta", ctypes.c_double),
                ("alfa", ctypes.c_double), ("cflmax", ctypes.c_double), ("dtmax", ctypes.c_double),
                ("loctime", I32), ("xper", I32), ("yper", I32), ("navier", I32), ("wall", I32), ("wallt", I32),
                ("top", I32), ("optx", I32), ("opty", I32), ("precision", I32),
                ("impl", I32), ("ispg", I32), ("eps_e", ctypes.c_double), ("left", I32), ("right", I32)]


def lib():
    """Load (once) and return the C-ABI library; raise if it is not built."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise ImportError("lns3d_gb300: %s is not built; run __graft_entry__.build() or "
                              "python -m lns3d_gb300._build" % path)
        L = ctypes.CDLL(path)
        L.lns_last_error.restype = ctypes.c_char_p
        L.lns_version.restype = ctypes.c_char_p
        L.lns_mixed_workspace_bytes.restype = ctypes.c_size_t
        L.lns_mixed_workspace_bytes.argtypes = [I32, I32, I32, I32]
        L.lns_tri_workspace_bytes.restype = ctypes.c_size_t
        L.lns_tri_workspace_bytes.argtypes = [I32, I32, I32]
        L.lns_ctx3d_bytes.restype = ctypes.c_size_t
        L.lns_ctx3d_bytes.argtypes = [P]
        L.lns_lin2d_bytes.restype = ctypes.c_size_t
        L.lns_lin2d_bytes.argtypes = [P]
        L.lns_server3d_bytes_in_use.restype = ctypes.c_size_t
        L.lns_server3d_bytes_in_use.argtypes = [P]
        L.lns_batch3d_bytes.restype = ctypes.c_size_t
        L.lns_batch3d_bytes.argtypes = [P]
        L.lns_ctx2d_bytes.restype = ctypes.c_size_t
        L.lns_ctx2d_bytes.argtypes = [P]
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = L
    return _lib


def check(rc, where):
    if rc != LNS_OK:
        raise LnsError(rc, where, lib().lns_last_error().decode())

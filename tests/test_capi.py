"""CPU tests of the C-ABI library: it loads, exports every declared entry
point, and validates arguments before touching a GPU."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"\b(lns_\w+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    import lns3d_gb300

    return lns3d_gb300.lib()


def test_header_declares_entry_points():
    names = declared_symbols()
    for base in ("penta2bc", "penta1bc", "cpenta2bc", "cpenta1bc", "penta2p", "penta1p", "cpenta2p", "cpenta1p",
                 "solve2bc", "solve1bc", "solve2p", "solve1p"):
        assert "lns_" + base in names and "lns_" + base + "_dev" in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    from lns3d_gb300._lib import SIGNATURES

    solver_syms = [n for n in declared_symbols()
                   if n not in ("lns_last_error", "lns_version",
                                "lns_mixed_workspace_bytes", "lns_ctx3d_bytes", "lns_ctx2d_bytes", "lns_lin2d_bytes", "lns_batch3d_bytes",
                                "lns_server3d_bytes_in_use", "lns_tri_workspace_bytes")]
    assert sorted(SIGNATURES) == solver_syms


def test_version(lib):
    assert b"sm_103a" in lib.lns_version()


@pytest.mark.parametrize("name,args", [
    ("lns_penta2bc", (7, 1, 4)),      # nblk must be 5
    ("lns_penta2bc", (6, 1, 5)),      # too few rows
    ("lns_penta1bc", (-1, 8, 5)),     # negative nsys
    ("lns_penta1bc", (1, 3, 5)),
])
def test_argument_errors_real(lib, name, args):
    a = np.zeros(125 * 64)
    rc = getattr(lib, name)(*args, a.ctypes.data, a.ctypes.data)
    assert rc == 1
    assert lib.lns_last_error()


@pytest.mark.parametrize("code", [-1, 3])
def test_argument_errors_code(lib, code):
    a = np.zeros(2 * 125 * 64)
    for name in ("lns_cpenta2bc", "lns_cpenta1bc"):
        assert getattr(lib, name)(8, 8, 5, a.ctypes.data, a.ctypes.data, code) == 1
        assert b"code" in lib.lns_last_error()


def test_python_mirror_type_checks():
    import lns3d_gb300 as g

    with pytest.raises(TypeError):
        g.penta2bc(8, 1, 5, np.zeros(125 * 8, np.float32), np.zeros(40))
    with pytest.raises(ValueError):
        g.penta2bc(8, 1, 5, np.zeros(10), np.zeros(40))
    with pytest.raises(g.LnsError) as e:
        g.penta2bc(8, 1, 4, np.zeros(125 * 8), np.zeros(40))
    assert e.value.code == 1


def test_zero_lines_is_a_no_op():
    import lns3d_gb300 as g

    # nsys = 0 is valid and launches nothing (no GPU needed)
    g.penta2bc(8, 0, 5, np.zeros(1), np.zeros(1))


def test_mixed_workspace_size(lib):
    # FP32 factors + FP32 residual + FP64 iterate, 256-byte aligned pieces
    b = lib.lns_mixed_workspace_bytes(256, 512, 1, 0)
    assert b >= 256 * 512 * (125 * 8 + 5 * 8 + 5 * 16)
    assert lib.lns_mixed_workspace_bytes(257, 512, 1, 1) > b
    assert lib.lns_mixed_workspace_bytes(0, 1, 1, 0) == 0


@pytest.mark.parametrize("refine", [-1, 17])
def test_mixed_argument_errors(lib, refine):
    a = np.zeros(2 * 125 * 64)
    assert lib.lns_cpenta2bc_mixed_dev(8, 8, 5, a.ctypes.data, a.ctypes.data, 2, refine, None, None) == 1
    assert lib.lns_cpenta2bc_mixed(8, 8, 5, a.ctypes.data, a.ctypes.data, refine) == 1


def _params3d(**kw):
    from lns3d_gb300._lib import Params3D

    base = dict(nx=64, ny=32, dxi=1 / 63, deta=1 / 31, Ma=0.8, Re=500.0, Pr=0.72, gamma=1.4, omega=0.05, beta=0.2,
                alfa=1.0, cflmax=1.0, dtmax=1e30, loctime=1, xper=1, yper=0, navier=1, wall=1, wallt=1, top=0,
                optx=-1, opty=-1, precision=0)
    base.update(kw)
    return Params3D(**base)


# right 5 at nx 64 > ny 32: its wave reads x(j, nx) of the (nx, ny) grid
@pytest.mark.parametrize("bad", [dict(xper=2), dict(xper=0, left=2), dict(xper=0, left=6), dict(xper=0, right=1),
                                 dict(xper=0, right=5), dict(xper=0, right=9), dict(xper=0, left=0, right=4),
                                 dict(xper=0, left=17), dict(xper=0, left=11), dict(xper=0, right=21),
                                 dict(xper=0, right=7, nx=20, ny=24), dict(yper=2), dict(navier=0), dict(wall=0), dict(wallt=2),
                                 dict(top=2), dict(nx=7), dict(ny=6), dict(precision=2), dict(dxi=0.0),
                                 dict(loctime=2), dict(ispg=-1), dict(yper=1, ny=7), dict(yper=1, top=1),
                                 dict(navier=2, yper=1), dict(eps_e=-1.0), dict(eps_e=float("nan"))])
def test_ctx3d_rejects_unsupported_options(lib, bad):
    ctx = ctypes.c_void_p()
    rc = lib.lns_ctx3d_create(ctypes.byref(_params3d(**bad)), ctypes.byref(ctx))
    assert rc == 1 and not ctx.value
    assert lib.lns_last_error()


def test_ctx3d_null_arguments(lib):
    assert lib.lns_ctx3d_create(None, None) == 1
    assert lib.lns_upload_metrics3d(None, None) == 1
    assert lib.lns_upload_mean3d(None, None, None) == 1
    assert lib.lns_step3d(None, None, 1, 1, None) == 1
    assert lib.lns_step3d_dev(None, None, 1, 1, None, None) == 1
    assert lib.lns_rhs3d_dev(None, None, None, None, None, None) == 1
    assert lib.lns_lhs3d_dev(None, 1, None, None) == 1
    assert lib.lns_get_field3d(None, 0, None) == 1
    assert lib.lns_ctx3d_destroy(None) == 0
    assert lib.lns_ctx3d_bytes(None) == 0
    assert lib.lns_ctx3d_profile(None, 1) == 1
    assert lib.lns_ctx3d_profile_read(None, None, None) == 1
    assert lib.lns_upload_sponge3d(None, None, None) == 1
    assert lib.lns_upload_buffer3d(None, None) == 1
    assert lib.lns_upload_inflow3d(None, None, None, 0.0) == 1
    assert lib.lns_upload_sponge_target3d(None, None) == 1
    assert lib.lns_upload_bump3d(None, None) == 1
    assert lib.lns_upload_profile3d(None, None, None, 0.0, 0.0) == 1
    assert lib.lns_lin2d_set_nbl(None, 0) == 1


def _params2d(**kw):
    from lns3d_gb300._lib import Params2D

    base = dict(nx=32, ny=24, dxi=1 / 31, deta=1 / 23, Ma=0.5, Re=1000.0, Pr=0.72, gamma=1.4, alfa=1.0, cflmax=1.0,
                dtmax=1e30, theta=0.0, loctime=0, xper=1, yper=0, navier=1, wall=0, wallt=1, top=0, optx=-1, opty=-1)
    base.update(kw)
    return Params2D(**base)


@pytest.mark.parametrize("bad", [dict(xper=2), dict(xper=0, left=1), dict(xper=0, left=4), dict(xper=0, right=2), dict(xper=0, right=9),
                                 dict(xper=0, Ma=1.2), dict(xper=0, extrap=2), dict(xper=0, extrap=-2),
                                 dict(xper=0, nbl=25), dict(xper=0, nbl=-1), dict(xper=0, update_nbl=2),
                                 dict(xper=0, lhs_order=2), dict(xper=0, nx=9), dict(yper=1), dict(navier=0), dict(wall=2), dict(wallt=2),
                                 dict(top=1), dict(nx=7), dict(ny=6), dict(Ma=1.0), dict(deta=0.0),
                                 dict(lhs_order=3), dict(lhs_order=2, ny=7), dict(impl=4),
                                 dict(impl=-1), dict(ispg=1), dict(eps_e=-0.5),
                                 dict(top=3, lhs_order=2)])
def test_ctx2d_rejects_unsupported_options(lib, bad):
    ctx = ctypes.c_void_p()
    rc = lib.lns_ctx2d_create(ctypes.byref(_params2d(**bad)), ctypes.byref(ctx))
    assert rc == 1 and not ctx.value
    assert lib.lns_last_error()


def test_ctx2d_null_arguments(lib):
    assert lib.lns_ctx2d_create(None, None) == 1
    assert lib.lns_upload_metrics2d(None, None) == 1
    assert lib.lns_upload_top2d(None, None, None) == 1
    assert lib.lns_itrbc2d_dev(None, None, None) == 1
    assert lib.lns_step2d(None, None, 1, 1, None) == 1
    assert lib.lns_step2d_dev(None, None, 1, 1, None, None) == 1
    assert lib.lns_rhs2d_dev(None, None, None, None, None, None) == 1
    assert lib.lns_lhs2d_dev(None, 1, None, None, None) == 1
    assert lib.lns_get_field2d(None, 0, None) == 1
    assert lib.lns_ctx2d_destroy(None) == 0
    assert lib.lns_ctx2d_bytes(None) == 0
    assert lib.lns_upload_sponge2d(None, None, None) == 1
    assert lib.lns_upload_side2d(None, 1, None, None) == 1
    assert lib.lns_upload_buffer2d(None, None) == 1


def test_batch3d_argument_errors(lib):
    assert lib.lns_batch3d_create(0, None, None) == 1
    bad = (type(_params3d()) * 2)(_params3d(), _params3d(precision=1))
    b = ctypes.c_void_p()
    assert lib.lns_batch3d_create(2, bad, ctypes.byref(b)) == 1 and not b.value
    assert lib.lns_batch3d_upload(None, 0, None, None, None) == 1
    assert lib.lns_batch3d_tune(None, 1, None) == 1
    assert lib.lns_batch3d_run(None, 1, 1, 1e-10, 1, None, None) == 1
    assert lib.lns_batch3d_get_state(None, 0, None) == 1
    assert lib.lns_batch3d_destroy(None) == 0
    assert lib.lns_batch3d_bytes(None) == 0


def test_server3d_argument_errors(lib):
    s = ctypes.c_void_p()
    assert lib.lns_server3d_create(1 << 30, 0, 1, 1, ctypes.byref(s)) == 1
    assert lib.lns_server3d_create(1 << 30, 4, 7, 1, ctypes.byref(s)) == 1
    assert lib.lns_server3d_submit(None, None, None, None, None, 1e-10, 10, None) == 1
    assert lib.lns_server3d_tick(None, 1, None, None) == 1
    assert lib.lns_server3d_poll(None, 1, None, None, None, None) == 1
    assert lib.lns_server3d_fetch(None, 1, None) == 1
    assert lib.lns_server3d_destroy(None) == 0
    assert lib.lns_server3d_bytes_in_use(None) == 0


@pytest.mark.parametrize("bad", [dict(beta=0.2), dict(omega=0.05), dict(precision=1), dict(xper=0, left=2, right=0),
                                 dict(xper=0, left=3, right=0), dict(xper=0, left=4, right=0),
                                 dict(xper=0, left=5, right=0), dict(xper=0, left=11, right=0),
                                 dict(xper=0, left=17, right=0), dict(xper=0, left=0, right=3),
                                 dict(xper=0, left=0, right=7), dict(xper=0, left=0, right=21)])
def test_lin2d_rejects_single_mode_options(lib, bad):
    """The linear 2D context takes beta = omega = 0, FP64 and a periodic xi
    direction, or the zero-disturbance (left 0), nonreflecting (left 1) or
    symmetry (left 7) plane with the zero-disturbance or nonreflecting right
    plane (right 0, 1)."""
    ctx = ctypes.c_void_p()
    base = dict(beta=0.0, omega=0.0)
    base.update(bad)
    rc = lib.lns_lin2d_create(ctypes.byref(_params3d(**base)), ctypes.byref(ctx))
    assert rc == 1 and not ctx.value
    assert lib.lns_last_error()

"""GPU parity of the nonlinear 2D implicit step (lns_ctx2d_*, through the C
ABI) against the CPU oracle (oracle/impdrv2d_oracle.c) on the vortex case.

Tolerances (FP64; the GPU fuses multiply-adds, the oracle does not):
  operators, time step, LHS        1e-12 of the field's largest entry
  RHS and residual                 1e-11 of the largest entry
  steps                            1e-12 of max|v| per step over the
                                   reference's 100-step comparison
"""
import numpy as np
import pytest

from oracle.impdrv2d import Oracle2D

pytestmark = pytest.mark.gpu

OPS_TOL, RHS_TOL, STEP_TOL = 1e-12, 1e-11, 1e-12


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def make(case, **kw):
    from lns3d_gb300 import ImpDrv2D

    return ImpDrv2D(case["params"], case["metrics"], case["bnt"], case["pot"], cflmax=1.0, loctime=0, **kw)


@pytest.fixture(scope="module")
def small():
    from lns3d_gb300.cases import vortex2d

    c = vortex2d(nx=40, ny=33, seed=2)
    # a state off the initial condition: the oracle's own first steps
    o = Oracle2D(c, cflmax=1.0, loctime=0)
    v = c["v"].copy(order="F")
    o.itrbc(v)
    for _ in range(3):
        o.step(v)
    return c, v


def dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()


def host(t, shape):
    return t.cpu().numpy().reshape(shape, order="F")


def test_rhs_operators_and_time_step_match_oracle(cuda, small):
    import ctypes

    import torch

    c, v = small
    o = Oracle2D(c, cflmax=1.0, loctime=0)
    vold = np.asfortranarray(v * (1.0 + 1e-3 * np.random.default_rng(1).standard_normal(v.shape)))
    L = o.L
    cfl = L.a3_set_time_step(ctypes.byref(o.g.g), ctypes.c_void_p(v.ctypes.data), ctypes.c_void_p(o.dtl.ctypes.data))
    r_ref, res_ref = o.rhs(v, vold, o.dtl)
    drv = make(c)
    dv, dvo = dev(v), dev(vold)
    dr = torch.zeros_like(dv)
    tot = torch.zeros(1, dtype=torch.float64, device="cuda")
    drv.rhs(dv, dvo, dr, tot)
    torch.cuda.synchronize()
    assert rel(drv.field("dtl"), o.dtl) < OPS_TOL
    for name in ("Ah", "Bh", "Dh", "Vh11", "Vh12", "Vh22"):
        assert rel(drv.field(name), o.ops[name]) < OPS_TOL, name
    assert rel(host(dr, v.shape), r_ref) < RHS_TOL
    assert abs(tot.item() - res_ref) <= RHS_TOL * res_ref
    assert cfl > 0


@pytest.mark.parametrize("direction", [1, 2])
def test_lhs_matches_oracle(cuda, small, direction):
    import torch

    c, v = small
    o = Oracle2D(c, cflmax=1.0, loctime=0)
    import ctypes

    o.L.a3_set_time_step(ctypes.byref(o.g.g), ctypes.c_void_p(v.ctypes.data), ctypes.c_void_p(o.dtl.ctypes.data))
    o.rhs(v, v, o.dtl)
    ref = o.lhs(v, o.dtl, direction)
    drv = make(c)
    dv = dev(v)
    drv.rhs(dv, dv, torch.zeros_like(dv))
    mat = torch.zeros(125 * c["params"]["nx"] * c["params"]["ny"], dtype=torch.float64, device="cuda")
    drv.lhs(direction, dv, mat)
    torch.cuda.synchronize()
    got = host(mat, ref.shape)
    assert rel(got, ref) < OPS_TOL
    # rows set by the boundary conditions agree to rounding of their own scale
    assert rel(got[:, :, :, :, -1], ref[:, :, :, :, -1]) < OPS_TOL


def test_itrbc_matches_oracle(cuda, small):
    c, v = small
    o = Oracle2D(c, cflmax=1.0, loctime=0)
    w = np.asfortranarray(v * (1.0 + 1e-2 * np.random.default_rng(3).standard_normal(v.shape)))
    want = w.copy(order="F")
    o.itrbc(want)
    drv = make(c)
    dw = dev(w)
    drv.itrbc(dw)
    assert rel(host(dw, w.shape), want) < 1e-14


@pytest.mark.parametrize("niter", [1, 2])
def test_steps_match_oracle(cuda, niter):
    from lns3d_gb300.cases import vortex2d

    c = vortex2d(nx=40, ny=33, seed=4)
    o = Oracle2D(c, cflmax=1.0, loctime=0)
    drv = make(c)
    v_ref = c["v"].copy(order="F")
    o.itrbc(v_ref)
    v_gpu = v_ref.copy(order="F")
    for s in range(5):
        res_ref = o.step(v_ref, niter=niter)
        res_gpu = drv.step(v_gpu, nsteps=1, niter=niter)[0]
        assert rel(v_gpu, v_ref) < STEP_TOL, s
        assert abs(res_gpu - res_ref) <= 1e-10 * res_ref, s


def test_config1_100_step_history(cuda):
    # the reference's comparison: 128 x 128, 100 steps, every step's state and
    # residual against the oracle
    from lns3d_gb300.cases import vortex2d

    c = vortex2d(nx=128, ny=128, seed=0)
    o = Oracle2D(c, cflmax=1.0, loctime=0)
    drv = make(c)
    v_ref = c["v"].copy(order="F")
    o.itrbc(v_ref)
    v_gpu = v_ref.copy(order="F")
    worst, worst_res = 0.0, 0.0
    for s in range(100):
        res_ref = o.step(v_ref)
        res_gpu = drv.step(v_gpu)[0]
        worst = max(worst, rel(v_gpu, v_ref))
        worst_res = max(worst_res, abs(res_gpu - res_ref) / res_ref)
    assert worst < STEP_TOL, worst
    assert worst_res < 1e-10, worst_res


def test_device_steps_match_host_steps(cuda, small):
    import torch

    c, v = small
    a, b = make(c), make(c)
    o = Oracle2D(c, cflmax=1.0, loctime=0)
    vh = v.copy(order="F")
    res_h = a.step(vh, nsteps=4)
    dv = dev(v)
    tot = torch.zeros(4, dtype=torch.float64, device="cuda")
    b.step(dv, nsteps=4, totres=tot)
    torch.cuda.synchronize()
    assert np.array_equal(host(dv, v.shape), vh)
    vo = v.copy(order="F")
    res_o = np.array([o.step(vo) for _ in range(4)])
    assert np.abs(tot.cpu().numpy() - res_o).max() <= 1e-10 * res_o.max()
    assert np.abs(np.asarray(res_h) - res_o).max() <= 1e-10 * res_o.max()


# ---------------------------------------------------------------- iLHS = 0
# The second-order LHS (src/lhs.f90, src/lhsbt2.f90, src/lhsbc{1,2}.f90)
# with the block-tridiagonal solves (src/nsolve2p.f90, src/nsolve1bc.f90).
# The device writes it in the pentadiagonal slots; both sides are compared
# as the dense matrices of their lines.


def _dense_lines(direction, nx, ny, tri=None, penta=None):
    import tricase
    from test_oracle import dense as penta_dense

    out = []
    nsys = ny if direction == 1 else nx
    for iv in range(nsys):
        if tri is not None:
            mat3, bc = tri
            case = ({"solver": "solve2p", "rows": nx, "mat": mat3} if direction == 1 else
                    {"solver": "solve1bc", "rows": ny, "mat": mat3, "bc": bc})
            out.append(tricase.dense_line(case, iv))
        else:
            case = ({"solver": "penta2p", "rows": nx, "mat": penta} if direction == 1 else
                    {"solver": "penta1bc", "rows": ny, "mat": penta})
            out.append(penta_dense(case, iv)[0])
    return np.array(out)


@pytest.mark.parametrize("direction,wall,wallt", [(1, 0, 1), (2, 0, 1), (2, 1, 0), (2, 3, 1)])
def test_second_order_lhs_matches_oracle(cuda, small, direction, wall, wallt):
    import ctypes

    import torch

    c, v = small
    c = dict(c, params=dict(c["params"], wall=wall, wallt=wallt))
    o = Oracle2D(c, cflmax=1.0, loctime=0, ilhs=0)
    o.L.a3_set_time_step(ctypes.byref(o.g.g), ctypes.c_void_p(v.ctypes.data), ctypes.c_void_p(o.dtl.ctypes.data))
    o.rhs(v, v, o.dtl)
    nx, ny = c["params"]["nx"], c["params"]["ny"]
    ref = _dense_lines(direction, nx, ny, tri=o.lhs2(v, o.dtl, direction))
    drv = make(c, ilhs=0)
    dv = dev(v)
    drv.rhs(dv, dv, torch.zeros_like(dv))
    mat = torch.zeros(125 * nx * ny, dtype=torch.float64, device="cuda")
    drv.lhs(direction, dv, mat)
    torch.cuda.synchronize()
    got = _dense_lines(direction, nx, ny, penta=host(mat, (5, 5, 5, nx, ny)))
    assert rel(got, ref) < OPS_TOL
    # the fourth-order LHS of the same context type differs (a wrong switch
    # would pass the comparison above only by accident)
    drv4 = make(c)
    drv4.rhs(dv, dv, torch.zeros_like(dv))
    drv4.lhs(direction, dv, mat)
    torch.cuda.synchronize()
    assert rel(_dense_lines(direction, nx, ny, penta=host(mat, (5, 5, 5, nx, ny))), ref) > 1e-3


@pytest.mark.parametrize("niter,wall", [(1, 0), (2, 0), (1, 3)])
def test_second_order_steps_match_oracle(cuda, niter, wall):
    from lns3d_gb300.cases import vortex2d

    c = vortex2d(nx=40, ny=33, seed=5)
    c["params"]["wall"] = wall
    o = Oracle2D(c, cflmax=1.0, loctime=0, ilhs=0)
    drv = make(c, ilhs=0)
    v_ref = c["v"].copy(order="F")
    o.itrbc(v_ref)
    v_gpu = v_ref.copy(order="F")
    v4 = v_ref.copy(order="F")
    for s in range(5):
        res_ref = o.step(v_ref, niter=niter)
        res_gpu = drv.step(v_gpu, nsteps=1, niter=niter)[0]
        assert rel(v_gpu, v_ref) < STEP_TOL, s
        assert abs(res_gpu - res_ref) <= 1e-10 * res_ref, s
    make(c).step(v4, nsteps=5, niter=niter)
    assert rel(v4, v_ref) > 1e-9


@pytest.mark.parametrize("impl,ilhs", [(2, 1), (3, 1), (2, 0), (3, 0)])
def test_time_schemes_match_oracle(cuda, impl, ilhs):
    """impl 2 (two-step backward: backward Euler first, then rtb at alfa =
    2/3) and impl 3 (midpoint: genmtrx on (v + vold)/2, alfa = 1/2),
    src/impdrv.f90:186-279, per step against the oracle, with both LHS
    orders; the first step of impl 2 is the backward Euler step."""
    from lns3d_gb300.cases import vortex2d

    c = vortex2d(nx=40, ny=33, seed=6)
    o = Oracle2D(c, cflmax=1.0, loctime=0, ilhs=ilhs, impl=impl)
    drv = make(c, ilhs=ilhs, impl=impl)
    v_ref = c["v"].copy(order="F")
    o.itrbc(v_ref)
    v_gpu = v_ref.copy(order="F")
    v_be = v_ref.copy(order="F")
    for s in range(4):
        res_ref = o.step(v_ref)
        res_gpu = drv.step(v_gpu, nsteps=1)[0]
        assert rel(v_gpu, v_ref) < STEP_TOL, s
        assert abs(res_gpu - res_ref) <= 1e-10 * res_ref, s
        if s == 0:
            make(c, ilhs=ilhs).step(v_be, nsteps=1)
            assert (rel(v_gpu, v_be) < STEP_TOL) == (impl == 2)


def test_time_scheme_argument_checks():
    from lns3d_gb300.cases import vortex2d

    c = vortex2d(nx=16, ny=12)
    with pytest.raises(ValueError):
        make(c, impl=4)


@pytest.mark.parametrize("kw", [dict(ispg=2), dict(eps_e=0.02), dict(ispg=2, eps_e=0.02),
                                dict(ispg=2, eps_e=0.02, ilhs=0)])
def test_sponge_and_smoother_match_oracle(cuda, small, kw):
    """The nonlinear sponge (ispg 2, src/genmtrx.f90:436-446) and the
    explicit smoother / implicit damping (src/smoother.f90, src/lhsf.f90,
    src/lhsbt2f.f90 with its transposed spgl view) against the oracle: the
    RHS, both LHS and steps."""
    import ctypes

    import torch

    c, v = small
    nx, ny = c["params"]["nx"], c["params"]["ny"]
    rng = np.random.default_rng(21)
    extra = dict(kw)
    if "ispg" in kw:
        extra.update(spg=np.asfortranarray(rng.uniform(size=(nx, ny))),
                     spg2=np.asfortranarray(0.3 * rng.uniform(size=(nx, ny))))
    if "eps_e" in kw:
        extra.update(buff=np.asfortranarray(0.5 + rng.uniform(size=(nx, ny))))
    o = Oracle2D(c, cflmax=1.0, loctime=0, **extra)
    o.L.a3_set_time_step(ctypes.byref(o.g.g), ctypes.c_void_p(v.ctypes.data), ctypes.c_void_p(o.dtl.ctypes.data))
    vold = np.asfortranarray(v * (1.0 + 1e-3 * rng.standard_normal(v.shape)))
    r_ref, res_ref = o.rhs(v, vold, o.dtl)
    drv = make(c, **extra)
    dv, dvo = dev(v), dev(vold)
    dr = torch.zeros_like(dv)
    tot = torch.zeros(1, dtype=torch.float64, device="cuda")
    drv.rhs(dv, dvo, dr, tot)
    torch.cuda.synchronize()
    assert rel(host(dr, v.shape), r_ref) < RHS_TOL
    for direction in (1, 2):
        mat = torch.zeros(125 * nx * ny, dtype=torch.float64, device="cuda")
        drv.lhs(direction, dv, mat)
        torch.cuda.synchronize()
        if kw.get("ilhs", 1) == 0:
            ref = _dense_lines(direction, nx, ny, tri=o.lhs2(v, o.dtl, direction))
            got = _dense_lines(direction, nx, ny, penta=host(mat, (5, 5, 5, nx, ny)))
            assert rel(got, ref) < OPS_TOL, direction
        else:
            ref = o.lhs(v, o.dtl, direction)
            assert rel(host(mat, ref.shape), ref) < OPS_TOL, direction
    from lns3d_gb300.cases import vortex2d

    c2 = vortex2d(nx=nx, ny=ny, seed=7)
    o2 = Oracle2D(c2, cflmax=1.0, loctime=0, **extra)
    d2 = make(c2, **extra)
    v_ref = c2["v"].copy(order="F")
    o2.itrbc(v_ref)
    v_gpu = v_ref.copy(order="F")
    for s in range(4):
        res_o = o2.step(v_ref)
        res_g = d2.step(v_gpu, nsteps=1)[0]
        assert rel(v_gpu, v_ref) < STEP_TOL, s
        assert abs(res_g - res_o) <= 1e-10 * res_o, s


def test_held_top_matches_oracle(cuda):
    """top = 3 (the held quiescent top, src/itrbc.f90 nonlinear branch,
    src/lhsbc2f.f90:332-339): both LHS and steps against the oracle; the
    far-field arrays are not needed for it."""
    import torch

    from lns3d_gb300.cases import vortex2d

    c = vortex2d(nx=40, ny=33, seed=8)
    c = dict(c, params=dict(c["params"], top=3))
    o = Oracle2D(c, cflmax=1.0, loctime=0)
    drv = make(c)
    v_ref = c["v"].copy(order="F")
    o.itrbc(v_ref)
    v_gpu = v_ref.copy(order="F")
    for s in range(4):
        res_o = o.step(v_ref)
        res_g = drv.step(v_gpu, nsteps=1)[0]
        assert rel(v_gpu, v_ref) < STEP_TOL, s
        assert abs(res_g - res_o) <= 1e-10 * res_o, s
    import ctypes

    nx, ny = 40, 33
    # operators and time step of the current state on both sides
    o.L.a3_set_time_step(ctypes.byref(o.g.g), ctypes.c_void_p(v_ref.ctypes.data),
                         ctypes.c_void_p(o.dtl.ctypes.data))
    o.rhs(v_ref, v_ref, o.dtl)
    dv = dev(v_ref)
    drv.rhs(dv, dv, torch.zeros_like(dv))
    for direction in (1, 2):
        ref = o.lhs(v_ref, o.dtl, direction)
        mat = torch.zeros(125 * nx * ny, dtype=torch.float64, device="cuda")
        drv.lhs(direction, dv, mat)
        torch.cuda.synchronize()
        assert rel(host(mat, ref.shape), ref) < OPS_TOL, direction

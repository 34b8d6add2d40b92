"""GPU parity of the linearised 3D implicit step (lns_ctx3d_*, through the C
ABI) against the CPU oracle (oracle/adi3d_oracle.c) on the shear-layer case.

Tolerances (FP64 path; the GPU contracts a*b+c into fused multiply-adds, the
oracle does not, so results agree to rounding, not bitwise):
  operators, time step, LHS        1e-12 of the field's largest entry
  RHS and residual                 1e-11 of the largest entry (the fourth-order
                                   stencils cancel ~1e2 of the operand scale)
  full steps                       1e-12 of max|v| per step, as the reference's
                                   per-step comparison asks
"""
import numpy as np
import pytest

from adi3dcase import Oracle3D

pytestmark = pytest.mark.gpu

OPS_TOL, RHS_TOL, STEP_TOL = 1e-12, 1e-11, 1e-12


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def small():
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=40, ny=33, seed=3)
    orc = Oracle3D(case, cflmax=20.0, loctime=1)
    return case, orc


def make_drv(case, precision=0, cflmax=20.0, loctime=1):
    from lns3d_gb300 import ImpDrv3D

    return ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=cflmax, loctime=loctime,
                    precision=precision)


def test_operators_match_oracle(cuda, small):
    case, orc = small
    drv = make_drv(case)
    for name in ("Ah", "Bh", "Dh", "Dhi", "Vh11", "Vh12", "Vh22", "ABhi"):
        assert rel(drv.field(name), orc.ops[name]) < OPS_TOL, name
    assert rel(drv.field("dtl"), orc.dtl) < OPS_TOL
    assert abs(drv.cfl - orc.cfl) <= OPS_TOL * abs(orc.cfl)


@pytest.mark.parametrize("loctime", [0, 1])
def test_time_step_modes(cuda, small, loctime):
    case, _ = small
    orc = Oracle3D(case, cflmax=5.0, loctime=loctime)
    drv = make_drv(case, cflmax=5.0, loctime=loctime)
    assert rel(drv.field("dtl"), orc.dtl) < OPS_TOL


@pytest.mark.parametrize("direction", [1, 2])
def test_lhs_matches_oracle(cuda, small, direction):
    import torch

    case, orc = small
    drv = make_drv(case)
    nx, ny = orc.nx, orc.ny
    mat = torch.zeros(125 * nx * ny, dtype=torch.complex128, device="cuda")
    drv.lhs(direction, mat)
    torch.cuda.synchronize()
    got = mat.cpu().numpy().reshape((5, 5, 5, nx, ny), order="F")
    ref = orc.lhs(direction)
    assert rel(got, ref) < OPS_TOL
    # the boundary-condition rows are exact
    assert np.array_equal(got[:, :, :, :, ny - 1], ref[:, :, :, :, ny - 1])


def test_rhs_matches_oracle(cuda, small):
    import ctypes

    import torch
    from adi3dcase import _lib, ptr

    case, orc = small
    drv = make_drv(case)
    rng = np.random.default_rng(11)
    shape = (5, orc.nx, orc.ny)
    v = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    vold = np.asfortranarray(v + 1e-3 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
    L = _lib()
    r = orc.lrhs(v)
    L.a3_rbe(ctypes.byref(orc.g), ptr(r), ptr(v), ptr(vold), ptr(orc.dtl))
    L.a3_rhsbc(ctypes.byref(orc.g), ptr(r), ptr(v))
    res = L.a3_resstat(ctypes.byref(orc.g), ptr(r), ptr(orc.dtl))
    dev = lambda a: torch.from_numpy(a.ravel(order="F")).cuda()
    dv, dvo = dev(v), dev(vold)
    dr = torch.zeros_like(dv)
    tot = torch.zeros(1, dtype=torch.float64, device="cuda")
    drv.rhs(dv, dvo, dr, tot)
    torch.cuda.synchronize()
    got = dr.cpu().numpy().reshape(shape, order="F")
    assert rel(got, r) < RHS_TOL
    assert abs(tot.item() - res) <= RHS_TOL * res


@pytest.mark.parametrize("niter", [1, 2])
def test_steps_match_oracle(cuda, niter):
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=40, ny=33, seed=5)
    orc = Oracle3D(case, cflmax=20.0, loctime=1)
    drv = make_drv(case)
    v_ref = case["v"].copy(order="F")
    v_gpu = case["v"].copy(order="F")
    for s in range(4):
        res_ref = orc.step(v_ref, niter=niter)
        res_gpu = drv.step(v_gpu, nsteps=1, niter=niter)[0]
        assert rel(v_gpu, v_ref) < STEP_TOL, s
        assert abs(res_gpu - res_ref) <= 1e-10 * res_ref, s


def test_device_steps_match_host_steps(cuda, small):
    import torch

    case, _ = small
    a, b = make_drv(case), make_drv(case)
    v_host = case["v"].copy(order="F")
    res_host = a.step(v_host, nsteps=6, niter=1)
    dv = torch.from_numpy(case["v"].ravel(order="F")).cuda()
    tot = torch.zeros(6, dtype=torch.float64, device="cuda")
    b.step(dv, nsteps=6, niter=1, totres=tot)
    torch.cuda.synchronize()
    got = dv.cpu().numpy().reshape(case["v"].shape, order="F")
    assert np.array_equal(got, v_host)
    assert np.array_equal(tot.cpu().numpy(), res_host)


def test_many_steps_track_oracle_and_converge(cuda):
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=48, ny=40, seed=0)
    orc = Oracle3D(case, cflmax=20.0, loctime=1)
    drv = make_drv(case)
    v_ref = case["v"].copy(order="F")
    v_gpu = case["v"].copy(order="F")
    res_ref = np.array([orc.step(v_ref) for _ in range(300)])
    res_gpu = drv.step(v_gpu, nsteps=300)
    assert rel(v_gpu, v_ref) < 1e-10
    assert np.abs(res_gpu - res_ref).max() <= 1e-9 * res_ref.max()
    assert res_gpu[-1] < 1e-2 * res_gpu[0]


def test_mixed_precision_converges_to_fp64_state(cuda):
    # A mixed step is the FP64 step with the correction solved by FP32 sweeps:
    # one step from the same state differs from the FP64 step by FP32 rounding
    # of the correction (bound 1e-4 of the correction: FP32 precision times
    # the growth along a 48-row line), and the FP64 residual drives both runs
    # down at the same rate.
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=48, ny=40, seed=0)
    d64, d32 = make_drv(case, precision=0), make_drv(case, precision=1)
    assert d32.device_bytes < d64.device_bytes
    v0 = case["v"].copy(order="F")
    a, b = v0.copy(order="F"), v0.copy(order="F")
    d64.step(a)
    d32.step(b)
    assert np.abs(b - a).max() <= 1e-4 * np.abs(a - v0).max()
    r64 = d64.step(a, nsteps=600)
    r32 = d32.step(b, nsteps=600)
    assert np.abs(r32 / r64 - 1.0).max() < 1e-2
    assert r32[-1] < 1e-3 * r32[0]


def test_state_mutation_refactors_after_new_mean(cuda, small):
    case, orc = small
    drv = make_drv(case)
    v = case["v"].copy(order="F")
    drv.step(v, nsteps=2)
    # a new mean flow rebuilds the operators and the factors
    vm2 = case["vm"].copy()
    vm2[4] *= 1.01
    drv.set_mean(vm2)
    case2 = dict(case, vm=vm2)
    orc2 = Oracle3D(case2, cflmax=20.0, loctime=1)
    v_ref = v.copy(order="F")
    orc2.step(v_ref)
    drv.step(v)
    assert rel(v, v_ref) < STEP_TOL


def test_rejects_bad_arguments(cuda, small):
    import torch
    from lns3d_gb300 import LnsError

    case, _ = small
    drv = make_drv(case)
    with pytest.raises(LnsError):
        drv.step(case["v"].copy(order="F"), nsteps=1, niter=0)
    with pytest.raises(ValueError):
        drv.step(np.zeros((5, 3, 3), np.complex128, order="F"))
    with pytest.raises(LnsError):
        drv.lhs(3, torch.zeros(125 * 40 * 33, dtype=torch.complex128, device="cuda"))


@pytest.mark.parametrize("nx,ny", [(40, 24), (41, 24), (40, 25), (41, 25)])
def test_row_pairs_agree_with_row_by_row(cuda, nx, ny):
    """Lines advanced two rows per step -- periodic xi lines when nx is even
    (an odd band), eta lines with boundary-closure rows when ny is even --
    and row by row agree to rounding, and both with the oracle; with nx and
    ny odd every line stays row by row whatever the switch says."""
    from lns3d_gb300 import ImpDrv3D
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=nx, ny=ny, seed=9)
    orc = Oracle3D(case, cflmax=20.0, loctime=1)
    mk = lambda pairs: ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1,
                                row_pairs=pairs)
    vp, vr, vo = (case["v"].copy(order="F") for _ in range(3))
    rp = mk(True).step(vp, nsteps=5)
    rr = mk(False).step(vr, nsteps=5)
    ro = [orc.step(vo) for _ in range(5)]
    if nx % 2 and ny % 2:
        assert np.array_equal(vp, vr) and np.array_equal(rp, rr)
    else:
        assert 0.0 < rel(vp, vr) < 1e-13
    for v in (vp, vr):
        assert rel(v, vo) < STEP_TOL
    assert np.abs(np.asarray(rp) - ro).max() <= 1e-10 * max(ro)


def test_row_pairs_switch_rejects_bad_values(cuda, small):
    from lns3d_gb300 import LnsError, lib

    case, _ = small
    drv = make_drv(case)
    with pytest.raises(LnsError):
        from lns3d_gb300._lib import check

        check(lib().lns_ctx3d_set_row_pairs(drv._ctx, 2), "lns_ctx3d_set_row_pairs")


def test_full_size_steps_match_oracle(cuda):
    # the 512 x 256 benchmark workload itself, three steps
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=512, ny=256, seed=0)
    orc = Oracle3D(case, cflmax=20.0, loctime=1)
    drv = make_drv(case)
    v_ref = case["v"].copy(order="F")
    v_gpu = case["v"].copy(order="F")
    res_ref = [orc.step(v_ref) for _ in range(3)]
    res_gpu = drv.step(v_gpu, nsteps=3)
    assert rel(v_gpu, v_ref) < STEP_TOL
    assert np.abs(np.array(res_gpu) - res_ref).max() <= 1e-10 * max(res_ref)


@pytest.mark.parametrize("precision", [0, 1])
def test_full_size_step_is_linear(cuda, precision):
    # size-independent property at the benchmark size: step(2a - 3b) equals
    # 2 step(a) - 3 step(b) to rounding (the step is linear in v)
    import torch
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=512, ny=256, seed=0)
    drv = make_drv(case, precision=precision)
    g = torch.Generator(device="cuda").manual_seed(3)
    n = 5 * 512 * 256
    a = torch.randn(n, dtype=torch.complex128, device="cuda", generator=g)
    b = torch.randn(n, dtype=torch.complex128, device="cuda", generator=g)
    c = 2.0 * a - 3.0 * b
    for v in (a, b, c):
        drv.step(v, nsteps=2)
    torch.cuda.synchronize()
    err = float((c - (2.0 * a - 3.0 * b)).abs().max() / c.abs().max())
    # FP64: rounding of the FP64 step; mixed: FP32 rounding of the correction
    assert err < (1e-12 if precision == 0 else 1e-4), err


@pytest.mark.parametrize("impl,niter", [(2, 1), (3, 1), (2, 2)])
def test_time_schemes_match_oracle(cuda, impl, niter):
    """impl 2 (two-step backward: backward Euler, then rtb3D with the LHS
    refactored at alfa = 2/3) and impl 3 (midpoint), src/impdrv3d.f90:130-199,
    against the oracle step by step; the device form splits the same steps
    over two calls."""
    import torch

    from lns3d_gb300 import ImpDrv3D
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=40, ny=33, seed=9)
    orc = Oracle3D(case, cflmax=20.0, loctime=1)
    drv = ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1, impl=impl)
    v_ref = case["v"].copy(order="F")
    v_gpu = case["v"].copy(order="F")
    for s in range(4):
        res_ref = orc.step_impl(v_ref, impl, niter=niter)
        res_gpu = drv.step(v_gpu, nsteps=1, niter=niter)[0]
        assert rel(v_gpu, v_ref) < STEP_TOL, s
        assert abs(res_gpu - res_ref) <= 1e-10 * res_ref, s
    dev = ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1, impl=impl)
    dv = torch.from_numpy(case["v"].ravel(order="F")).cuda()
    dev.step(dv, nsteps=1, niter=niter)
    dev.step(dv, nsteps=3, niter=niter)
    torch.cuda.synchronize()
    assert rel(dv.cpu().numpy().reshape(v_ref.shape, order="F"), v_ref) < STEP_TOL


def test_time_schemes_differ_and_reject_bad_impl(cuda, small):
    from lns3d_gb300 import ImpDrv3D, LnsError

    case, _ = small
    out = {}
    for impl in (1, 2, 3):
        d = ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1, impl=impl)
        v = case["v"].copy(order="F")
        d.step(v, nsteps=3)
        out[impl] = v
    assert rel(out[1], out[2]) > 1e-8 and rel(out[1], out[3]) > 1e-8
    with pytest.raises(LnsError):
        ImpDrv3D(case["params"], case["metrics"], case["vm"], impl=4)


@pytest.mark.parametrize("ispg", [1, 5])
def test_sponge_matches_oracle(cuda, ispg):
    """The sponge (ispg 1: spg; ispg 5: spg + spg2) in the RHS
    (src/lrhs3d.f90:220-240) and the eta LHS (src/lhs2f3d.f90:207-224,
    src/lhsbt2f3d.f90:147-167): RHS, both LHS and steps against the oracle."""
    import ctypes

    import torch
    from adi3dcase import _lib, ptr, sponge

    from lns3d_gb300 import ImpDrv3D
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=40, ny=33, seed=8)
    spg, spg2 = sponge(40, 33, amp=1.0)
    orc = Oracle3D(case, cflmax=20.0, loctime=1, ispg=ispg, spg=spg, spg2=spg2)
    mk = lambda: ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1, ispg=ispg,
                          spg=spg, spg2=spg2)
    drv = mk()
    nx, ny = 40, 33
    for direction in (1, 2):
        mat = torch.zeros(125 * nx * ny, dtype=torch.complex128, device="cuda")
        drv.lhs(direction, mat)
        torch.cuda.synchronize()
        got = mat.cpu().numpy().reshape((5, 5, 5, nx, ny), order="F")
        assert rel(got, orc.lhs(direction)) < OPS_TOL, direction
    rng = np.random.default_rng(12)
    shape = (5, nx, ny)
    v = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    vold = np.asfortranarray(v + 1e-3 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
    L = _lib()
    r = orc.lrhs(v)
    L.a3_rbe(ctypes.byref(orc.g), ptr(r), ptr(v), ptr(vold), ptr(orc.dtl))
    L.a3_rhsbc(ctypes.byref(orc.g), ptr(r), ptr(v))
    dev = lambda a: torch.from_numpy(a.ravel(order="F")).cuda()
    dv, dvo = dev(v), dev(vold)
    dr = torch.zeros_like(dv)
    drv.rhs(dv, dvo, dr, torch.zeros(1, dtype=torch.float64, device="cuda"))
    torch.cuda.synchronize()
    assert rel(dr.cpu().numpy().reshape(shape, order="F"), r) < RHS_TOL
    drv = mk()
    v_ref = case["v"].copy(order="F")
    v_gpu = case["v"].copy(order="F")
    for s in range(4):
        res_ref = orc.step(v_ref)
        res_gpu = drv.step(v_gpu, nsteps=1)[0]
        assert rel(v_gpu, v_ref) < STEP_TOL, s
        assert abs(res_gpu - res_ref) <= 1e-10 * res_ref, s


def test_sponge_needs_upload(cuda):
    """ispg != 0: stepping before lns_upload_sponge3d is an argument error;
    ispg > 4 needs spg2."""
    import ctypes

    from lns3d_gb300._lib import Params3D, lib
    from lns3d_gb300.adi3d import METRICS
    from lns3d_gb300.cases import shear_layer

    nx, ny = 16, 12
    case = shear_layer(nx=nx, ny=ny, seed=1)
    p = case["params"]
    L = lib()
    P = lambda a: ctypes.c_void_p(a.ctypes.data)
    m = np.empty((nx, ny, 10), order="F")
    for k, name in enumerate(METRICS):
        m[:, :, k] = case["metrics"][name]
    vm = np.asfortranarray(case["vm"])
    v = np.zeros(10 * nx * ny)
    sp = np.full(nx * ny, 0.1)
    for ispg in (1, 5):
        prm = Params3D(nx=nx, ny=ny, dxi=p["dxi"], deta=p["deta"], Ma=p["Ma"], Re=p["Re"], Pr=p["Pr"],
                       gamma=p["gamma"], omega=p["omega"], beta=p["kz"], alfa=1.0, cflmax=1.0, dtmax=1e30,
                       loctime=1, xper=1, yper=0, navier=1, wall=p["wall"], wallt=p["wallt"], top=0, optx=-1,
                       opty=-1, ispg=ispg)
        ctx = ctypes.c_void_p()
        assert L.lns_ctx3d_create(ctypes.byref(prm), ctypes.byref(ctx)) == 0
        try:
            assert L.lns_upload_metrics3d(ctx, P(m)) == 0
            assert L.lns_upload_mean3d(ctx, P(vm), None) == 0
            assert L.lns_step3d(ctx, P(v), 1, 1, None) == 1
            assert b"sponge" in L.lns_last_error()
            if ispg == 5:
                assert L.lns_upload_sponge3d(ctx, P(sp), None) == 1
            assert L.lns_upload_sponge3d(ctx, P(sp), P(sp)) == 0
            assert L.lns_step3d(ctx, P(v), 1, 1, None) == 0
        finally:
            L.lns_ctx3d_destroy(ctx)


@pytest.mark.parametrize("with_sponge", [False, True])
def test_smoother_matches_oracle(cuda, with_sponge):
    """The explicit smoother (src/smoother3d.f90) and the implicit damping of
    both LHS (src/lhs1f3d.f90:168-200, src/lhs2f3d.f90:171-203,
    src/lhsbt2f3d.f90:277-298) with a non-uniform buff, alone and with the
    sponge: RHS, both LHS and steps against the oracle."""
    import ctypes

    import torch
    from adi3dcase import _lib, ptr, sponge

    from lns3d_gb300 import ImpDrv3D
    from lns3d_gb300.cases import shear_layer

    nx, ny = 40, 33
    case = shear_layer(nx=nx, ny=ny, seed=10)
    buff = np.asfortranarray(0.5 + np.random.default_rng(3).uniform(size=(nx, ny)))
    kw = dict(eps_e=0.02, buff=buff)
    if with_sponge:
        spg, spg2 = sponge(nx, ny)
        kw.update(ispg=1, spg=spg, spg2=spg2)
    orc = Oracle3D(case, cflmax=20.0, loctime=1, **kw)
    mk = lambda: ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1, **kw)
    drv = mk()
    for direction in (1, 2):
        mat = torch.zeros(125 * nx * ny, dtype=torch.complex128, device="cuda")
        drv.lhs(direction, mat)
        torch.cuda.synchronize()
        got = mat.cpu().numpy().reshape((5, 5, 5, nx, ny), order="F")
        assert rel(got, orc.lhs(direction)) < OPS_TOL, direction
    rng = np.random.default_rng(13)
    shape = (5, nx, ny)
    v = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    vold = np.asfortranarray(v + 1e-3 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
    L = _lib()
    r = orc.lrhs(v)
    L.a3_rbe(ctypes.byref(orc.g), ptr(r), ptr(v), ptr(vold), ptr(orc.dtl))
    L.a3_rhsbc(ctypes.byref(orc.g), ptr(r), ptr(v))
    dev = lambda a: torch.from_numpy(a.ravel(order="F")).cuda()
    dv, dvo = dev(v), dev(vold)
    dr = torch.zeros_like(dv)
    drv.rhs(dv, dvo, dr, torch.zeros(1, dtype=torch.float64, device="cuda"))
    torch.cuda.synchronize()
    assert rel(dr.cpu().numpy().reshape(shape, order="F"), r) < RHS_TOL
    drv = mk()
    v_ref = case["v"].copy(order="F")
    v_gpu = case["v"].copy(order="F")
    for s in range(4):
        res_ref = orc.step(v_ref)
        res_gpu = drv.step(v_gpu, nsteps=1)[0]
        assert rel(v_gpu, v_ref) < STEP_TOL, s
        assert abs(res_gpu - res_ref) <= 1e-10 * res_ref, s


def test_smoother_default_buffer_is_ones(cuda):
    from lns3d_gb300 import ImpDrv3D
    from lns3d_gb300.cases import shear_layer

    nx, ny = 24, 20
    case = shear_layer(nx=nx, ny=ny, seed=2)
    a = ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1, eps_e=0.01)
    b = ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1, eps_e=0.01,
                 buff=np.ones((nx, ny)))
    va, vb = case["v"].copy(order="F"), case["v"].copy(order="F")
    a.step(va, nsteps=3)
    b.step(vb, nsteps=3)
    assert np.array_equal(va, vb)


@pytest.mark.parametrize("ispg", [2, 3, 4])
def test_target_sponges_match_oracle(cuda, ispg):
    """The inflow sponges (ispg 2, 3: the target wave formed on the device
    from the mean flow, x, x0 and wamp; src/lrhs3d.f90:242-280) and the
    eigenfunction sponge (ispg 4, src/sponge.f90:596-604): RHS, eta LHS and
    steps against the oracle."""
    import ctypes

    import torch
    from adi3dcase import _lib, ptr, sponge

    from lns3d_gb300 import ImpDrv3D
    from lns3d_gb300.cases import shear_layer

    nx, ny = 40, 33
    case = shear_layer(nx=nx, ny=ny, seed=11)
    spg, spg2 = sponge(nx, ny, amp=1.0)
    rng = np.random.default_rng(14)
    wamp = rng.uniform(0.5, 1.5, nx)
    cvic = np.asfortranarray(1e-3 * (rng.standard_normal((5, nx, ny)) + 1j * rng.standard_normal((5, nx, ny))))
    kw = dict(ispg=ispg, spg=spg, spg2=spg2, x0=-1.0, wamp=wamp, cvic=cvic)
    orc = Oracle3D(case, cflmax=20.0, loctime=1, **kw)
    mk = lambda: ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1, x=case["x"], **kw)
    drv = mk()
    mat = torch.zeros(125 * nx * ny, dtype=torch.complex128, device="cuda")
    drv.lhs(2, mat)
    torch.cuda.synchronize()
    assert rel(mat.cpu().numpy().reshape((5, 5, 5, nx, ny), order="F"), orc.lhs(2)) < OPS_TOL
    shape = (5, nx, ny)
    v = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    vold = np.asfortranarray(v + 1e-3 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
    L = _lib()
    r = orc.lrhs(v)
    L.a3_rbe(ctypes.byref(orc.g), ptr(r), ptr(v), ptr(vold), ptr(orc.dtl))
    L.a3_rhsbc(ctypes.byref(orc.g), ptr(r), ptr(v))
    dev = lambda a: torch.from_numpy(a.ravel(order="F")).cuda()
    dv, dvo = dev(v), dev(vold)
    dr = torch.zeros_like(dv)
    drv.rhs(dv, dvo, dr, torch.zeros(1, dtype=torch.float64, device="cuda"))
    torch.cuda.synchronize()
    assert rel(dr.cpu().numpy().reshape(shape, order="F"), r) < RHS_TOL
    # The inflow sponges force the state towards a wave of O(1) amplitude
    # that the device forms with its own exp / sin / cos: steps agree to
    # 1e-12 of the larger of the state and that target.
    scale_t = 0.0
    if ispg in (2, 3):
        L.a3_inflow_target.argtypes = [ctypes.POINTER(type(orc.g)), ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        t = np.zeros(10)
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                L.a3_inflow_target(ctypes.byref(orc.g), i, j, t.ctypes.data)
                scale_t = max(scale_t, np.abs(t).max())
    drv = mk()
    v_ref = case["v"].copy(order="F")
    v_gpu = case["v"].copy(order="F")
    for s in range(4):
        res_ref = orc.step(v_ref)
        res_gpu = drv.step(v_gpu, nsteps=1)[0]
        err = np.abs(v_gpu - v_ref).max() / max(np.abs(v_ref).max(), scale_t)
        assert err < STEP_TOL, s
        assert abs(res_gpu - res_ref) <= 1e-10 * res_ref, s


def test_forced_top_boundary_matches_oracle(cuda):
    """top = 1 (src/itrbc3d.f90:145-196, src/rhsbc3d.f90:129-160): the
    incoming acoustic wave on row ny, formed on the device from the mean flow,
    x, x0 and wamp; RHS, LHS and steps against the oracle, to 1e-12 of the
    larger of the state and the wave (the device forms the wave with its own
    exp, sin and cos)."""
    import ctypes

    import torch
    from adi3dcase import _lib, ptr

    from lns3d_gb300 import ImpDrv3D
    from lns3d_gb300.cases import shear_layer

    nx, ny = 40, 33
    case = shear_layer(nx=nx, ny=ny, seed=12)
    case = dict(case, params=dict(case["params"], top=1))
    rng = np.random.default_rng(15)
    wamp = rng.uniform(0.5, 1.5, nx)
    orc = Oracle3D(case, cflmax=20.0, loctime=1, x0=-2.0, wamp=wamp)
    mk = lambda: ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1, x=case["x"], x0=-2.0,
                          wamp=wamp)
    L = _lib()
    L.a3_top_target.argtypes = [ctypes.POINTER(type(orc.g)), ctypes.c_int, ctypes.c_void_p]
    t = np.zeros(10)
    scale_t = 0.0
    for i in range(1, nx + 1):
        L.a3_top_target(ctypes.byref(orc.g), i, t.ctypes.data)
        scale_t = max(scale_t, np.abs(t).max())
    drv = mk()
    mat = torch.zeros(125 * nx * ny, dtype=torch.complex128, device="cuda")
    drv.lhs(2, mat)
    torch.cuda.synchronize()
    assert rel(mat.cpu().numpy().reshape((5, 5, 5, nx, ny), order="F"), orc.lhs(2)) < OPS_TOL
    shape = (5, nx, ny)
    v = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    vold = np.asfortranarray(v + 1e-3 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
    r = orc.lrhs(v)
    L.a3_rbe(ctypes.byref(orc.g), ptr(r), ptr(v), ptr(vold), ptr(orc.dtl))
    L.a3_rhsbc(ctypes.byref(orc.g), ptr(r), ptr(v))
    dev = lambda a: torch.from_numpy(a.ravel(order="F")).cuda()
    dv, dvo = dev(v), dev(vold)
    dr = torch.zeros_like(dv)
    drv.rhs(dv, dvo, dr, torch.zeros(1, dtype=torch.float64, device="cuda"))
    torch.cuda.synchronize()
    got = dr.cpu().numpy().reshape(shape, order="F")
    assert np.abs(got - r).max() / max(np.abs(r).max(), scale_t) < RHS_TOL
    drv = mk()
    v_ref = case["v"].copy(order="F")
    v_gpu = case["v"].copy(order="F")
    for s in range(4):
        res_ref = orc.step(v_ref)
        res_gpu = drv.step(v_gpu, nsteps=1)[0]
        assert np.abs(v_gpu - v_ref).max() / max(np.abs(v_ref).max(), scale_t) < STEP_TOL, s
        assert abs(res_gpu - res_ref) <= 1e-10 * res_ref, s


@pytest.mark.parametrize("wallt", [0, 1])
def test_bump_wall_matches_oracle(cuda, wallt):
    """wall = 3, the bump (src/itrbc3d.f90:46-121, src/rhsbc3d.f90:45-104,
    src/lhsbc2f3d.f90:41-48): eta LHS, RHS and steps against the oracle."""
    import ctypes

    import torch
    from adi3dcase import _lib, ptr

    from lns3d_gb300 import ImpDrv3D
    from lns3d_gb300.cases import shear_layer

    nx, ny = 40, 33
    case = shear_layer(nx=nx, ny=ny, seed=13)
    case = dict(case, params=dict(case["params"], wall=3, wallt=wallt))
    rng = np.random.default_rng(16)
    bump = np.asfortranarray(1e-3 * (rng.standard_normal((5, nx)) + 1j * rng.standard_normal((5, nx))))
    orc = Oracle3D(case, cflmax=20.0, loctime=1, bump=bump)
    mk = lambda: ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=20.0, loctime=1, bump=bump)
    drv = mk()
    mat = torch.zeros(125 * nx * ny, dtype=torch.complex128, device="cuda")
    drv.lhs(2, mat)
    torch.cuda.synchronize()
    assert rel(mat.cpu().numpy().reshape((5, 5, 5, nx, ny), order="F"), orc.lhs(2)) < OPS_TOL
    shape = (5, nx, ny)
    v = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    vold = np.asfortranarray(v + 1e-3 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
    L = _lib()
    r = orc.lrhs(v)
    L.a3_rbe(ctypes.byref(orc.g), ptr(r), ptr(v), ptr(vold), ptr(orc.dtl))
    L.a3_rhsbc(ctypes.byref(orc.g), ptr(r), ptr(v))
    dev = lambda a: torch.from_numpy(a.ravel(order="F")).cuda()
    dv, dvo = dev(v), dev(vold)
    dr = torch.zeros_like(dv)
    drv.rhs(dv, dvo, dr, torch.zeros(1, dtype=torch.float64, device="cuda"))
    torch.cuda.synchronize()
    assert rel(dr.cpu().numpy().reshape(shape, order="F"), r) < RHS_TOL
    drv = mk()
    v_ref = case["v"].copy(order="F")
    v_gpu = case["v"].copy(order="F")
    for s in range(4):
        res_ref = orc.step(v_ref)
        res_gpu = drv.step(v_gpu, nsteps=1)[0]
        assert rel(v_gpu, v_ref) < STEP_TOL, s
        assert abs(res_gpu - res_ref) <= 1e-10 * res_ref, s

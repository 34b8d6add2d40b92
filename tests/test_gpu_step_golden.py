"""GPU steps against the reference's own step code: golden files written by
the translated reference program (tests/golden/gen_step_golden.py) on the
seeded cases, which are regenerated here with the same arguments.

The reference runs itrBC (itrBC3D) once before its step loop
(src/impdrv.f90:160, src/impdrv3d.f90:125-126), so the GPU runs do too.
Bars: the state within 1e-12 of its largest entry after every listed run
(the GPU fuses multiply-adds, the reference does not), the residual history
within 1e-10 relative.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STATE_TOL = 1e-12
RES_TOL = 1e-10


def golden(name):
    import sys

    sys.path.insert(0, GOLDEN)
    import gen_step_golden

    kind, cargs, rargs = gen_step_golden.GOLDEN[name]
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return kind, cargs, dict(rargs), d


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("name", ["step2d_vortex128", "step2d_vortex_tri", "step2d_vortex_midpoint"])
def test_step2d_matches_reference_golden(cuda, name):
    from lns3d_gb300 import ImpDrv2D
    from lns3d_gb300.cases import vortex2d

    kind, cargs, rargs, d = golden(name)
    case = vortex2d(**cargs)
    nsteps = rargs.pop("nsteps")
    drv = ImpDrv2D(case["params"], case["metrics"], case["bnt"], case["pot"], cflmax=rargs.get("cflmax", 1.0),
                   loctime=rargs.get("loctime", 0), ilhs=rargs.get("ilhs", 1), impl=rargs.get("impl", 1))
    v = case["v"].copy(order="F")
    drv.itrbc(v)
    res = drv.step(v, nsteps=nsteps)
    assert rel(v, d["v"]) < STATE_TOL, rel(v, d["v"])
    assert np.abs(np.asarray(res) - d["hist"]).max() <= RES_TOL * d["hist"].max()


@pytest.mark.parametrize("name", ["step3d_shear", "step3d_shear_two_step", "step3d_shear_midpoint"])
def test_step3d_matches_reference_golden(cuda, name):
    from lns3d_gb300 import ImpDrv3D
    from lns3d_gb300.cases import shear_layer

    kind, cargs, rargs, d = golden(name)
    case = shear_layer(**cargs)
    nsteps = rargs.pop("nsteps")
    drv = ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=rargs.get("cflmax", 20.0),
                   loctime=rargs.get("loctime", 1), impl=rargs.get("impl", 1))
    v = case["v"].copy(order="F")
    drv.itrbc(v)
    res = drv.step(v, nsteps=nsteps)
    assert rel(v, d["v"]) < STATE_TOL, rel(v, d["v"])
    assert np.abs(np.asarray(res) - d["hist"]).max() <= RES_TOL * d["hist"].max()


def test_step3d_periodic_inviscid_box_matches_reference_golden(cuda):
    """The reference's test/3d deck (cfl.inp): periodic in both directions,
    inviscid, two correctors per step."""
    from lns3d_gb300 import ImpDrv3D
    from lns3d_gb300.cases import acoustic_box

    kind, cargs, rargs, d = golden("step3d_box")
    case = acoustic_box(**cargs)
    drv = ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=rargs["cflmax"], dtmax=rargs["dtmax"],
                   loctime=rargs["loctime"])
    v = case["v"].copy(order="F")
    drv.itrbc(v)
    res = drv.step(v, nsteps=rargs["nsteps"], niter=rargs["niter"])
    assert rel(v, d["v"]) < STATE_TOL, rel(v, d["v"])
    want = d["hist"][rargs["niter"] - 1::rargs["niter"]]
    assert np.abs(np.asarray(res) - want).max() <= RES_TOL * want.max()


def test_linear_2d_step_matches_reference_golden(cuda):
    """The linear 2D step (src/impdrv.f90 with linear = 1) on the
    wall-bounded shear layer."""
    from lns3d_gb300 import ImpDrvLin2D
    from lns3d_gb300.cases import shear_layer

    kind, cargs, rargs, d = golden("step2d_lin_shear")
    case = shear_layer(**cargs)
    drv = ImpDrvLin2D(case["params"], case["metrics"], case["vm"], cflmax=rargs["cflmax"], loctime=rargs["loctime"])
    v = np.asfortranarray(case["v"].real)
    drv.itrbc(v)
    res = drv.step(v, nsteps=rargs["nsteps"])
    assert rel(v, d["v"]) < STATE_TOL, rel(v, d["v"])
    assert np.abs(np.asarray(res) - d["hist"]).max() <= RES_TOL * d["hist"].max()


@pytest.mark.parametrize("name", ["step2d_lin_open", "step2d_lin_sym", "step2d_lin_nr", "step2d_lin_nr_right"])
def test_linear_2d_open_xi_matches_reference_golden(cuda, name):
    """The linear 2D step with a non-periodic xi direction: the zero-
    disturbance planes (left 0, right 0: src/itrbc.f90:310-316, 534-540,
    src/rhsbc.f90:189-191, 238-240, src/lhsbc1f.f90:108-115, 183-190,
    src/lhsbc2f.f90:124-131, 164-171) with the boundary-closure xi rows, and
    the symmetry plane (left 7: mirrored stencils, src/grad.f90:155-249, the
    symmetric rows of src/lhsbs1f.f90, v = 0 and r = 0 for the second
    velocity component, src/itrbc.f90:525-527, src/rhsbc.f90:229-231), and
    the nonreflecting planes (left 1, right 1: the density row above nbl,
    src/itrbc.f90:318-346, 542-566, src/rhsbc.f90:193-201, 242-250,
    src/lhsbc1f.f90:117-139, 192-221, src/lhsbc2f.f90:133-144, 173-184)."""
    import sys

    from lns3d_gb300 import ImpDrvLin2D

    sys.path.insert(0, GOLDEN)
    import gen_step_golden

    kind, cargs, rargs, d = golden(name)
    case = gen_step_golden.open_layer(**cargs)
    drv = ImpDrvLin2D(case["params"], case["metrics"], case["vm"], cflmax=rargs["cflmax"], loctime=rargs["loctime"],
                      nbl=rargs.get("module", {}).get("nbl", 0))
    v = np.asfortranarray(case["v"].real)
    drv.itrbc(v)
    res = drv.step(v, nsteps=rargs["nsteps"])
    assert rel(v, d["v"]) < STATE_TOL, rel(v, d["v"])
    assert np.abs(np.asarray(res) - d["hist"]).max() <= RES_TOL * d["hist"].max()


def test_reference_test2d_fixture(cuda):
    """The reference's own test/2d case (its grid, metric, mean and initial
    files, its deck lns3d.inp): 10 steps of the linear 2D step through the
    C ABI, against the restart files the reference wrote at steps 4, 8, 10."""
    from lns3d_gb300 import ImpDrvLin2D, refio
    from lns3d_gb300.cases import kz_of

    d = np.load(os.path.join(GOLDEN, "step2d_test2d.npz"))
    deck = refio.parse_deck(str(d["deck"]))
    nx, ny = d["x"].shape
    inviscid = deck["Re"] == 0.0
    params = dict(nx=nx, ny=ny, dxi=1.0 / (nx - 1), deta=1.0 / (ny - 1), Ma=deck["Ma"],
                  Re=1e99 if inviscid else deck["Re"], Pr=deck["Pr"], gamma=1.4, gamma1=0.4, omega=0.0,
                  kz=kz_of(deck["Lz"]), alfa=1.0, xper=int(deck["xper"]), yper=int(deck["yper"]),
                  navier=0 if inviscid else 1, wall=-1, wallt=-1, top=-1, optx=deck["optx"], opty=deck["opty"])
    metrics = {k[2:]: d[k] for k in d.files if k.startswith("m_")}
    drv = ImpDrvLin2D(params, metrics, d["vm"], cflmax=deck["cflmax"], dtmax=deck["dtmax"], loctime=deck["loctime"],
                      impl=deck["impl"])
    v = np.asfortranarray(d["v0"])
    drv.itrbc(v)
    res = []
    done = 0
    for step in (4, 8, 10):
        res.extend(drv.step(v, nsteps=step - done, niter=deck["niter"]))
        done = step
        want = d["v_step%d" % step]
        assert rel(v, want) < STATE_TOL, (step, rel(v, want))
    # ires = 1: the reference also measures the residual after each update
    want = d["hist"][0::deck["niter"] + 1]
    assert np.abs(np.asarray(res) - want).max() <= RES_TOL * want.max()


@pytest.mark.parametrize("name", ["step3d_open", "step3d_open_wave", "step3d_open_eig", "step3d_open_hold",
                                  "step3d_open_acoustic", "step3d_open_acoustic_both",
                                  "step3d_sym_left", "step3d_sym_both", "step3d_sym_smooth"])
def test_step3d_nonperiodic_xi_matches_reference_golden(cuda, name):
    """A non-periodic xi direction: the boundary-closure rows of the xi LHS
    (src/lhsbt1f3d.f90), the zero-disturbance, incoming-wave,
    eigenfunction and acoustic inflow planes, the zero-disturbance,
    eigenfunction, acoustic and held outflow planes
    (src/itrbc3d.f90:203-414, src/rhsbc3d.f90:167-324,
    src/lhsbc1f3d.f90:412-448), the symmetry planes (mirrored stencils,
    src/lhsbs1f3d.f90) and the cpenta2bc-factored xi sweep."""
    import sys

    from lns3d_gb300 import ImpDrv3D

    sys.path.insert(0, GOLDEN)
    import gen_step_golden

    kind, cargs, rargs, d = golden(name)
    case = gen_step_golden.open_layer(**cargs)
    drv = ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=rargs["cflmax"], loctime=rargs["loctime"],
                   x=case["x"], x0=rargs.get("x0", 0.0), profile=case.get("profile"), eps_e=rargs.get("eps_e", 0.0),
                   lalpha=rargs.get("module", {}).get("lalpha", 0j))
    v = case["v"].copy(order="F")
    drv.itrbc(v)
    res = drv.step(v, nsteps=rargs["nsteps"])
    assert rel(v, d["v"]) < STATE_TOL, rel(v, d["v"])
    assert np.abs(np.asarray(res) - d["hist"]).max() <= RES_TOL * d["hist"].max()


@pytest.mark.parametrize("name", ["step2d_vortex_open", "step2d_vortex_open_sym", "step2d_vortex_mirror",
                                  "step2d_vortex_hold"])
def test_step2d_nonperiodic_xi_matches_reference_golden(cuda, name):
    """The nonlinear 2D step with a non-periodic xi direction: Riemann planes
    on both sides (left.pot / right.pot), and the symmetry plane with the
    right plane extrapolated over a viscous layer that itrBC moves, and
    mirrored symmetry planes on both sides with the smoother."""
    from lns3d_gb300 import ImpDrv2D
    from lns3d_gb300.cases import vortex2d_open

    kind, cargs, rargs, d = golden(name)
    case = vortex2d_open(**cargs)
    nsteps = rargs.pop("nsteps")
    module = rargs.pop("module", {})
    drv = ImpDrv2D(case["params"], case["metrics"], case["bnt"], case["pot"], cflmax=rargs.get("cflmax", 1.0),
                   loctime=rargs.get("loctime", 0), left_far=case["left_far"], right_far=case["right_far"],
                   extrap=case["extrap"], nbl=module.get("nbl", 0), update_nbl=module.get("update_nbl", 0),
                   eps_e=rargs.get("eps_e", 0.0))
    v = case["v"].copy(order="F")
    drv.itrbc(v)
    res = drv.step(v, nsteps=nsteps)
    assert rel(v, d["v"]) < STATE_TOL, rel(v, d["v"])
    assert np.abs(np.asarray(res) - d["hist"]).max() <= RES_TOL * d["hist"].max()

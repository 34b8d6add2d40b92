"""The hand restatements of the implicit steps (oracle/adi3d_oracle.c,
oracle/impdrv2d_oracle.c) against the reference's own step code.

The reference program and the routines of its steps are translated to C by
oracle/f90sub2c.py (oracle/_ref/libref_step.so) and run here as
``lns3d < deck`` on the synthetic cases written in the reference's file
formats.  The restatements must give the same states and residual history:
bit for bit where both evaluate the same expressions in the same order
(they are compiled without FMA contraction, as the translation is).  The
GPU tests compare the GPU with the restatements at 1e-12 and with golden
files of this translated reference (tests/golden/step*.npz).
"""
import numpy as np
import pytest

refstep = pytest.importorskip("oracle.refstep")
if not refstep.available():
    pytest.skip("the translated reference is not built (oracle/_ref/libref_step.so)", allow_module_level=True)

import refcase  # noqa: E402
from lns3d_gb300.cases import shear_layer, vortex2d  # noqa: E402
from oracle.adi3d import Oracle3D  # noqa: E402
from oracle.impdrv2d import Oracle2D  # noqa: E402


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


# ----------------------------------------------------------------------------
# 3D linearised single-mode step (src/impdrv3d.f90)
# ----------------------------------------------------------------------------

CASES_3D = [
    dict(id="be", impl=1, niter=1),
    dict(id="be_niter2", impl=1, niter=2),
    dict(id="two_step", impl=2, niter=1),
    dict(id="midpoint", impl=3, niter=1),
    dict(id="global_dt", impl=1, niter=1, loctime=0, cflmax=5.0),
    dict(id="wall2_wallt0", impl=1, niter=1, wall=2, wallt=0),
    dict(id="sixth_order", impl=1, niter=1, optx=0, opty=0),
    dict(id="top1_forced", impl=1, niter=1, top=1),
    dict(id="sponge1", impl=1, niter=1, deck=dict(ispg=1, As=1.0, Ns=3, xs=0.7, xt=1.0)),
    dict(id="sponge5", impl=1, niter=1, deck=dict(ispg=5, As=1.0, Ns=3, xs=0.7, xt=1.0, As2=0.5, Ns2=2, xs2=0.3,
                                                 xt2=0.0)),
    dict(id="smoother", impl=1, niter=1, deck=dict(eps_e=0.01)),
]


def _case3d(cfg, nx=24, ny=17, seed=2):
    case = shear_layer(nx=nx, ny=ny, seed=seed)
    for k in ("wall", "wallt", "optx", "opty", "top"):
        if k in cfg:
            case["params"][k] = cfg[k]
    return case


@pytest.mark.parametrize("cfg", CASES_3D, ids=[c["id"] for c in CASES_3D])
def test_step3d_restatement_equals_reference(cfg):
    nsteps = 3
    case = _case3d(cfg)
    kw = dict(impl=cfg["impl"], niter=cfg["niter"], loctime=cfg.get("loctime", 1), cflmax=cfg.get("cflmax", 20.0))
    deck = cfg.get("deck", {})
    v_ref, hist, run = refcase.run3d(case, nsteps, **kw, **deck)
    try:
        assert run.prog.oob() == 0
        okw = {}
        if deck.get("ispg"):   # the sponge arrays as the reference's init_sponge formed them
            spg2 = run.prog.array("spg2")
            okw = dict(ispg=deck["ispg"], spg=np.array(run.prog.array("spg")),
                       spg2=None if spg2 is None else np.array(spg2))
        if deck.get("eps_e"):
            okw["eps_e"] = deck["eps_e"]
        orc = Oracle3D(case, cflmax=kw["cflmax"], loctime=kw["loctime"],
                       x0=0.0, wamp=np.ones(case["params"]["nx"]) if cfg.get("top") == 1 else None, **okw)
        v = case["v"].copy(order="F")
        orc.itrbc(v)        # the driver's itrBC3D before the step loop (src/impdrv3d.f90:125-126)
        res = []
        for _ in range(nsteps):
            if cfg["impl"] == 1:
                res.append(orc.step(v, niter=cfg["niter"]))
            else:
                res.append(orc.step_impl(v, cfg["impl"], niter=cfg["niter"]))
        assert np.array_equal(v, v_ref), rel(v, v_ref)
        # the history holds one line per corrector; the oracle returns the last of each step
        assert np.array_equal(np.array(res), hist[cfg["niter"] - 1::cfg["niter"]])
    finally:
        run.close()


def test_periodic_inviscid_box_equals_reference():
    """The reference's test/3d case (test/3d/cfl.inp): periodic in both
    directions (cpenta1p for the eta sweep), inviscid (Re = 0 in the deck),
    two correctors per step, global time step."""
    from lns3d_gb300.cases import acoustic_box

    case = acoustic_box(nx=24, ny=21)
    nsteps = 3
    v_ref, hist, run = refcase.run3d(case, nsteps, Re=0.0, Pr=1.0, dtmax=0.0070710678e10, cflmax=0.1, niter=2,
                                     loctime=0, Lz=case["span"])
    try:
        assert run.prog.oob() == 0 and run.prog.get("navier") == 0
        orc = Oracle3D(case, cflmax=0.1, loctime=0, dtmax=0.0070710678e10)
        v = case["v"].copy(order="F")
        orc.itrbc(v)
        res = [orc.step(v, niter=2) for _ in range(nsteps)]
        assert np.array_equal(v, v_ref), rel(v, v_ref)
        assert np.array_equal(np.array(res), hist[1::2])
    finally:
        run.close()


def test_operators_equal_reference():
    """genmtrx(vm, kz, vm) of the linear run (src/lns3d.f90:149): every
    frozen operator array bit for bit."""
    case = _case3d({})
    _, _, run = refcase.run3d(case, 1)
    try:
        orc = Oracle3D(case, cflmax=20.0, loctime=1)
        for k in ("Ah", "Bh", "Dh", "Dhi", "Vh11", "Vh12", "Vh22", "ABhi"):
            assert np.array_equal(run.prog.array(k), orc.ops[k]), k
    finally:
        run.close()


def test_lhs_equal_reference():
    """lhs1f3D / lhs2f3D with their boundary rows (src/lhs1f3d.f90,
    src/lhs2f3d.f90, src/lhsbt2f3d.f90, src/lhsbc2f3d.f90), called one at a
    time on the module state of a run."""
    case = _case3d({})
    _, _, run = refcase.run3d(case, 1)
    try:
        P = run.prog
        nx, ny = case["params"]["nx"], case["params"]["ny"]
        orc = Oracle3D(case, cflmax=20.0, loctime=1)
        vm = np.asfortranarray(case["vm"])
        dtl = np.zeros((nx, ny), order="F")
        P.set("istep", 0)
        P.call("set_time_step", vm, dtl)
        assert np.array_equal(dtl, orc.dtl)
        v = np.asfortranarray(case["v"])
        P.set("alfa", 1.0)
        for direction, name, ops in ((1, "lhs1f3d", ("Ah", "Dh", "Dhi", "Vh11", "ABhi")),
                                     (2, "lhs2f3d", ("Bh", "Dh", "Dhi", "Vh22", "ABhi"))):
            mat = np.zeros((5, 5, 5, nx, ny), np.complex128, order="F")
            P.call(name, mat, *[np.asfortranarray(P.array(k)) for k in ops], dtl, v)
            assert np.array_equal(mat, orc.lhs(direction)), name
    finally:
        run.close()


def test_rhs_equal_reference():
    """lrhs3D with cgrad, cgrad2, cgradbc (src/lrhs3d.f90:33-218)."""
    case = _case3d({})
    _, _, run = refcase.run3d(case, 1)
    try:
        P = run.prog
        orc = Oracle3D(case, cflmax=20.0, loctime=1)
        v = np.asfortranarray(case["v"])
        r = np.zeros_like(v)
        P.call("lrhs3d", v, r, np.asfortranarray(case["vm"]), np.asfortranarray(case["x"]),
               np.asfortranarray(case["y"]))
        assert np.array_equal(r, orc.lrhs(v))
    finally:
        run.close()


def test_reference_as_written_shows_the_row_n3_fault():
    """The complex boundary solve as written updates row n-1 from row n-3
    with transposed indices (src/cpenta1bc.f:675): the translated reference
    performs those transposed accesses and its state differs from the
    corrected one, which the restatement and the GPU follow."""
    case = _case3d({})
    v_fix, _, run_fix = refcase.run3d(case, 2)
    v_asis, _, run_asis = refcase.run3d(case, 2, asis=True)
    try:
        assert run_fix.prog.transposed() == 0
        assert run_asis.prog.transposed() > 0
        assert rel(v_asis, v_fix) > 1e-10
    finally:
        run_fix.close()
        run_asis.close()


# ----------------------------------------------------------------------------
# 2D nonlinear step (src/impdrv.f90, linear = 0)
# ----------------------------------------------------------------------------

CASES_2D = [
    dict(id="penta", ilhs=1, impl=1),
    dict(id="tri", ilhs=0, impl=1),
    dict(id="two_step", ilhs=1, impl=2),
    dict(id="midpoint", ilhs=1, impl=3),
    dict(id="niter2", ilhs=1, impl=1, niter=2),
    dict(id="wall1_isothermal", ilhs=1, impl=1, wall=1, wallt=0),
    dict(id="local_dt", ilhs=1, impl=1, loctime=1),
    dict(id="top3_held", ilhs=1, impl=1, top=3, Ma=0.5),
    dict(id="sponge2", ilhs=1, impl=1, deck=dict(ispg=2, As=1.0, Ns=3, xs=0.7, xt=1.0)),
    dict(id="smoother", ilhs=1, impl=1, deck=dict(eps_e=0.01)),
    dict(id="tri_smoother", ilhs=0, impl=1, deck=dict(eps_e=0.01)),
]


@pytest.mark.parametrize("cfg", CASES_2D, ids=[c["id"] for c in CASES_2D])
def test_step2d_restatement_equals_reference(cfg):
    nsteps = 3
    case = vortex2d(nx=24, ny=20, seed=3)
    for k in ("wall", "wallt", "top"):
        if k in cfg:
            case["params"][k] = cfg[k]
    niter = cfg.get("niter", 1)
    loctime = cfg.get("loctime", 0)
    deck = cfg.get("deck", {})
    v_ref, hist, run = refcase.run2d(case, nsteps, ilhs=cfg["ilhs"], impl=cfg["impl"], niter=niter,
                                     loctime=loctime, **deck)
    try:
        assert run.prog.oob() == 0
        okw = {}
        if deck.get("ispg"):
            okw = dict(ispg=deck["ispg"], spg=np.array(run.prog.array("spg")), spg2=np.array(run.prog.array("spg2")))
        if deck.get("eps_e"):
            okw["eps_e"] = deck["eps_e"]
        orc = Oracle2D(case, cflmax=1.0, loctime=loctime, ilhs=cfg["ilhs"], impl=cfg["impl"], **okw)
        v = case["v"].copy(order="F")
        orc.itrbc(v)
        res = [orc.step(v, niter=niter) for _ in range(nsteps)]
        assert np.array_equal(v, v_ref), rel(v, v_ref)
        assert np.array_equal(np.array(res), hist[niter - 1::niter])
    finally:
        run.close()


# ----------------------------------------------------------------------------
# the two translations of the solvers agree
# ----------------------------------------------------------------------------

@pytest.mark.parametrize("asis", [True, False], ids=["as_written", "row_n3_corrected"])
@pytest.mark.parametrize("solver", ["cpenta1bc", "cpenta2bc", "cpenta1p", "cpenta2p", "penta1bc", "penta2bc",
                                    "penta1p", "penta2p"])
def test_solver_translations_agree(solver, asis):
    """The solvers inside the translated program (f90sub2c.py, fixed-form
    reader) equal the solver restatement bit for bit: as written against
    its reference-compatible mode (which tests/test_oracle.py pins to the
    separately translated solvers, f77sub2c.py), and with the row n-3 fault
    corrected against its default mode."""
    import oracle
    import pentacase

    c = pentacase.info(solver)
    if not asis and not (c["complex"] and not c["periodic"]):
        pytest.skip("the correction touches the complex boundary solvers only")
    case = pentacase.make_case(solver, 20, 6, seed=4)
    flags = oracle.COMPAT_PERIODIC_SLOT | (oracle.COMPAT_CBC_RHS if asis else 0)
    want = pentacase.run_oracle(case, code=2, flags=flags)
    P = refstep.RefProgram(asis=asis)
    try:
        out = pentacase.copy(case)
        d = pentacase.dims(case)
        args = [d[0], d[1], 5, out["mat"], out["rhs"]]
        if c["periodic"]:
            args += [out["per"], out["per2"]]
        if c["complex"]:
            args += [2]
        P.call(solver, *args)
        assert np.array_equal(out["rhs"], want["rhs"])
    finally:
        P.close()

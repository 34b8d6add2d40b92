"""The reference's own parabolic-cylinder fixture on the GPU.

test/pcyl/sweep=35/M=0.8/Re=1e5/ref holds the converged boundary-layer
mean flow of the swept leading edge (384 x 128, body fitted) with the
metric.dat, top.pot and right.pot of its run; tests/golden/gen_pcyl_golden.py
stores it with what the translated reference program does with it under
the case's res.inp deck: the non-periodic xi direction with the symmetry
plane on the left (left 2), the Riemann outflow on the right (right 0) and
its extrapolation over the viscous layer (extrap 1, nbl from itrBC).

Bars: itrBC and the time step within 1e-14 of the largest entry, the LHS
on the boundary columns within 1e-13, the RHS within 5e-11 of its largest
entry (the state is converged, so the RHS is 2e-3 where its terms are of
order one: the reference built with fused multiply-adds differs from
itself by 1.0e-11 of that largest entry there); the state within 2e-12 of its
largest entry after one step and 2e-11 after four, the residual history
within 1e-10 relative.  The reference built with fused multiply-adds
differs from itself by 7.9e-14 after one step and 3.7e-13 after four
(2.0e-12 in the residual history): CFL 400 on the global time step makes
each step an ill-conditioned solve.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pcyl_sweep35.npz")


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def driver(case):
    from lns3d_gb300 import ImpDrv2D

    r = case["run"]
    return ImpDrv2D(case["params"], case["metrics"], case["bnt"], case["pot"], cflmax=r["cflmax"],
                    dtmax=r["dtmax"], loctime=r["loctime"], theta=r["theta"], eps_e=r["eps_e"],
                    right_far=case["right_far"], extrap=r["extrap"], nbl=r["nbl"], update_nbl=r["update_nbl"])


@pytest.fixture(scope="module")
def pcyl():
    from lns3d_gb300 import cases

    d = np.load(FIXTURE)
    return d, cases.pcyl(d)


def test_pcyl_boundary_rows_match_reference(cuda, pcyl):
    """itrBC, set_time_step, genmtrx + rbe + rhsBC and both LHS on the
    fixture's state, on the columns next to the xi planes."""
    import torch

    d, case = pcyl
    nx, ny = case["params"]["nx"], case["params"]["ny"]
    cols, edge = d["cols"], d["edge"]
    drv = driver(case)
    v = torch.from_numpy(case["v"].ravel(order="F").copy()).to(cuda)
    drv.itrbc(v)
    vh = v.cpu().numpy().reshape(5, nx, ny, order="F")
    assert rel(vh[:, cols, :], d["v_bc"]) < 1e-14, rel(vh[:, cols, :], d["v_bc"])
    r = torch.zeros_like(v)
    drv.rhs(v, v.clone(), r)
    torch.cuda.synchronize()
    assert rel(drv.field("dtl")[cols, :], d["dtl"]) < 1e-14
    rh = r.cpu().numpy().reshape(5, nx, ny, order="F")[:, cols, :]
    assert rel(rh, d["r"]) < 5e-11, rel(rh, d["r"])
    for direction, key in ((1, "lhs1"), (2, "lhs2")):
        mat = torch.zeros(125 * nx * ny, dtype=torch.float64, device=cuda)
        drv.lhs(direction, v, mat)
        m = mat.cpu().numpy().reshape(5, 5, 5, nx, ny, order="F")[:, :, :, edge, :]
        assert rel(m, d[key]) < 1e-13, (key, rel(m, d[key]))
    drv.close()


@pytest.mark.parametrize("nsteps", [1, 4])
def test_pcyl_steps_match_reference(cuda, pcyl, nsteps):
    """The step on the reference's converged pcyl mean flow: the state on
    the stored columns, the residual history and the residual level."""
    d, case = pcyl
    cols = d["cols"]
    drv = driver(case)
    v = case["v"].copy(order="F")
    drv.itrbc(v)
    res = drv.step(v, nsteps=nsteps)
    want, tol = (d["v1"], 2e-12) if nsteps == 1 else (d["vN"], 2e-11)
    assert rel(v[:, cols, :], want) < tol, rel(v[:, cols, :], want)
    hist = d["hist"][:nsteps]
    assert np.abs(np.asarray(res) - hist).max() <= 1e-10 * hist.max()
    # the stored solution is near its converged level under this deck
    assert 1e-3 < res[0] < 5e-3
    drv.close()


def test_riemann_plane_needs_its_far_field(cuda, pcyl):
    """A Riemann xi plane whose far field was never uploaded fails the first
    step with LNS_ERR_ARG (the option checks of creation run on the CPU in
    tests/test_capi.py)."""
    from lns3d_gb300 import ImpDrv2D
    from lns3d_gb300._lib import LnsError

    _, case = pcyl
    r = case["run"]
    drv = ImpDrv2D(case["params"], case["metrics"], case["bnt"], case["pot"], cflmax=r["cflmax"],
                   dtmax=r["dtmax"], eps_e=r["eps_e"], extrap=r["extrap"], nbl=r["nbl"])
    v = case["v"].copy(order="F")
    with pytest.raises(LnsError):
        drv.step(v, nsteps=1)
    drv.close()

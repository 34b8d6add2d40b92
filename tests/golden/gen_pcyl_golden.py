"""Generates tests/golden/pcyl_sweep35.npz: the reference's own parabolic-
cylinder fixture (test/pcyl/sweep=35/M=0.8/Re=1e5/ref: the converged
boundary-layer mean flow of the swept leading edge on its 384 x 128 body-
fitted grid, with the metric.dat, top.pot and right.pot of that run) and
what the translated reference program (oracle/_ref/libref_step.so) does
with it, for the GPU tests, which run where the reference tree is absent.

The run is the case's res.inp deck (src/lns3d.f90 < res.inp with the
&extras namelist of mean.nml: nbl = 32, update_nbl) with the physical
parameters of the stored solution, which its README gives as Pr = 0.7 and
which has an adiabatic wall (its wall temperature falls from the
stagnation value along the body): Pr 0.7 and wallt 1 in place of the
deck's 1.0 and 0.  Everything else is the deck's: Ma 0.8, Re 1e5, CFL 400
with dtmax 1 and one global time step, fourth-order stencils, a non-
periodic xi direction with the symmetry plane on the left (left 2) and the
Riemann outflow on the right (right 0) with first-order extrapolation in
the viscous layer (extrap 1), the Riemann top, the smoother at eps_e 0.01.

Stored: the inputs (metrics, the state, the two .pot files) and, from two
runs of the program (one step, and NSTEPS steps), the state on a subset of
columns (every eighth, and the six next to each xi boundary, which hold
the rows a non-periodic xi direction adds), the residual history and nbl
after the last itrBC of each run; and, on the fixture's state after
itrBC, set_time_step, genmtrx + rbe (vold = v) + rhsBC on
the same columns and both LHS (lhs1f with lhsbt1f and lhsbc1f, lhs2f with
lhsbt2f and lhsbc2f) on rows 1..3 and nx-2..nx of every xi line.

Run from the repository root:  python tests/golden/gen_pcyl_golden.py
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import refcase  # noqa: E402
from lns3d_gb300 import refio  # noqa: E402

CASE_DIR = "/root/reference/test/pcyl/sweep=35/M=0.8/Re=1e5"
NSTEPS = 4
# columns (0-based) on which the final state and the boundary rows are kept
COLS = sorted(set([0, 1, 2, 3, 4, 5] + list(range(8, 378, 8)) + [378, 379, 380, 381, 382, 383]))
# columns of the stored LHS: rows 1..3 and nx-2..nx of every xi line
EDGE = [0, 1, 2, 381, 382, 383]


def deck(nsteps):
    text = open(os.path.join(CASE_DIR, "res.inp")).read()
    subs = [("1.0                             ! Pr number", "0.7                             ! Pr number"),
            ("20000                           ! nstep", "%-31d ! nstep" % nsteps),
            ("1, 1000                         ! itout, ntout", "1, 1000000                      ! itout, ntout"),
            ("0, 0, 2, 0, 0                   ! BC: top, wall, left, right, wallt",
             "0, 0, 2, 0, 1                   ! BC: top, wall, left, right, wallt")]
    for a, b in subs:
        assert a in text, a
        text = text.replace(a, b)
    return text


def run(ref, nsteps, boundary_rows=False):
    """The program on the fixture for nsteps steps: the final state, the
    totres history, nbl and alfa; with boundary_rows, on the fixture's
    state after itrBC (nbl_bc, v_bc): set_time_step (dtl), genmtrx + rbe
    with vold = v + rhsBC (r), and lhs1f, lhs2f on the EDGE columns, called
    one at a time on the module state the run left."""
    from oracle.refstep import RefProgram

    r = refcase.Run()
    try:
        for f in ("grid.dat", "metric.dat", "top.pot", "right.pot"):
            shutil.copy(os.path.join(ref, f), r.path(f))
        shutil.copy(os.path.join(ref, "mean.R.0"), r.path("output.R.0"))
        r.prog = P = RefProgram()
        P.set("nbl", 32)        # mean.nml's &extras
        P.set("update_nbl", 1)
        P.run(r.dir, deck(nsteps))
        assert P.oob() == 0
        hist = refcase.history(r.path("output.h.1"))
        assert len(hist) == nsteps
        vN = refio.read_field(r.last_restart())[1]
        out = dict(v=vN, hist=hist, nbl=P.get("nbl"), alfa=P.get("alfa"))
        if boundary_rows:
            nx, ny = vN.shape[1:]
            v = np.asfortranarray(refio.read_field(os.path.join(ref, "mean.R.0"))[1])
            vm = np.zeros_like(v)
            P.call("itrbc", v, vm)
            out["nbl_bc"] = P.get("nbl")
            dtl = np.zeros((nx, ny), order="F")
            P.call("set_time_step", v, dtl)
            r_ = np.zeros_like(v)
            P.call("genmtrx", v, 0.0, r_)
            P.call("rbe", r_, v, np.asfortranarray(v.copy()), dtl)
            P.call("rhsbc", r_, v, vm)
            out.update(v_bc=v, dtl=dtl, r=r_)
            ops = {k: np.asfortranarray(P.array(k)) for k in ("Ah", "Bh", "Dh", "Vh11", "Vh22")}
            for name, args in (("lhs1f", ("Ah", "Dh", "Vh11")), ("lhs2f", ("Bh", "Dh", "Vh22"))):
                mat = np.zeros((5, 5, 5, nx, ny), order="F")
                P.call(name, mat, *[ops[k] for k in args], dtl, v)
                out[name] = mat[:, :, :, EDGE, :]
            assert P.oob() == 0
        return out
    finally:
        r.close()


def generate():
    ref = os.path.join(CASE_DIR, "ref")
    x, _ = refio.read_grid(os.path.join(ref, "grid.dat"))[:2]
    nx, ny = x.shape
    met = refio.read_metrics(os.path.join(ref, "metric.dat"), nx, ny)
    v0 = refio.read_field(os.path.join(ref, "mean.R.0"))[1]
    one = run(ref, 1)
    last = run(ref, NSTEPS, boundary_rows=True)
    assert one["hist"][0] == last["hist"][0]
    np.savez_compressed(
        os.path.join(HERE, "pcyl_sweep35.npz"),
        nsteps=NSTEPS, deck=deck(NSTEPS), nbl0=32, alfa=one["alfa"],
        v0=v0, top_pot=refio.read_pot(os.path.join(ref, "top.pot")),
        right_pot=refio.read_pot(os.path.join(ref, "right.pot")), cols=np.array(COLS), edge=np.array(EDGE),
        v1=one["v"][:, COLS, :], nbl1=one["nbl"], vN=last["v"][:, COLS, :], hist=last["hist"], nblN=last["nbl"],
        nbl_bc=last["nbl_bc"], v_bc=last["v_bc"][:, COLS, :], dtl=last["dtl"][COLS, :],
        r=last["r"][:, COLS, :], lhs1=last["lhs1f"], lhs2=last["lhs2f"],
        **{"m_" + k: a for k, a in met.items()})


if __name__ == "__main__":
    generate()
    print("wrote pcyl_sweep35")

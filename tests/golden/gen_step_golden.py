"""Generates tests/golden/step*.npz: outputs of the reference's own step
code (the translated reference program, oracle/_ref/libref_step.so) on the
seeded synthetic cases, for the GPU tests, which run where the reference
sources are absent.

Each file holds the final state of the run and the residual history the
reference wrote (one totres per corrector).  The inputs are not stored: the
tests regenerate them from lns3d_gb300.cases with the same arguments.

Run from the repository root:  python tests/golden/gen_step_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import refcase  # noqa: E402
from lns3d_gb300.cases import acoustic_box, shear_layer, vortex2d, vortex2d_open  # noqa: E402

# name -> (kind, case arguments, run arguments)
GOLDEN = {
    # the nonlinear 2D case at its full size: 128 x 128, 100 steps at CFL 1
    "step2d_vortex128": ("2d", dict(nx=128, ny=128, seed=0), dict(nsteps=100, cflmax=1.0, loctime=0)),
    "step2d_vortex_tri": ("2d", dict(nx=48, ny=40, seed=1), dict(nsteps=10, cflmax=1.0, loctime=0, ilhs=0)),
    "step2d_vortex_midpoint": ("2d", dict(nx=48, ny=40, seed=1), dict(nsteps=10, cflmax=1.0, loctime=0, impl=3)),
    # the linearised 3D step on the shear layer: local time step at CFL 20
    "step3d_shear": ("3d", dict(nx=96, ny=64, seed=0), dict(nsteps=30, cflmax=20.0, loctime=1)),
    "step3d_shear_two_step": ("3d", dict(nx=40, ny=33, seed=1), dict(nsteps=10, cflmax=20.0, loctime=1, impl=2)),
    "step3d_shear_midpoint": ("3d", dict(nx=40, ny=33, seed=1), dict(nsteps=10, cflmax=20.0, loctime=1, impl=3)),
    # the reference's test/3d case (test/3d/cfl.inp): an inviscid oblique acoustic
    # wave in a box periodic in both directions, two correctors per step
    "step3d_box": ("3dbox", dict(nx=64, ny=63), dict(nsteps=20, Re=0.0, Pr=1.0, dtmax=0.0070710678e10,
                                                     cflmax=0.1, niter=2, loctime=0, Lz=1.0)),
    # the linear 2D step (src/impdrv.f90 with linear = 1) on the wall-bounded
    # shear layer at beta = omega = 0
    "step2d_lin_shear": ("2dlin", dict(nx=48, ny=33, seed=3, beta=0.0, omega=0.0),
                         dict(nsteps=10, cflmax=20.0, loctime=1)),
    # a non-periodic xi direction: zero-disturbance inflow and outflow planes,
    # and an incoming acoustic wave at the inflow plane.  With the wave the
    # reference's step is ill-conditioned at CFL 20 on this case (one step
    # takes the state from 0.4 to 2e4, and the reference built with FMA
    # contraction differs from itself by 5e-10); at CFL 0.2 that difference
    # is 3e-16 after five steps, which carry the wave into the interior
    "step3d_open": ("3dopen", dict(nx=48, ny=33, seed=4, left=0, right=0), dict(nsteps=10, cflmax=20.0, loctime=1)),
    "step3d_open_wave": ("3dopen", dict(nx=48, ny=33, seed=4, left=1, right=0),
                         dict(nsteps=5, cflmax=0.2, loctime=1, x0=0.5)),
    # the eigenfunction planes (left 4 inflow, right 4 outflow with the
    # inflow namelist's complex lalpha) and the held outflow (right 8)
    "step3d_open_eig": ("3dopen", dict(nx=48, ny=33, seed=5, left=4, right=4, profile_seed=7),
                        dict(nsteps=10, cflmax=20.0, loctime=1, module=dict(lalpha=0.3 + 0.05j))),
    "step3d_open_hold": ("3dopen", dict(nx=48, ny=33, seed=6, left=0, right=8),
                         dict(nsteps=10, cflmax=20.0, loctime=1)),
    # the acoustic planes (left 5 inflow; right 5 outflow, which reads x at
    # the (nx, ny) array's point (j, nx) and so needs ny >= nx), at the
    # incoming wave's CFL 0.2
    "step3d_open_acoustic": ("3dopen", dict(nx=48, ny=33, seed=10, left=5, right=0),
                             dict(nsteps=5, cflmax=0.2, loctime=1)),
    "step3d_open_acoustic_both": ("3dopen", dict(nx=32, ny=40, seed=11, left=5, right=5),
                                  dict(nsteps=5, cflmax=0.2, loctime=1)),
    # symmetry planes (left / right 7): mirrored stencils and xi LHS rows
    "step3d_sym_left": ("3dopen", dict(nx=48, ny=33, seed=7, left=7, right=0),
                        dict(nsteps=10, cflmax=20.0, loctime=1)),
    "step3d_sym_both": ("3dopen", dict(nx=40, ny=33, seed=8, left=7, right=7),
                        dict(nsteps=10, cflmax=20.0, loctime=1)),
    "step3d_sym_smooth": ("3dopen", dict(nx=40, ny=33, seed=9, left=7, right=7),
                          dict(nsteps=10, cflmax=20.0, loctime=1, eps_e=0.01)),
    # the linear 2D step with a non-periodic xi direction: the zero-
    # disturbance planes (left 0, right 0), at CFL 2 (at CFL 20 the reference
    # built with FMA contraction differs from itself by 1.2e-12 after ten
    # steps, at CFL 2 by 5e-15)
    "step2d_lin_open": ("2dlinopen", dict(nx=48, ny=33, seed=12, beta=0.0, omega=0.0, left=0, right=0),
                        dict(nsteps=10, cflmax=2.0, loctime=1)),
    # its symmetry plane (left 7: no mirrored stencils, v = 0 on the plane)
    "step2d_lin_sym": ("2dlinopen", dict(nx=48, ny=33, seed=13, beta=0.0, omega=0.0, left=7, right=0),
                       dict(nsteps=10, cflmax=2.0, loctime=1)),
    # its nonreflecting planes (left 1, right 1) above the &extras nbl, at
    # CFL 0.5 (with the left plane the reference's step grows the state by
    # two orders a step at CFL 2); right 1 also writes column 1's density
    # row, in the second case over a zero-disturbance left plane
    "step2d_lin_nr": ("2dlinopen", dict(nx=48, ny=33, seed=14, beta=0.0, omega=0.0, left=1, right=1),
                      dict(nsteps=10, cflmax=0.5, loctime=1, module=dict(nbl=4))),
    "step2d_lin_nr_right": ("2dlinopen", dict(nx=48, ny=33, seed=15, beta=0.0, omega=0.0, left=0, right=1),
                            dict(nsteps=10, cflmax=2.0, loctime=1)),
    # the nonlinear 2D step with a non-periodic xi direction: Riemann planes
    # on both sides; the symmetry plane on the left with the right plane
    # extrapolated (zeroth order) over a viscous layer that itrBC moves
    # (the &extras namelist's nbl and update_nbl)
    "step2d_vortex_open": ("2dopen", dict(nx=48, ny=40, seed=1, left=0, right=0),
                           dict(nsteps=10, cflmax=1.0, loctime=0)),
    "step2d_vortex_open_sym": ("2dopen", dict(nx=48, ny=40, seed=2, left=2, right=0, extrap=0),
                               dict(nsteps=10, cflmax=1.0, loctime=0, module=dict(nbl=6, update_nbl=1))),
    # mirrored symmetry planes (left / right 7), with the smoother
    "step2d_vortex_mirror": ("2dopen", dict(nx=48, ny=40, seed=3, left=7, right=7),
                             dict(nsteps=10, cflmax=1.0, loctime=0, eps_e=0.01)),
    # the held outflow plane (right 8)
    "step2d_vortex_hold": ("2dopen", dict(nx=48, ny=40, seed=4, left=0, right=8),
                           dict(nsteps=10, cflmax=1.0, loctime=0)),
}


def open_layer(left, right, profile_seed=None, **kw):
    """The shear layer with a non-periodic xi direction (xper = 0); with
    profile_seed, an eigenfunction for the planes left 4 / right 4: each
    variable a seeded complex amplitude of the disturbance's size times a
    Gaussian of the layer's width."""
    case = shear_layer(**kw)
    case["params"].update(xper=0, left=left, right=right)
    if profile_seed is not None:
        rng = np.random.default_rng(profile_seed)
        y = case["y"][0, :]
        amp = 1e-6 * (rng.standard_normal(5) + 1j * rng.standard_normal(5))
        case["profile"] = np.asfortranarray(amp[:, None] * np.exp(-y[None, :] ** 2))
    return case


# the reference's own linear 2D fixture (test/2d: a linear wave on a fluid at
# rest, Euler, periodic in both directions, big-endian SGI files), run as its
# run.sh does: ic.dat copied to output.R.0, lns3d < lns3d.inp with byte swap
TEST2D_DIR = "/root/reference/test/2d"


def generate_test2d():
    import shutil

    from lns3d_gb300 import refio

    r = refcase.Run()
    try:
        for f in ("grid.dat", "metric.dat", "mean.dat"):
            shutil.copy(os.path.join(TEST2D_DIR, f), r.path(f))
        shutil.copy(os.path.join(TEST2D_DIR, "ic.dat"), r.path("output.R.0"))
        deck = open(os.path.join(TEST2D_DIR, "lns3d.inp")).read()
        r.run(deck, swap=True)
        assert r.prog.oob() == 0
        x, y = refio.read_grid(r.path("grid.dat"), endian=">")
        nx, ny = x.shape
        met = refio.read_metrics(r.path("metric.dat"), nx, ny, endian=">")
        _, vm, _ = refio.read_field(r.path("mean.dat"), endian=">")
        _, v0, _ = refio.read_field(r.path("output.R.0"), endian=">")
        outs = {}
        for k in (1, 2, 3):
            h, v, _ = refio.read_field(r.path("output.R.%d" % k), endian=">")
            outs["v_step%d" % h["lstep"]] = v
        np.savez_compressed(os.path.join(HERE, "step2d_test2d.npz"), x=x, y=y, vm=vm, v0=v0,
                            hist=refcase.history(r.path("output.h.1")), deck=deck,
                            **{"m_" + k: a for k, a in met.items()}, **outs)
    finally:
        r.close()


def generate(name):
    if name == "step2d_test2d":
        return generate_test2d()
    kind, cargs, rargs = GOLDEN[name]
    rargs = dict(rargs)
    nsteps = rargs.pop("nsteps")
    if kind == "2d":
        v, hist, run = refcase.run2d(vortex2d(**cargs), nsteps, **rargs)
    elif kind == "3dbox":
        v, hist, run = refcase.run3d(acoustic_box(**cargs), nsteps, **rargs)
    elif kind == "2dlin":
        v, hist, run = refcase.run2dlin(shear_layer(**cargs), nsteps, **rargs)
    elif kind == "3dopen":
        v, hist, run = refcase.run3d(open_layer(**cargs), nsteps, **rargs)
    elif kind == "2dlinopen":
        v, hist, run = refcase.run2dlin(open_layer(**cargs), nsteps, **rargs)
    elif kind == "2dopen":
        v, hist, run = refcase.run2d(vortex2d_open(**cargs), nsteps, **rargs)
    else:
        v, hist, run = refcase.run3d(shear_layer(**cargs), nsteps, **rargs)
    try:
        assert run.prog.oob() == 0
    finally:
        run.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), v=v, hist=hist, nsteps=nsteps)


if __name__ == "__main__":
    for name in (sys.argv[1:] or list(GOLDEN) + ["step2d_test2d"]):
        generate(name)
        print("wrote", name)

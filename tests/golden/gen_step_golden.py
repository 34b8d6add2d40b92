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
from lns3d_gb300.cases import shear_layer, vortex2d  # noqa: E402

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
}


def generate(name):
    kind, cargs, rargs = GOLDEN[name]
    rargs = dict(rargs)
    nsteps = rargs.pop("nsteps")
    if kind == "2d":
        v, hist, run = refcase.run2d(vortex2d(**cargs), nsteps, **rargs)
    else:
        v, hist, run = refcase.run3d(shear_layer(**cargs), nsteps, **rargs)
    try:
        assert run.prog.oob() == 0
    finally:
        run.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), v=v, hist=hist, nsteps=nsteps)


if __name__ == "__main__":
    for name in (sys.argv[1:] or GOLDEN):
        generate(name)
        print("wrote", name)

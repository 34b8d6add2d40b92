"""Runs of the translated reference program (oracle/refstep.py) on the
synthetic cases: the case is written in the reference's file formats
(lns3d_gb300/refio.py) into a run directory with a deck, the reference's
own main program runs there, and its restart and history files are read
back.  Used by the CPU parity tests and by tests/golden/gen_step_golden.py.
"""
import math
import os
import shutil
import tempfile

import numpy as np

from lns3d_gb300 import refio


def deck3d(case, nsteps, cflmax=20.0, dtmax=1e30, loctime=1, impl=1, niter=1, **kw):
    p = case["params"]
    d = dict(Ma=p["Ma"], Re=p["Re"], Pr=p["Pr"], cflmax=cflmax, dtmax=dtmax, nstep=nsteps, xper=bool(p["xper"]),
             yper=bool(p["yper"]), optx=p["optx"], opty=p["opty"], linear=1, impl=impl, iLHS=1, niter=niter,
             loctime=loctime, top=p["top"], wall=p["wall"], left=p.get("left", -1), right=p.get("right", -1),
             wallt=p["wallt"], omega=p["omega"], Lz=span_of_kz(p["kz"]), ires=0, ntout=1000000)
    d.update(kw)
    return refio.write_deck(d)


def span_of_kz(kz):
    return 2.0 * math.pi / kz if kz else 0.0


def deck2d(case, nsteps, cflmax=1.0, dtmax=1e30, loctime=0, impl=1, niter=1, ilhs=1, **kw):
    p = case["params"]
    d = dict(Ma=p["Ma"], Re=p["Re"], Pr=p["Pr"], cflmax=cflmax, dtmax=dtmax, nstep=nsteps, xper=bool(p["xper"]),
             yper=bool(p["yper"]), optx=p["optx"], opty=p["opty"], linear=0, impl=impl, iLHS=ilhs, niter=niter,
             loctime=loctime, top=p["top"], wall=p["wall"], left=-1, right=-1, wallt=p["wallt"], omega=0.0,
             Lz=0.0, theta=case.get("theta", 0.0), ires=0, ntout=1000000)
    d.update(kw)
    return refio.write_deck(d)


def history(path):
    """totres of every resstat call: item 5 of the history lines that
    resstat3D (nine numbers, src/resstat3d.f90:87) and resstat (eleven,
    src/resstat.f90:85) write; the restart notes have two."""
    return np.array([row[4] for row in refio.read_history(path) if len(row) in (9, 11)])


class Run:
    """One run directory; removed by close()."""

    def __init__(self):
        self.dir = tempfile.mkdtemp(prefix="lns3d_ref_")
        self.prog = None

    def close(self):
        if self.prog is not None:
            self.prog.close()
        shutil.rmtree(self.dir, ignore_errors=True)

    def path(self, name):
        return os.path.join(self.dir, name)

    def run(self, deck, swap=False, asis=False, module=None):
        """module: values of module variables to set before the program
        starts (the &extras namelist, which the translated program does not
        read)."""
        from oracle.refstep import RefProgram

        self.prog = RefProgram(asis=asis)
        for k, val in (module or {}).items():
            self.prog.set(k, val)
        self.prog.run(self.dir, deck, swap=swap)
        return self.prog

    def last_restart(self):
        n = 0
        while os.path.exists(self.path("output.R.%d" % (n + 1))):
            n += 1
        return self.path("output.R.%d" % n)


def run3d(case, nsteps, asis=False, module=None, **kw):
    """The reference's ImpDrv3D on the case: (final v, totres history, Run).
    A case with an eigenfunction plane (left 4) carries its profile,
    complex (5, ny), written as inflow.dat (src/gendist.f90:40-47) beside an
    inflow.nml, whose namelist the translated program does not read (its
    lalpha is set through module)."""
    p = case["params"]
    r = Run()
    refio.write_grid(r.path("grid.dat"), case["x"], case["y"])
    refio.write_metrics(r.path("metric.dat"), case["metrics"])
    refio.write_field(r.path("mean.dat"), case["vm"], Re=p["Re"], Ma=p["Ma"], Pr=p["Pr"])
    refio.write_field(r.path("output.R.0"), case["v"], Re=p["Re"], Ma=p["Ma"], Pr=p["Pr"])
    if case.get("profile") is not None:
        with open(r.path("inflow.nml"), "w") as f:
            f.write("&inflow\n/\n")
        with open(r.path("inflow.dat"), "w") as f:
            for j, col in enumerate(np.asarray(case["profile"]).T):
                vals = [float(j + 1)] + [x for z in col for x in (z.real, z.imag)]
                f.write(" ".join("%.17e" % x for x in vals) + "\n")
    r.run(deck3d(case, nsteps, **kw), asis=asis, module=module)
    _, v, _ = refio.read_field(r.last_restart(), complex_=True)
    return v, history(r.path("output.h.1")), r


def run2d(case, nsteps, module=None, **kw):
    """The reference's nonlinear impdrv on the case: (final v, totres history,
    Run).  A case with a non-periodic xi direction carries its deck's left,
    right and extrap, and the far fields of its Riemann planes (left_far,
    right_far: (bn, pot)), written as left.pot / right.pot."""
    p = case["params"]
    r = Run()
    refio.write_grid(r.path("grid.dat"), case["x"], case["y"])
    refio.write_metrics(r.path("metric.dat"), case["metrics"])
    refio.write_field(r.path("output.R.0"), case["v"], Re=p["Re"], Ma=p["Ma"], Pr=p["Pr"])
    refio.write_pot(r.path("top.pot"), np.asarray(case["pot"]).T)
    for name in ("left", "right"):
        if case.get(name + "_far") is not None:
            refio.write_pot(r.path(name + ".pot"), np.asarray(case[name + "_far"][1]).T)
    if not p["xper"]:
        kw = dict(dict(left=p["left"], right=p["right"], extrap=case.get("extrap", -1)), **kw)
    r.run(deck2d(case, nsteps, **kw), module=module)
    _, v, _ = refio.read_field(r.last_restart())
    return v, history(r.path("output.h.1")), r


def run2dlin(case, nsteps, module=None, **kw):
    """The reference's linear impdrv (linear = 1, Lz = 0: src/lrhs.f90) on
    the real part of the case's state: (final v, totres history, Run);
    module: variables of the program's modules set before the run (the
    &extras namelist's nbl)."""
    p = case["params"]
    r = Run()
    refio.write_grid(r.path("grid.dat"), case["x"], case["y"])
    refio.write_metrics(r.path("metric.dat"), case["metrics"])
    refio.write_field(r.path("mean.dat"), case["vm"], Re=p["Re"], Ma=p["Ma"], Pr=p["Pr"])
    refio.write_field(r.path("output.R.0"), np.asfortranarray(np.real(case["v"])), Re=p["Re"], Ma=p["Ma"],
                      Pr=p["Pr"])
    d = dict(omega=0.0, Lz=0.0)
    d.update(kw)
    r.run(deck3d(case, nsteps, **d), module=module)
    _, v, _ = refio.read_field(r.last_restart())
    return v, history(r.path("output.h.1")), r

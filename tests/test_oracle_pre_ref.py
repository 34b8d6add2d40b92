"""The grid metrics of lns3d_gb300.pre against the reference's own
pre-processor (pre/src_ij/pre.f90, translated by oracle/f90sub2c.py into
oracle/_ref/libref_pre.so and run here as ``pre`` on a grid file): bit for bit,
for a Cartesian grid differenced without periodicity (the 2D benchmark case)
and for an O-grid with pre's periodic xi direction.
"""
import os
import shutil
import tempfile

import numpy as np
import pytest

refstep = pytest.importorskip("oracle.refstep")
if not os.path.exists(refstep.LIB_PRE):
    pytest.skip("the translated pre-processor is not built (oracle/_ref/libref_pre.so)", allow_module_level=True)

from lns3d_gb300 import pre, refio  # noqa: E402
from lns3d_gb300.cases import vortex_grid  # noqa: E402


def run_pre(x, y, periodic):
    """pre < answers in a scratch directory: its metric file, read back."""
    d = tempfile.mkdtemp(prefix="lns3d_pre_")
    try:
        refio.write_grid(os.path.join(d, "grid.dat"), x, y)
        prog = refstep.RefProgram(lib=refstep.LIB_PRE)
        # periodicity, grid file (default), metric file (default), body row
        prog.run(d, "%d\n\n\n1\n" % (1 if periodic else 0), program="pre")
        assert prog.oob() == 0 and prog.transposed() == 0
        nx, ny = x.shape
        return refio.read_metrics(os.path.join(d, "metric.new"), nx, ny)
    finally:
        shutil.rmtree(d, ignore_errors=True)


def test_cartesian_grid_metrics_equal_pre():
    x, y = vortex_grid(128, 128)
    want = run_pre(x, y, periodic=False)
    got = pre.metrics(x, y, xper=False)
    for k in refio.METRIC_NAMES:
        assert np.array_equal(got[k], want[k]), k


def test_periodic_ogrid_metrics_equal_pre():
    nx, ny = 65, 33
    th = np.linspace(0.0, 2.0 * np.pi, nx)
    r = 1.0 + 9.0 * np.linspace(0.0, 1.0, ny) ** 1.5
    x = np.asfortranarray(np.cos(th)[:, None] * r[None, :] * (1.0 + 0.1 * np.sin(3.0 * th))[:, None])
    y = np.asfortranarray(np.sin(th)[:, None] * r[None, :])
    x[-1], y[-1] = x[0], y[0]   # the last point repeats the first
    want = run_pre(x, y, periodic=True)
    got = pre.metrics(x, y, xper=True)
    for k in refio.METRIC_NAMES:
        assert np.array_equal(got[k], want[k]), k


def test_linear_coordinates_have_exact_metrics():
    """pre's closures are exact for linear coordinates: a uniform grid has
    constant first metrics and zero second metrics."""
    x, y = np.meshgrid(np.linspace(-2.0, 3.0, 17), np.linspace(0.0, 4.0, 11), indexing="ij")
    m = pre.metrics(np.asfortranarray(x), np.asfortranarray(y))
    assert np.allclose(m["m1"], 1.0 / 5.0, rtol=1e-14) and np.allclose(m["n2"], 1.0 / 4.0, rtol=1e-14)
    for k in ("m2", "n1", "m11", "m12", "m22", "n11", "n12", "n22"):
        assert np.abs(m[k]).max() < 1e-12, k

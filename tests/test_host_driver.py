"""The host program lns3d_gpu (lns3d_gb300/csrc/host/lns3d_gpu.cpp): the
reference's implicit run over the C ABI, reading the reference's deck and
files and writing its restart and history files.

CPU: the deck is read as src/input.f90 reads it (compared with
lns3d_gb300.refio.parse_deck, and with the derived values of the
reference: Re = 0 gives an inviscid run with Re = 1e99, kz = 2 pi / Lz, the
periodic directions' boundary codes reset to -1).
GPU: the reference's own test/2d case (its files, big-endian, and its deck)
run by lns3d_gpu reproduces the restart files the reference wrote."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from lns3d_gb300 import _build, refio

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DRIVER = os.path.join(_build.LIBDIR, _build.DRIVER_NAME)

needs_driver = pytest.mark.skipif(not os.path.exists(DRIVER), reason="lns3d_gpu is not built")


def echo(deck):
    out = subprocess.run([DRIVER, "--echo-deck"], input=deck, capture_output=True, text=True, check=True).stdout
    vals = {}
    for line in out.splitlines():
        k, v = line.split()
        vals[k] = float(v)
    return vals


@needs_driver
@pytest.mark.parametrize("deck_kw", [
    dict(),
    dict(Re=0.0, xper=True, yper=True, top=0, wall=1, wallt=1, Lz=1.0),
    dict(linear=1, Lz=31.41592653589793, omega=0.05, impl=2, niter=3, loctime=1),
    dict(ispg=1, As=1.0, Ns=3, xs=0.7, xt=1.0, eps_e=0.01, ibuff=1),
])
def test_deck_is_read_as_the_reference_reads_it(deck_kw):
    text = refio.write_deck(deck_kw)
    want = refio.parse_deck(text)
    got = echo(text)
    for k, v in want.items():
        if k == "Re" and v == 0.0:
            assert got["Re"] == 1e99 and got["navier"] == 0      # src/input.f90:40-44
        elif k in ("left", "right") and want["xper"]:
            assert got[k] == -1                                   # src/input.f90:115-120
        elif k in ("wall", "wallt", "top") and want["yper"]:
            assert got[k] == -1                                   # src/input.f90:122-128
        else:
            assert got[k] == float(v), k
    assert got["kz"] == (2.0 * np.pi / want["Lz"] if want["Lz"] else 0.0)


@needs_driver
def test_reference_test2d_deck_is_read():
    d = np.load(os.path.join(GOLDEN, "step2d_test2d.npz"))
    deck = str(d["deck"])
    got = echo(deck)
    want = refio.parse_deck(deck)
    assert got["nstep"] == want["nstep"] == 10 and got["linear"] == 1 and got["navier"] == 0


@pytest.mark.gpu
@needs_driver
def test_driver_runs_the_reference_test2d_case(cuda):
    d = np.load(os.path.join(GOLDEN, "step2d_test2d.npz"))
    run = tempfile.mkdtemp(prefix="lns3d_gpu_")
    try:
        refio.write_grid(os.path.join(run, "grid.dat"), d["x"], d["y"], endian=">")
        refio.write_metrics(os.path.join(run, "metric.dat"), {k[2:]: d[k] for k in d.files if k.startswith("m_")},
                            endian=">")
        refio.write_field(os.path.join(run, "mean.dat"), d["vm"], Ma=1.0, Pr=1.0, endian=">")
        refio.write_field(os.path.join(run, "output.R.0"), d["v0"], Ma=1.0, Pr=1.0, endian=">")
        env = dict(os.environ, GFORTRAN_CONVERT_UNIT="swap")
        subprocess.run([DRIVER], input=str(d["deck"]), cwd=run, env=env, check=True, capture_output=True, text=True)
        for k, step in ((1, 4), (2, 8), (3, 10)):
            h, v, _ = refio.read_field(os.path.join(run, "output.R.%d" % k), endian=">")
            assert h["lstep"] == step
            want = d["v_step%d" % step]
            assert np.abs(v - want).max() / np.abs(want).max() < 1e-12, step
        hist = np.array(refio.read_history(os.path.join(run, "output.h.1")))
        want = d["hist"][0::2]     # ires = 1: the reference also writes the residual after each update
        assert np.abs(hist[:, 4] - want).max() <= 1e-10 * want.max()
    finally:
        shutil.rmtree(run, ignore_errors=True)

"""The step goldens on the CPU: every case of tests/golden/gen_step_golden.py
has its committed fixture, the fixture's shapes agree with the seeded case
the GPU test rebuilds, its residual history has the case's step count, and
a GPU test names the case."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)

import gen_step_golden  # noqa: E402

GPU_TESTS = "".join(open(os.path.join(HERE, f)).read() for f in sorted(os.listdir(HERE))
                    if f.startswith("test_gpu") and f.endswith(".py"))


def build_case(kind, cargs):
    from lns3d_gb300.cases import shear_layer, vortex2d, vortex2d_open

    if kind == "2d":
        return vortex2d(**cargs)
    if kind == "3dbox":
        return gen_step_golden.acoustic_box(**cargs)
    if kind in ("3dopen", "2dlinopen"):
        return gen_step_golden.open_layer(**cargs)
    if kind == "2dopen":
        return vortex2d_open(**cargs)
    return shear_layer(**cargs)


@pytest.mark.parametrize("name", sorted(gen_step_golden.GOLDEN))
def test_fixture_matches_its_case(name):
    kind, cargs, rargs = gen_step_golden.GOLDEN[name]
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    case = build_case(kind, cargs)
    p = case["params"]
    assert d["v"].shape == (5, p["nx"], p["ny"])
    assert int(d["nsteps"]) == rargs["nsteps"]
    # one residual per step or per corrector, and with ires = 1 also one after each update
    n, k = rargs["nsteps"], rargs.get("niter", 1)
    assert len(d["hist"]) in (n, n * k, n * (k + 1))
    assert np.isfinite(d["v"]).all() and np.isfinite(d["hist"]).all()
    if "left" in cargs:
        assert p["xper"] == 0 and p["left"] == cargs["left"] and p["right"] == cargs["right"]


@pytest.mark.parametrize("name", sorted(gen_step_golden.GOLDEN))
def test_fixture_has_a_gpu_test(name):
    assert '"%s"' % name in GPU_TESTS, name

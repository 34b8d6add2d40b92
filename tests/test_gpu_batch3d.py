"""GPU tests of batched linearised problems (lns_batch3d_*, through the C
ABI): every problem of a batch -- different grid sizes, beta and omega --
must end with exactly the state and residuals of its own lns_ctx3d run (the
same kernels on the same data: the context's periodic lines row by row, as
a batch's), alone or in the mix; convergence steps and the autotuner must
leave results unchanged."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def problems():
    from lns3d_gb300.cases import shear_layer

    out = []
    for k, (nx, ny, beta, omega) in enumerate([(40, 33, 0.0, 0.02), (64, 24, 0.2, 0.05), (32, 40, 0.4, 0.1),
                                               (48, 48, 0.1, 0.07)]):
        c = shear_layer(nx=nx, ny=ny, beta=beta, omega=omega, seed=k)
        out.append(c)
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_matches_individual_runs(cuda, precision):
    from lns3d_gb300 import Batch3D, ImpDrv3D

    probs = problems()
    batch = Batch3D(probs, cflmax=20.0, loctime=1, precision=precision)
    steps, res = batch.run(max_steps=12, tol=0.0, check_every=5)
    assert (steps == -1).all()
    for k, c in enumerate(probs):
        drv = ImpDrv3D(c["params"], c["metrics"], c["vm"], cflmax=20.0, loctime=1, precision=precision,
                       row_pairs=False)
        v = c["v"].copy(order="F")
        r = drv.step(v, nsteps=12)
        assert np.array_equal(batch.state(k), v), k
        assert res[k] == r[-1], k


def test_batch_convergence_steps_match_residual_history(cuda):
    from lns3d_gb300 import Batch3D, ImpDrv3D

    probs = problems()[:3]
    tol = 1e-8
    batch = Batch3D(probs, cflmax=20.0, loctime=1, precision=1)
    steps, res = batch.run(max_steps=800, tol=tol, check_every=20)
    for k, c in enumerate(probs):
        drv = ImpDrv3D(c["params"], c["metrics"], c["vm"], cflmax=20.0, loctime=1, precision=1)
        v = c["v"].copy(order="F")
        hist = drv.step(v, nsteps=800)
        below = np.nonzero(hist <= tol)[0]
        want = int(below[0]) + 1 if below.size else -1
        assert steps[k] == want, (k, steps[k], want)


def test_tune_keeps_states_and_results(cuda):
    from lns3d_gb300 import Batch3D

    probs = problems()
    a = Batch3D(probs, cflmax=20.0, loctime=1, precision=0)
    b = Batch3D(probs, cflmax=20.0, loctime=1, precision=0)
    before = [b.state(k) for k in range(len(probs))]
    w = b.tune()
    assert w in (1, 2, 4)
    assert all(np.array_equal(b.state(k), before[k]) for k in range(len(probs)))
    a.run(max_steps=6)
    b.run(max_steps=6)
    assert all(np.array_equal(a.state(k), b.state(k)) for k in range(len(probs)))


def test_result_is_the_same_alone_and_in_the_mix(cuda):
    from lns3d_gb300 import Batch3D

    probs = problems()
    mix = Batch3D(probs, cflmax=20.0, loctime=1, precision=1)
    alone = Batch3D([probs[2]], cflmax=20.0, loctime=1, precision=1)
    mix.run(max_steps=10)
    alone.run(max_steps=10)
    assert np.array_equal(mix.state(2), alone.state(0))

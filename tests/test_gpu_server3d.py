"""GPU tests of the serving layer (lns_server3d_*, through the C ABI):
requests admitted into a running batch give the same result alone and in
the mix, stop at the step their residual met the tolerance, and wait for
device memory when the budget is full."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-8


def case(nx, ny, beta, omega, seed):
    from lns3d_gb300.cases import shear_layer

    return shear_layer(nx=nx, ny=ny, beta=beta, omega=omega, seed=seed)


def drain(srv, ids, nsteps=20, max_ticks=400):
    for _ in range(max_ticks):
        if all(srv.poll(i)["state"] in ("done", "stopped", "failed") for i in ids):
            return
        srv.tick(nsteps)
    raise AssertionError("requests did not finish")


def test_result_is_the_same_alone_and_in_the_mix(cuda):
    from lns3d_gb300 import Server3D

    x = case(40, 33, 0.3, 0.04, 11)
    others = [case(48, 24, 0.1, 0.02, 1), case(32, 40, 0.2, 0.08, 2), case(56, 32, 0.0, 0.05, 3)]
    alone = Server3D(1 << 33, max_slots=8)
    ia = alone.submit(x, tol=TOL, max_steps=1500, cflmax=20.0)
    drain(alone, [ia], nsteps=7)
    mix = Server3D(1 << 33, max_slots=8)
    ids = [mix.submit(o, tol=TOL, max_steps=1500, cflmax=20.0) for o in others]
    mix.tick(13)                   # x arrives while the others are running
    ix = mix.submit(x, tol=TOL, max_steps=1500, cflmax=20.0)
    drain(mix, ids + [ix], nsteps=11)
    pa, pm = alone.poll(ia), mix.poll(ix)
    assert pa["state"] == pm["state"] == "done"
    assert pa["steps"] == pm["steps"]
    assert np.array_equal(alone.fetch(ia), mix.fetch(ix))


def test_request_stops_at_the_converged_step(cuda):
    from lns3d_gb300 import ImpDrv3D, Server3D

    x = case(40, 33, 0.3, 0.04, 11)
    srv = Server3D(1 << 33, max_slots=4)
    i = srv.submit(x, tol=TOL, max_steps=1500, cflmax=20.0)
    drain(srv, [i], nsteps=9)
    p = srv.poll(i)
    drv = ImpDrv3D(x["params"], x["metrics"], x["vm"], cflmax=20.0, loctime=1, precision=1)
    v = x["v"].copy(order="F")
    hist = drv.step(v, nsteps=p["steps"] - 1)
    assert hist.max() > TOL or p["steps"] == 1
    # the served state is the one whose residual met the tolerance: the
    # state after steps - 1 steps
    assert np.array_equal(srv.fetch(i), v)


def test_admission_waits_for_memory(cuda):
    from lns3d_gb300 import Server3D

    probs = [case(48, 40, 0.1 * k, 0.05, k) for k in range(4)]
    probe = Server3D(1 << 34, max_slots=1)
    probe.submit(probs[0], tol=TOL, max_steps=5, cflmax=20.0)
    probe.tick(1)
    one = probe.bytes_in_use
    srv = Server3D(int(2.5 * one), max_slots=8)
    ids = [srv.submit(p, tol=TOL, max_steps=30, cflmax=20.0) for p in probs]
    running, queued = srv.tick(5)
    assert running == 2 and queued == 2
    assert srv.bytes_in_use <= 2.5 * one
    drain(srv, ids, nsteps=10)
    assert all(srv.poll(i)["state"] == "stopped" for i in ids)


def test_request_stops_exactly_at_max_steps(cuda):
    """A step limit that is not a multiple of the tick length: the tick is cut
    so that the request runs exactly max_steps steps, and the fetched state
    is that of a lone run of max_steps steps."""
    from lns3d_gb300 import ImpDrv3D, Server3D

    x = case(40, 33, 0.3, 0.04, 11)
    other = case(48, 24, 0.1, 0.02, 1)
    srv = Server3D(1 << 33, max_slots=4)
    i = srv.submit(x, tol=1e-30, max_steps=17, cflmax=20.0)
    j = srv.submit(other, tol=1e-30, max_steps=40, cflmax=20.0)
    drain(srv, [i, j], nsteps=10)
    p = srv.poll(i)
    assert p["state"] == "stopped" and p["steps"] == 17
    drv = ImpDrv3D(x["params"], x["metrics"], x["vm"], cflmax=20.0, loctime=1, precision=1)
    v = x["v"].copy(order="F")
    hist = drv.step(v, nsteps=17)
    assert np.array_equal(srv.fetch(i), v)
    assert p["res"] == hist[-1]
    assert srv.poll(j)["steps"] == 40


def test_joins_and_leaves_keep_the_captured_step(cuda):
    """Eight same-size requests through four slots, leaving at different
    steps: the ones queued join as slots free up, which rewrites the work
    tables in place, so the step is captured once; each result equals a
    lone run of the same request."""
    from lns3d_gb300 import ImpDrv3D, Server3D

    reqs = [case(40, 33, 0.05 * k, 0.02 + 0.01 * k, 20 + k) for k in range(8)]
    limits = [12, 30, 18, 42, 24, 36, 6, 48]
    srv = Server3D(1 << 33, max_slots=4)
    ids = [srv.submit(c, tol=1e-30, max_steps=m, cflmax=20.0) for c, m in zip(reqs, limits)]
    drain(srv, ids, nsteps=6)
    assert srv.graph_captures == 1
    for k in (0, 3, 7):
        assert srv.poll(ids[k])["state"] == "stopped"
        c = reqs[k]
        drv = ImpDrv3D(c["params"], c["metrics"], c["vm"], cflmax=20.0, loctime=1, precision=1)
        v = c["v"].copy(order="F")
        drv.step(v, nsteps=limits[k])
        assert np.array_equal(srv.fetch(ids[k]), v), k

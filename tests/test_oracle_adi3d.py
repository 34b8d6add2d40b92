"""CPU known-answer tests of the 3D-step oracle (oracle/adi3d_oracle.c).

The reference's tests hold no routine-level vectors for these routines, so
the restatement is checked against properties its algorithm must have:
  * the fourth-order stencils and their closures (src/stencil.f90) are exact
    on polynomials: interior and boundary first derivatives to degree 4,
    second derivatives to degree 3 at the closures and degree 5 in the
    interior;
  * the periodic stencils are exact on the periodic grid's Fourier modes to
    their design order;
  * the step is linear in the disturbance (impdrv3d with impl 1);
  * the steady disturbance v = 0 is a fixed point with zero residual.
"""
import ctypes

import numpy as np
import pytest

from adi3dcase import A3Grid, Oracle3D, _lib, ptr


def grid(nx, ny, xper=0, yper=0, opt=-1):
    g = A3Grid(nx=nx, ny=ny, dxi=1.0 / (nx - 1), deta=1.0 / (ny - 1), xper=xper, yper=yper, optx=opt, opty=opt)
    return g


def derivs(g, f):
    L = _lib()
    nx, ny = g.nx, g.ny
    v = np.asfortranarray(f.reshape(1, nx, ny))
    out = {k: np.zeros((1, nx, ny), order="F") for k in ("g1", "g2", "g11", "g12", "g22")}
    assert L.a3_deriv1(ctypes.byref(g), 1, ptr(v), ptr(out["g1"]), ptr(out["g2"])) == 0
    assert L.a3_deriv2(ctypes.byref(g), 1, ptr(v), ptr(out["g1"]), ptr(out["g11"]), ptr(out["g12"]),
                       ptr(out["g22"])) == 0
    return {k: a[0] for k, a in out.items()}


@pytest.mark.parametrize("deg", [0, 1, 2, 3, 4])
def test_first_derivative_exact_on_polynomials(deg):
    nx, ny = 21, 17
    g = grid(nx, ny)
    xi = np.linspace(0, 1, nx)[:, None] * np.ones((1, ny))
    eta = np.ones((nx, 1)) * np.linspace(0, 1, ny)[None, :]
    d = derivs(g, np.asfortranarray(xi ** deg + 2.0 * eta ** deg))
    want1 = deg * xi ** max(deg - 1, 0) if deg else 0 * xi
    want2 = 2.0 * deg * eta ** max(deg - 1, 0) if deg else 0 * eta
    assert np.abs(d["g1"] - want1).max() < 1e-9
    assert np.abs(d["g2"] - want2).max() < 1e-9


@pytest.mark.parametrize("deg", [0, 1, 2, 3])
def test_second_derivatives_exact_on_polynomials(deg):
    nx, ny = 21, 17
    g = grid(nx, ny)
    xi = np.linspace(0, 1, nx)[:, None] * np.ones((1, ny))
    eta = np.ones((nx, 1)) * np.linspace(0, 1, ny)[None, :]
    f = np.asfortranarray(xi ** deg + eta ** deg + xi * eta ** max(deg - 1, 0))
    d = derivs(g, f)
    w11 = deg * (deg - 1) * xi ** max(deg - 2, 0) if deg >= 2 else 0 * xi
    w22 = deg * (deg - 1) * eta ** max(deg - 2, 0) if deg >= 2 else 0 * eta
    if deg - 1 >= 2:
        w22 = w22 + xi * (deg - 1) * (deg - 2) * eta ** (deg - 3)
    w12 = (deg - 1) * eta ** max(deg - 2, 0) if deg >= 2 else (0 * eta if deg == 0 else 0 * eta)
    if deg == 1:
        w12 = 0 * eta  # xi * eta**0 = xi
    assert np.abs(d["g11"] - w11).max() < 1e-7
    assert np.abs(d["g22"] - w22).max() < 1e-7
    assert np.abs(d["g12"] - w12).max() < 1e-7


def test_interior_second_derivative_degree_five():
    nx, ny = 21, 9
    g = grid(nx, ny)
    xi = np.linspace(0, 1, nx)[:, None] * np.ones((1, ny))
    d = derivs(g, np.asfortranarray(xi ** 5))
    want = 20 * xi ** 3
    assert np.abs(d["g11"][3:-3] - want[3:-3]).max() < 1e-8


@pytest.mark.parametrize("opt", [-1, 0, 1])
def test_periodic_derivatives_of_fourier_modes(opt):
    # point nx repeats point 1; a low mode is resolved to the stencil's order
    nx, ny = 129, 9
    g = grid(nx, ny, xper=1, opt=opt)
    xi = np.linspace(0, 1, nx)[:, None] * np.ones((1, ny))
    k = 2 * np.pi
    d = derivs(g, np.asfortranarray(np.sin(k * xi)))
    assert np.abs(d["g1"] - k * np.cos(k * xi)).max() < 2e-5 * k
    assert np.abs(d["g11"] + k * k * np.sin(k * xi)).max() < 2e-5 * k * k
    # the repeated point carries the value of point 1
    assert np.array_equal(d["g1"][-1], d["g1"][0])


def test_step_is_linear_in_the_disturbance():
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=24, ny=16, seed=4)
    o = Oracle3D(case, cflmax=20.0, loctime=1)
    rng = np.random.default_rng(1)
    shape = case["v"].shape
    a = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    b = np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    c = np.asfortranarray(2.0 * a - 3.0 * b)
    for v in (a, b, c):
        o.step(v, niter=2)
    assert np.abs(c - (2.0 * a - 3.0 * b)).max() < 1e-12 * np.abs(c).max()


def test_zero_disturbance_is_a_fixed_point():
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=24, ny=16)
    o = Oracle3D(case, cflmax=20.0, loctime=1)
    v = np.zeros_like(case["v"], order="F")
    res = o.step(v, niter=2)
    assert res == 0.0 and not v.any()


def test_time_scheme_steps_are_consistent():
    """The oracle's scheme step: impl 1 equals the backward Euler step bit for
    bit; impl 2's first step (lstep = 0) is backward Euler; the midpoint step
    keeps the zero state at zero (src/impdrv3d.f90:130-199)."""
    import numpy as np

    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=24, ny=20, seed=4)
    a, b, c = (Oracle3D(case, cflmax=20.0, loctime=1) for _ in range(3))
    va, vb, vc = (case["v"].copy(order="F") for _ in range(3))
    ra = a.step(va)
    rb = b.step_impl(vb, 1)
    rc = c.step_impl(vc, 2)
    assert np.array_equal(va, vb) and ra == rb
    assert np.array_equal(va, vc) and ra == rc
    z = Oracle3D(case, cflmax=20.0, loctime=1)
    v0 = np.zeros_like(case["v"], order="F")
    z.step_impl(v0, 3)
    assert np.abs(v0).max() == 0.0


@pytest.mark.parametrize("ispg", [1, 5])
def test_sponge_terms_known_answer(ispg):
    """The sponge (src/lrhs3d.f90:220-240; eta LHS src/lhs2f3d.f90:207-224
    and src/lhsbt2f3d.f90:147-167): the RHS gains sp v and the eta LHS
    alfa dtl sp on the diagonal of every row the boundary conditions leave,
    sp = spg (ispg 1) or spg + spg2 (ispg > 4); the xi LHS is unchanged."""
    from adi3dcase import sponge
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=24, ny=20, seed=1)
    spg, spg2 = sponge(24, 20)
    plain = Oracle3D(case, cflmax=20.0, loctime=1)
    o = Oracle3D(case, cflmax=20.0, loctime=1, ispg=ispg, spg=spg, spg2=spg2)
    sp = spg if ispg == 1 else spg + spg2
    rng = np.random.default_rng(2)
    v = np.asfortranarray(rng.standard_normal((5, 24, 20)) + 1j * rng.standard_normal((5, 24, 20)))
    assert np.array_equal(o.lrhs(v), plain.lrhs(v) + sp[None] * v)
    assert np.array_equal(o.lhs(1), plain.lhs(1))
    m_s, m_p = o.lhs(2), plain.lhs(2)
    d = m_s - m_p
    want = case["params"]["alfa"] * o.dtl * sp
    for a in range(5):
        # rows 2..ny-1 keep every block row; the wall row keeps its continuity
        # row only when wall = 2 (the case's wall 1 replaces it)
        # (m + x) - m recovers x to the rounding of m's scale
        tol = 4e-16 * (np.abs(m_p[2, a, a, :, 1:-1]) + np.abs(want[:, 1:-1]))
        assert (np.abs(d[2, a, a, :, 1:-1] - want[:, 1:-1]) <= tol).all()
    mask = np.ones(d.shape, bool)
    for a in range(5):
        mask[2, a, a, :, 1:-1] = False
    assert not d[mask].any()


def test_sponge_damps_the_perturbation():
    from adi3dcase import sponge
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=24, ny=20, seed=4)
    spg, spg2 = sponge(24, 20, amp=2.0)
    norms = []
    for kw in ({}, dict(ispg=1, spg=spg, spg2=spg2), dict(ispg=5, spg=spg, spg2=spg2)):
        o = Oracle3D(case, cflmax=20.0, loctime=1, **kw)
        v = case["v"].copy(order="F")
        for _ in range(6):
            o.step(v)
        assert np.isfinite(v).all()
        norms.append(np.linalg.norm(v[:, :, 12:]))
    assert norms[1] < norms[0] and norms[2] < norms[0]


def test_smoother_and_damping_known_answer():
    """The explicit smoother (src/smoother3d.f90, added at the end of
    lrhs3D) and the implicit damping of the LHS (src/lhs1f3d.f90:168-200,
    src/lhs2f3d.f90:171-203, src/lhsbt2f3d.f90:277-298): an impulse at an
    interior point spreads with the sixth-order coefficients fa1..fa7 along
    both directions, scaled by eps_e buff; the LHS gains alfa dtl eps_e buff
    times fb1..fb5 on the diagonals of the band, and (-1, 2, -1) in slots 2..4
    of the eta rows 2 and ny-1."""
    from lns3d_gb300.cases import shear_layer

    nx, ny = 24, 20
    case = shear_layer(nx=nx, ny=ny, seed=1)
    rng = np.random.default_rng(5)
    buff = np.asfortranarray(0.5 + rng.uniform(size=(nx, ny)))
    eps = 0.02
    plain = Oracle3D(case, cflmax=20.0, loctime=1)
    o = Oracle3D(case, cflmax=20.0, loctime=1, eps_e=eps, buff=buff)
    v = np.zeros((5, nx, ny), np.complex128, order="F")
    i0, j0 = 10, 9          # 0-based interior point
    v[2, i0, j0] = 1.0 + 2.0j
    d = o.lrhs(v) - plain.lrhs(v)
    fa = [-1.666666666666667E-01, 2.0, -6.5, 9.333333333333333, -6.5, 2.0, -1.666666666666667E-01]
    want = np.zeros_like(d)
    for s in range(-3, 4):
        want[2, i0, j0 - s] += eps * buff[i0, j0 - s] * fa[3 + s] * v[2, i0, j0]
        want[2, i0 - s, j0] += eps * buff[i0 - s, j0] * fa[3 + s] * v[2, i0, j0]
    scale = np.abs(plain.lrhs(v)).max()
    assert np.abs(d - want).max() <= 1e-15 * scale
    assert not d[[0, 1, 3, 4]].any()
    alfa = case["params"]["alfa"]
    fb = [1.0, -4.0, 6.0, -4.0, 1.0]
    w = alfa * o.dtl * eps * buff
    for direction in (1, 2):
        dm = o.lhs(direction) - plain.lhs(direction)
        scale = np.abs(plain.lhs(direction)).max()
        rows = range(1, ny - 1) if direction == 1 else range(2, ny - 2)
        for k in range(5):
            for a in range(5):
                got = dm[k, a, a][:, list(rows)]
                assert np.abs(got - w[:, list(rows)] * fb[k]).max() <= 4e-16 * scale
        if direction == 2:
            for jj in (1, ny - 2):
                for k, c in ((1, -1.0), (2, 2.0), (3, -1.0)):
                    for a in range(5):
                        assert np.abs(dm[k, a, a, :, jj] - w[:, jj] * c).max() <= 4e-16 * scale
                assert not dm[0, :, :, :, jj].any() and not dm[4, :, :, :, jj].any()
            assert not dm[:, :, :, :, 0].any() and not dm[:, :, :, :, ny - 1].any()
        off = dm.copy()
        for a in range(5):
            off[:, a, a] = 0.0
        assert not off.any()


def test_smoother_keeps_steps_stable():
    from lns3d_gb300.cases import shear_layer

    case = shear_layer(nx=24, ny=20, seed=4)
    o = Oracle3D(case, cflmax=20.0, loctime=1, eps_e=0.01)
    v = case["v"].copy(order="F")
    res = [o.step(v) for _ in range(6)]
    assert np.isfinite(v).all() and all(np.isfinite(res))


@pytest.mark.parametrize("ispg", [2, 3, 4])
def test_target_sponges_known_answer(ispg):
    """The inflow sponges (ispg 2, 3; src/lrhs3d.f90:242-280): r += spg v +
    spg2 (v - t) with t the decaying wave c3 = [wamp] exp(-a (x - x0))
    exp(i kk x) mapped to (rho, u, v, w, T); the eigenfunction sponge (ispg 4,
    src/sponge.f90:596-604): r += (spg + spg2)(v - cvic).  The eta LHS gains
    alfa dtl (spg + spg2) on its diagonal for all three."""
    from adi3dcase import sponge
    from lns3d_gb300.cases import shear_layer

    nx, ny = 24, 20
    case = shear_layer(nx=nx, ny=ny, seed=1)
    spg, spg2 = sponge(nx, ny)
    rng = np.random.default_rng(9)
    wamp = rng.uniform(0.5, 1.5, nx)
    cvic = np.asfortranarray(rng.standard_normal((5, nx, ny)) + 1j * rng.standard_normal((5, nx, ny)))
    plain = Oracle3D(case, cflmax=20.0, loctime=1)
    o = Oracle3D(case, cflmax=20.0, loctime=1, ispg=ispg, spg=spg, spg2=spg2, x0=-1.0, wamp=wamp, cvic=cvic)
    v = np.asfortranarray(rng.standard_normal((5, nx, ny)) + 1j * rng.standard_normal((5, nx, ny)))
    if ispg == 4:
        want = plain.lrhs(v) + (spg + spg2)[None] * (v - cvic)
    else:
        p = case["params"]
        vm, x = case["vm"], case["x"]
        cm = np.sqrt(vm[4]) / p["Ma"]
        um = vm[1]
        d = 0.5 * (1.3333333333333333333 + p["gamma1"] / p["Pr"]) / p["Re"]
        kk = p["omega"] / (cm + um)
        a = p["omega"] ** 2 * d / (cm + um) ** 3
        c3 = np.exp(-a * (x + 1.0)) * np.exp(1j * kk * x)
        if ispg == 3:
            c3 = wamp[:, None] * c3
        t = np.zeros_like(v)
        t[0] = 0.5 * c3 / cm ** 2
        t[1] = c3 * 0.5 / (vm[0] * cm)
        t[4] = (p["gamma"] * p["Ma"] ** 2 * c3 * 0.5 - vm[4] * 0.5 * c3 / cm ** 2) / vm[0]
        want = (plain.lrhs(v) + spg[None] * v) + spg2[None] * (v - t)
    got = o.lrhs(v)
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
    dm = o.lhs(2) - plain.lhs(2)
    w = case["params"]["alfa"] * o.dtl * (spg + spg2)
    for a_ in range(5):
        assert np.abs(dm[2, a_, a_, :, 1:-1] - w[:, 1:-1]).max() <= 4e-16 * np.abs(plain.lhs(2)).max()
    assert np.array_equal(o.lhs(1), plain.lhs(1))


def _wave(case, x0, wamp, j):
    """The reference's forced wave at row j (src/itrbc3d.f90:166-196)."""
    p = case["params"]
    vm, x = case["vm"][:, :, j], case["x"][:, j]
    cm = np.sqrt(vm[4]) / p["Ma"]
    um = vm[1]
    d = 0.5 * (1.3333333333333333333 + p["gamma1"] / p["Pr"]) / p["Re"]
    kk = p["omega"] / (cm + um)
    a = p["omega"] ** 2 * d / (cm + um) ** 3
    c3 = wamp * np.exp(-a * (x - x0)) * np.exp(1j * kk * x)
    t = np.zeros((5, len(x)), np.complex128)
    t[0] = 0.5 * c3 / cm ** 2
    t[1] = c3 * 0.5 / (vm[0] * cm)
    t[4] = (p["gamma"] * p["Ma"] ** 2 * c3 * 0.5 - vm[4] * 0.5 * c3 / cm ** 2) / vm[0]
    return t


def test_forced_top_boundary_known_answer():
    """top = 1 (src/itrbc3d.f90:145-196, src/rhsbc3d.f90:129-160): itrBC3D
    puts the incoming acoustic wave on row ny, rhsBC3D sets r = -(v - t)
    there, and the LHS row is the identity; steps keep the wave on the top
    row."""
    from lns3d_gb300.cases import shear_layer

    nx, ny = 24, 20
    case = shear_layer(nx=nx, ny=ny, seed=1)
    case = dict(case, params=dict(case["params"], top=1))
    rng = np.random.default_rng(3)
    wamp = rng.uniform(0.5, 1.5, nx)
    o = Oracle3D(case, cflmax=20.0, loctime=1, x0=-2.0, wamp=wamp)
    t = _wave(case, -2.0, wamp, ny - 1)
    v = np.asfortranarray(rng.standard_normal((5, nx, ny)) + 1j * rng.standard_normal((5, nx, ny)))
    w = v.copy(order="F")
    L = _lib()
    L.a3_itrbc(ctypes.byref(o.g), ptr(w))
    assert np.abs(w[:, :-1, -1] - t[:, :-1]).max() <= 1e-13 * np.abs(t).max()
    assert np.array_equal(w[:, -1, :], w[:, 0, :])
    r = np.asfortranarray(rng.standard_normal((5, nx, ny)) + 0j)
    L.a3_rhsbc(ctypes.byref(o.g), ptr(r), ptr(v))
    assert np.abs(r[:, :-1, -1] + (v[:, :-1, -1] - t[:, :-1])).max() <= 1e-13 * np.abs(t).max()
    m = o.lhs(2)
    eye = np.zeros((5, 5, 5), np.complex128)
    eye[2] = np.eye(5)
    assert all(np.array_equal(m[:, :, :, i, -1], eye) for i in range(nx))
    v = case["v"].copy(order="F")
    for _ in range(3):
        o.step(v)
    assert np.isfinite(v).all()
    assert np.abs(v[:, :-1, -1] - t[:, :-1]).max() <= 1e-13 * np.abs(t).max()


@pytest.mark.parametrize("wallt", [0, 1])
def test_bump_wall_known_answer(wallt):
    """wall = 3, the bump (src/itrbc3d.f90:46-121, src/rhsbc3d.f90:45-104,
    src/lhsbc2f3d.f90:41-48): itrBC3D puts the bump's velocities u1w..u3w on
    the wall, rho by third-order extrapolation, T = tw (isothermal) or from
    the gc closure set to twp (adiabatic); rhsBC3D gives the matching
    residual rows; the continuity row of the eta LHS is (-1, 4, -6, 4, -1)."""
    from lns3d_gb300.cases import shear_layer

    nx, ny = 24, 20
    case = shear_layer(nx=nx, ny=ny, seed=1)
    case = dict(case, params=dict(case["params"], wall=3, wallt=wallt))
    rng = np.random.default_rng(6)
    bump = 1e-3 * (rng.standard_normal((5, nx)) + 1j * rng.standard_normal((5, nx)))
    o = Oracle3D(case, cflmax=20.0, loctime=1, bump=bump)
    L = _lib()
    v = np.asfortranarray(rng.standard_normal((5, nx, ny)) + 1j * rng.standard_normal((5, nx, ny)))
    w = v.copy(order="F")
    L.a3_itrbc(ctypes.byref(o.g), ptr(w))
    assert np.array_equal(w[1:4, :-1, 0], bump[0:3, :-1])
    assert np.allclose(w[0, :, 0], 4 * w[0, :, 1] - 6 * w[0, :, 2] + 4 * w[0, :, 3] - w[0, :, 4], rtol=0, atol=1e-13)
    gc = [-2.083333333333333333333E+00, 4.0, -3.0, 1.333333333333333333333E+00, -2.5E-01]
    if wallt == 0:
        assert np.array_equal(w[4, :-1, 0], bump[3, :-1])
    else:
        s = sum(gc[k] * w[4, :, k] for k in range(5))
        assert np.allclose(s[:-1], bump[4, :-1], rtol=0, atol=1e-12)
    r = np.asfortranarray(rng.standard_normal((5, nx, ny)) + 0j)
    L.a3_rhsbc(ctypes.byref(o.g), ptr(r), ptr(v))
    assert np.allclose(r[1:4, :-1, 0], -(v[1:4, :-1, 0] - bump[0:3, :-1]), rtol=0, atol=1e-14)
    want0 = v[0, :, 0] - (4.0 * v[0, :, 1] - 6.0 * v[0, :, 2] + 4.0 * v[0, :, 3] - v[0, :, 4])
    assert np.allclose(r[0, :-1, 0], want0[:-1], rtol=0, atol=1e-13)
    m = o.lhs(2)
    for i, s_ in enumerate([3, 4, 5, 1, 2]):
        assert m[s_ - 1, 0, 0, 0, 0] == [-1.0, 4.0, -6.0, 4.0, -1.0][i]
    assert not m[:, 0, 1:, :, 0].any()
    v = case["v"].copy(order="F")
    for _ in range(3):
        o.step(v)
    assert np.isfinite(v).all() and np.array_equal(v[1:4, :-1, 0], bump[0:3, :-1])

"""Synthetic inputs of the linearised single-Fourier-mode ADI workloads.

The reference reads its grid, metrics and mean flow from ``grid.dat``,
``metric.dat`` and ``mean.dat`` (src/gengrid.f90:17-80, src/genmean.f90);
these generators produce the same arrays for an analytic mesh:

* grid: x uniform on [0, Lx] and periodic (point nx repeats point 1), y on
  [-Ly, Ly] clustered at the layer as y = Ly sinh(s (2 eta - 1)) / sinh(s); the
  computational coordinates are xi, eta in [0, 1] with d xi = 1/(nx-1),
  d eta = 1/(ny-1) (src/gengrid.f90:36-45);
* metrics: the ten arrays m1, m2, n1, n2, m11, m12, m22, n11, n12, n22 of the
  reference (d xi/dx, ..., d^2 eta/dy^2), exact for the analytic mapping;
* mean flow: a parallel compressible shear layer u = (1 + tanh(y/delta))/2,
  v = w = 0, T from the Crocco-Busemann relation for equal free-stream
  temperatures, T = 1 + (gamma-1)/2 Ma^2 u (1-u), rho = 1/T (uniform
  pressure);
* initial disturbance: seed-normal complex amplitudes times a Gaussian
  window in x (and one in y), scaled to a maximum of `amp`.

The default period Lx = 5.5 keeps every streamwise wavenumber of the
periodic box (2 pi k / Lx >= 1.14) above the Kelvin-Helmholtz neutral
wavenumber of the tanh layer (alpha delta = 1), so the layer is linearly
stable and the implicit pseudo-time iteration converges to the steady
(zero) disturbance; a longer box admits growing modes and the residual
grows, in the reference algorithm as here.

Arrays are numpy, Fortran-ordered, with the reference shapes: metrics
(nx, ny), vm (5, nx, ny), v (5, nx, ny) complex.

The deck values carry the reference's own constants: gamma1 = 0.4 as
src/init.f90:28 sets it (not gamma - 1, which differs in the last bit), and
the spanwise wavenumber as src/input.f90 forms it from the deck's span,
kz = 2 pi / Lz with Lz = 2 pi / beta.
"""
import math

import numpy as np

GAMMA = 1.4
GAMMA1 = 0.4


def span_of(beta):
    """The deck's Lz for a spanwise wavenumber beta (0: a 2D run)."""
    return 2.0 * math.pi / beta if beta else 0.0


def kz_of(Lz):
    """kz as src/input.f90 forms it from the deck's Lz."""
    return 2.0 * math.pi / Lz if Lz else 0.0


def shear_layer(nx=512, ny=256, Lx=5.5, Ly=10.0, stretch=3.0, delta=1.0, Ma=0.8, Re=500.0, Pr=0.72,
                beta=0.2, omega=0.05, amp=1e-6, seed=0, window=None):
    xi = np.linspace(0.0, 1.0, nx)
    eta = np.linspace(0.0, 1.0, ny)
    s = stretch
    z = s * (2.0 * eta - 1.0)
    y1 = Ly * np.sinh(z) / np.sinh(s)
    dy = Ly * 2.0 * s * np.cosh(z) / np.sinh(s)            # dy/deta
    d2y = Ly * 4.0 * s * s * np.sinh(z) / np.sinh(s)       # d2y/deta2
    x = np.asfortranarray(np.repeat((Lx * xi)[:, None], ny, axis=1))
    y = np.asfortranarray(np.repeat(y1[None, :], nx, axis=0))
    ones = np.ones((nx, ny))
    zeros = np.zeros((nx, ny))
    metrics = {
        "m1": ones / Lx, "m2": zeros.copy(), "n1": zeros.copy(),
        "n2": np.repeat((1.0 / dy)[None, :], nx, axis=0),
        "m11": zeros.copy(), "m12": zeros.copy(), "m22": zeros.copy(),
        "n11": zeros.copy(), "n12": zeros.copy(),
        "n22": np.repeat((-d2y / dy ** 3)[None, :], nx, axis=0),
    }
    metrics = {k: np.asfortranarray(v) for k, v in metrics.items()}
    u = 0.5 * (1.0 + np.tanh(y / delta))
    t = 1.0 + 0.5 * (GAMMA - 1.0) * Ma * Ma * u * (1.0 - u)
    vm = np.zeros((5, nx, ny), order="F")
    vm[0] = 1.0 / t
    vm[1] = u
    vm[4] = t
    rng = np.random.default_rng(seed)
    pert = rng.standard_normal((5, nx, ny)) + 1j * rng.standard_normal((5, nx, ny))
    w = window if window is not None else Lx / 8.0
    pert *= np.exp(-(((x - 0.5 * Lx) / w) ** 2))[None, :, :]
    pert *= np.exp(-((y / (0.25 * Ly)) ** 2))[None, :, :]
    pert *= amp / np.abs(pert).max()
    v = np.asfortranarray(pert.astype(np.complex128))
    params = dict(nx=nx, ny=ny, dxi=1.0 / (nx - 1), deta=1.0 / (ny - 1), Ma=Ma, Re=Re, Pr=Pr, gamma=GAMMA,
                  gamma1=GAMMA1, omega=omega, kz=kz_of(span_of(beta)), alfa=1.0, xper=1, yper=0, navier=1, wall=1, wallt=1,
                  top=0, optx=-1, opty=-1)
    return dict(params=params, x=x, y=y, metrics=metrics, vm=vm, v=v)


def _oseen_f(x):
    """f(x) of the Oseen vortex pressure (util/mkvortex.f90:238-249):
    1/2 - e^-x + e^-2x / 2 + x Ei(-2x) - x Ei(-x), and 1/2 beyond x = sqrt(200)."""
    from scipy.special import expi

    x = np.asarray(x, dtype=np.float64)
    out = np.full_like(x, 0.5)
    m = x <= np.sqrt(200.0)
    xm = x[m]
    out[m] = 0.5 - np.exp(-xm) + 0.5 * np.exp(-2.0 * xm) + xm * expi(-2.0 * xm) - xm * expi(-xm)
    return out


def vortex_grid(nx=128, ny=128, L=10.0, stretch=2.0):
    """The grid of the two-dimensional case: [-L, L]^2, x uniform, y =
    L tanh(s (2 eta - 1)) / tanh(s) on a uniform eta in [0, 1]."""
    xi = np.linspace(0.0, 1.0, nx)
    eta = np.linspace(0.0, 1.0, ny)
    y1 = L * np.tanh(stretch * (2.0 * eta - 1.0)) / np.tanh(stretch)
    x = np.asfortranarray(np.repeat((-L + 2.0 * L * xi)[:, None], ny, axis=1))
    y = np.asfortranarray(np.repeat(y1[None, :], nx, axis=0))
    return x, y


def vortex2d(nx=128, ny=128, L=10.0, stretch=2.0, Ma=0.5, Re=1000.0, Pr=0.72, circulation=1.0, seed=0,
             jitter=0.1):
    """The nonlinear two-dimensional case: an Oseen vortex in a uniform stream.

    * grid (vortex_grid): [-L, L]^2, x uniform and periodic (point nx is the
      periodic image of point 1), y = L tanh(s (2 eta - 1)) / tanh(s);
    * metrics as the reference's pre-processor forms them from the grid
      (lns3d_gb300.pre, pinned to pre/src_ij/pre.f90), differenced without
      its periodic option: that option wraps the coordinates themselves,
      which suits grids periodic in both coordinates (O-grids), while x here
      jumps by the period at the seam; the top boundary normal from the
      metrics as src/gengrid.f90:139-143 forms it;
    * state: uniform flow rho = u = T = 1 plus an Oseen vortex of core radius 1
      (alpha = 1.2564312086261697, util/mkvortex.f90:36) with the given
      circulation, its centre jittered uniformly by +-jitter from the origin
      by seed; the vortex pressure follows radial equilibrium with the
      isentropic relation (rho = (p/p_inf)^(1/gamma), T = p/(p_inf rho));
    * far field: the top.pot values are the state's top row, as the
      reference's vortex generator writes them (util/mkvortex.f90:183-188);
    * deck: Ma 0.5, Re 1000, Pr 0.72, viscous no-slip adiabatic wall at j = 1
      (wall 0, wallt 1), Riemann far field at j = ny (top 0), global time
      step at CFL 1.
    """
    from lns3d_gb300 import pre

    x, y = vortex_grid(nx, ny, L, stretch)
    metrics = pre.metrics(x, y, xper=False)
    rng = np.random.default_rng(seed)
    x0, y0 = rng.uniform(-jitter, jitter, 2)
    alpha = 1.2564312086261697
    xiv = 1.0 - np.exp(-alpha)
    amp = circulation * xiv / (2.0 * np.pi)        # v_theta(r) -> circulation / (2 pi r) far away
    gamma = GAMMA
    fact = 1.0 / (gamma * Ma * Ma)
    r = np.sqrt((x - x0) ** 2 + (y - y0) ** 2)
    th = np.arctan2(y - y0, x - x0)
    rs = np.where(r > 0.0, r, 1.0)
    vth = np.where(r > 0.0, amp * (1.0 - np.exp(-alpha * rs ** 2)) / (rs * xiv), 0.0)
    pr = np.where(r > 0.0, fact * (1.0 - (gamma - 1.0) * Ma ** 2 * amp ** 2 / (xiv * rs) ** 2
                                   * _oseen_f(alpha * rs ** 2)) ** (gamma / (gamma - 1.0)), fact)
    rho = (pr / fact) ** (1.0 / gamma)
    t = pr / (fact * rho)
    v = np.zeros((5, nx, ny), order="F")
    v[0] = rho
    v[1] = 1.0 - np.sin(th) * vth
    v[2] = np.cos(th) * vth
    v[4] = t
    v[:, -1, :] = v[:, 0, :]        # periodic point
    pot = np.asfortranarray(v[:, :, -1].copy())   # rho, u, v, w, T on the top row
    params = dict(nx=nx, ny=ny, dxi=1.0 / (nx - 1), deta=1.0 / (ny - 1), Ma=Ma, Re=Re, Pr=Pr, gamma=GAMMA,
                  gamma1=GAMMA1, omega=0.0, kz=0.0, alfa=1.0, xper=1, yper=0, navier=1, wall=0, wallt=1,
                  top=0, optx=-1, opty=-1)
    n1, n2 = metrics["n1"][:, -1], metrics["n2"][:, -1]
    bnt = np.zeros((nx, 2), order="F")     # (n1, n2) / |n| at j = ny (src/gengrid.f90:139-143)
    bnt[:, 0] = n1 / np.sqrt(n1 * n1 + n2 * n2)
    bnt[:, 1] = n2 / np.sqrt(n1 * n1 + n2 * n2)
    return dict(params=params, x=x, y=y, metrics=metrics, v=np.asfortranarray(v), pot=pot, bnt=bnt, theta=0.0)


def acoustic_box(nx=64, ny=63, Lx=1.0, Ly=1.0, Lz=1.0, Ma=1.0, Pr=1.0):
    """The reference's test/3d case: an inviscid oblique acoustic wave in a
    square box periodic in both directions (test/3d/README.md).

    * grid: uniform on [0, Lx] x [0, Ly] (test/3d/grid.inp), metrics exact;
    * mean flow: fluid at rest, rho = T = 1 (util/mkmean.f90, "no flow");
    * disturbance: the wave of util/mkdist3d.f90:155-215 with kx = 2 pi/Lx,
      ky = 2 pi/Ly: c3 = exp(i (kx x + ky y)), rho = c3 / (2 cm^2),
      u = c3 / (2 rho_m cm), v = w = 0, p = c3 / 2,
      T = (gamma Ma^2 p - T_m rho) / rho_m, cm = sqrt(T_m) / Ma;
    * deck (test/3d/cfl.inp): Ma 1, Re 0 (inviscid: Navier false and Re =
      1e99, src/input.f90:40-44), Pr 1, xper and yper, the span Lz.
    """
    x1 = np.linspace(0.0, Lx, nx)
    y1 = np.linspace(0.0, Ly, ny)
    x = np.asfortranarray(np.repeat(x1[:, None], ny, axis=1))
    y = np.asfortranarray(np.repeat(y1[None, :], nx, axis=0))
    ones = np.ones((nx, ny))
    zeros = np.zeros((nx, ny))
    metrics = {"m1": ones / Lx, "m2": zeros.copy(), "n1": zeros.copy(), "n2": ones / Ly,
               "m11": zeros.copy(), "m12": zeros.copy(), "m22": zeros.copy(),
               "n11": zeros.copy(), "n12": zeros.copy(), "n22": zeros.copy()}
    metrics = {k: np.asfortranarray(v) for k, v in metrics.items()}
    vm = np.zeros((5, nx, ny), order="F")
    vm[0] = 1.0
    vm[4] = 1.0
    kx, ky = 2.0 * math.pi / Lx, 2.0 * math.pi / Ly
    cm = np.sqrt(vm[4]) / Ma
    c3 = (np.cos(kx * x) * np.cos(ky * y) - np.sin(kx * x) * np.sin(ky * y)
          + 1j * (np.cos(kx * x) * np.sin(ky * y) + np.sin(kx * x) * np.cos(ky * y)))
    v = np.zeros((5, nx, ny), np.complex128, order="F")
    v[0] = 0.5 * c3 / cm ** 2
    v[1] = c3 * 0.5 / (vm[0] * cm)
    p = c3 * 0.5
    v[4] = (GAMMA * Ma ** 2 * p - vm[4] * v[0]) / vm[0]
    params = dict(nx=nx, ny=ny, dxi=1.0 / (nx - 1), deta=1.0 / (ny - 1), Ma=Ma, Re=1e99, Pr=Pr, gamma=GAMMA,
                  gamma1=GAMMA1, omega=0.0, kz=kz_of(Lz), alfa=1.0, xper=1, yper=1, navier=0, wall=-1, wallt=-1,
                  top=-1, optx=-1, opty=-1)
    return dict(params=params, x=x, y=y, metrics=metrics, vm=vm, v=v, span=Lz)


def boundary_normals(metrics):
    """The unit outward normals of the four boundaries as src/gengrid.f90:
    133-155 forms them from the metrics: bnb (nx, 2) at j = 1, bnt (nx, 2)
    at j = ny, bnl (ny, 2) at i = 1 and bnr (ny, 2) at i = nx."""
    out = {}
    for name, (a, b, sel, sign) in {"bnb": ("n1", "n2", (slice(None), 0), -1.0),
                                     "bnt": ("n1", "n2", (slice(None), -1), 1.0),
                                     "bnl": ("m1", "m2", (0, slice(None)), -1.0),
                                     "bnr": ("m1", "m2", (-1, slice(None)), 1.0)}.items():
        p, q = metrics[a][sel], metrics[b][sel]
        bn = np.zeros((p.size, 2), order="F")
        bn[:, 0] = sign * p / np.sqrt(p * p + q * q)
        bn[:, 1] = sign * q / np.sqrt(p * p + q * q)
        out[name] = bn
    return out


def pcyl(fixture):
    """The reference's swept parabolic-cylinder case (test/pcyl/sweep=35/
    M=0.8/Re=1e5) from its stored fixture (tests/golden/pcyl_sweep35.npz:
    the converged mean flow, metric.dat, top.pot and right.pot of the
    reference's own run, 384 x 128): Ma 0.8, Re 1e5, Pr 0.7, fourth-order
    stencils, xi non-periodic with the symmetry plane on the left (left 2)
    and the Riemann outflow on the right (right 0) extrapolated over the
    viscous layer (extrap 1, nbl 32 updated by itrBC), adiabatic no-slip
    wall, Riemann top, one global time step at CFL 400 (dtmax 1), smoother
    at eps_e 0.01 (the case's res.inp deck with the Pr and wall of the
    stored solution)."""
    names = ("m1", "m2", "n1", "n2", "m11", "m12", "m22", "n11", "n12", "n22")
    metrics = {k: np.asfortranarray(fixture["m_" + k]) for k in names}
    nx, ny = metrics["m1"].shape
    bn = boundary_normals(metrics)
    params = dict(nx=nx, ny=ny, dxi=1.0 / (nx - 1), deta=1.0 / (ny - 1), Ma=0.8, Re=1.0e5, Pr=0.7, gamma=GAMMA,
                  gamma1=GAMMA1, omega=0.0, kz=0.0, alfa=float(fixture["alfa"]), xper=0, yper=0, navier=1, wall=0,
                  wallt=1, top=0, optx=-1, opty=-1, left=2, right=0)
    return dict(params=params, metrics=metrics, v=np.asfortranarray(fixture["v0"]),
                bnt=bn["bnt"], pot=np.asfortranarray(np.asarray(fixture["top_pot"]).T),
                right_far=(bn["bnr"], np.asfortranarray(np.asarray(fixture["right_pot"]).T)),
                run=dict(cflmax=400.0, dtmax=1.0, loctime=0, theta=35.0, eps_e=0.01, extrap=1,
                         nbl=int(fixture["nbl0"]), update_nbl=True))


def vortex2d_open(nx=48, ny=40, seed=1, left=0, right=0, extrap=-1, **kw):
    """The two-dimensional vortex case (vortex2d) with a non-periodic xi
    direction: Riemann planes (left 0, right 0) or a symmetry plane (left
    2) at x = -L and x = L, their normals as src/gengrid.f90:145-155 forms
    them and their left.pot / right.pot values the state's boundary
    columns (as the top.pot values are its top row); extrap the deck's
    extrapolation of the right plane over the viscous layer."""
    case = vortex2d(nx=nx, ny=ny, seed=seed, **kw)
    case["params"].update(xper=0, left=left, right=right)
    bn = boundary_normals(case["metrics"])
    v = case["v"]
    case["left_far"] = (bn["bnl"], np.asfortranarray(v[:, 0, :].copy())) if left == 0 else None
    case["right_far"] = (bn["bnr"], np.asfortranarray(v[:, -1, :].copy())) if right == 0 else None
    case["extrap"] = extrap
    return case

"""Grid metrics from a grid, as the reference's pre-processor forms them
(pre/src_ij/pre.f90:74-150 with its gradient pre/src_ij/grad.f90).

The reference runs ``pre`` on ``grid.dat`` to write the metric file the
solver reads (``metric.dat``: m1, m2, n1, n2, m11, m12, m22, n11, n12, n22).
``pre`` differentiates the grid in computational space (xi, eta uniform on
[0, 1]) with its gradient operator, inverts the Jacobian, and differentiates
the first metrics once more:

    IdetJ = 1 / (x_xi y_eta - x_eta y_xi)
    m1 = y_eta IdetJ,  n1 = -y_xi IdetJ,  m2 = -x_eta IdetJ,  n2 = x_xi IdetJ
    m11 = m1 (m1)_xi + n1 (m1)_eta     n11 = m1 (n1)_xi + n1 (n1)_eta
    m22 = m2 (m2)_xi + n2 (m2)_eta     n22 = m2 (n2)_xi + n2 (n2)_eta
    m12 = m1 (m2)_xi + n1 (m2)_eta     n12 = m1 (n2)_xi + n1 (n2)_eta

``pre`` always differences with its fourth-order option (opt = -1: the
seven-point stencil with its outer weights zero), without the Carpenter
closures or symmetry planes; the only choice it offers is a periodic xi
direction, whose stencils wrap with the last point repeating the first, so it
suits grids whose coordinates are themselves periodic in xi (an O-grid), not
a Cartesian box periodic in x.  Every sum is evaluated in the reference's
order, term by term left to right, so the results are the reference's to
the last bit (checked against the translated ``pre`` in the CPU tests).
"""
import numpy as np

# pre/src_ij/stencil.f90: fourth-order one-sided and off-centre closures
# (weights over points 1..5 from the boundary, times 1/h)
_GC = (-25.0 / 12.0, 4.0, -3.0, 4.0 / 3.0, -0.25)                # point 1
_GB = (-0.25, -10.0 / 12.0, 1.5, -0.5, 1.0 / 12.0)               # point 2
_GA = (1.0 / 12.0, -8.0 / 12.0, 8.0 / 12.0, -1.0 / 12.0)         # point 3: points 1, 2, 4, 5


def _interior_weights(hinv):
    """pre/src_ij/grad.f90:37-55 with opt = -1 (c = 0): the weights of
    points i-3..i-1, i+1..i+3, already times 1/h."""
    c = 0.0
    a = (2.0 + 15.0 * c) / 3.0
    b = -(1.0 + 48.0 * c) / 12.0
    return (-c * hinv, -b * hinv, -a * hinv, a * hinv, b * hinv, c * hinv)


def _sum(terms):
    """Left-to-right sum of products (the reference's evaluation order)."""
    acc = terms[0][0] * terms[0][1]
    for w, f in terms[1:]:
        acc = acc + w * f
    return acc


def d1(f, axis, h, periodic=False):
    """The reference pre's first derivative of f along axis (0: xi, 1: eta)
    on a uniform computational grid of spacing h (pre/src_ij/grad.f90)."""
    F = np.moveaxis(np.asarray(f, dtype=np.float64), axis, 0)
    n = F.shape[0]
    if n < 7:
        raise ValueError("pre's stencils need at least seven points")
    hinv = 1.0 / h
    g = _interior_weights(hinv)
    G = np.empty_like(F)

    def seven(i, idx):
        return _sum(list(zip(g, (F[k] for k in idx))))

    for i in range(3, n - 3):
        G[i] = seven(i, (i - 3, i - 2, i - 1, i + 1, i + 2, i + 3))
    if periodic:
        # the last point repeats the first: period n-1 (grad.f90:85-126)
        m = n - 1
        for i in (0, 1, 2, n - 3, n - 2):
            G[i] = seven(i, tuple((i + o) % m for o in (-3, -2, -1, 1, 2, 3)))
        G[n - 1] = G[0]
    else:
        # boundary differences (grad.f90:187-241)
        G[0] = _sum(list(zip(_GC, (F[k] for k in range(5))))) * hinv
        G[1] = _sum(list(zip(_GB, (F[k] for k in range(5))))) * hinv
        G[2] = _sum(list(zip(_GA, (F[0], F[1], F[3], F[4])))) * hinv
        G[n - 3] = _sum(list(zip(_GA, (F[n - 5], F[n - 4], F[n - 2], F[n - 1])))) * hinv
        G[n - 2] = -(_sum(list(zip(_GB, (F[n - 1 - k] for k in range(5)))))) * hinv
        G[n - 1] = -(_sum(list(zip(_GC, (F[n - 1 - k] for k in range(5)))))) * hinv
    return np.moveaxis(G, 0, axis)


def metrics(x, y, xper=False, yper=False):
    """The ten metric arrays of the reference's metric file from the grid
    coordinates x, y (nx, ny), as pre/src_ij/pre.f90:74-150 forms them;
    xper: pre's hard-wired periodic xi direction (its first question)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    nx, ny = x.shape
    dxi = 1.0 / float(nx - 1)
    deta = 1.0 / float(ny - 1)

    def grad(f):
        return d1(f, 0, dxi, xper), d1(f, 1, deta, yper)

    x_xi, x_eta = grad(x)
    y_xi, y_eta = grad(y)
    idetj = 1.0 / (x_xi * y_eta - x_eta * y_xi)
    m1 = y_eta * idetj
    n1 = -y_xi * idetj
    m2 = -x_eta * idetj
    n2 = x_xi * idetj
    m1_xi, m1_eta = grad(m1)
    m2_xi, m2_eta = grad(m2)
    n1_xi, n1_eta = grad(n1)
    n2_xi, n2_eta = grad(n2)
    out = {
        "m1": m1, "m2": m2, "n1": n1, "n2": n2,
        "m11": m1 * m1_xi + n1 * m1_eta,
        "m12": m1 * m2_xi + n1 * m2_eta,
        "m22": m2 * m2_xi + n2 * m2_eta,
        "n11": m1 * n1_xi + n1 * n1_eta,
        "n12": m1 * n2_xi + n1 * n2_eta,
        "n22": m2 * n2_xi + n2 * n2_eta,
    }
    return {k: np.asfortranarray(v) for k, v in out.items()}

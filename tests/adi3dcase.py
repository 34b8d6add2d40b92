"""The 3D-step oracle harness, re-exported for the tests."""
from oracle.adi3d import A3Grid, A3Ops, Oracle3D, _lib, ptr  # noqa: F401


def sponge(nx, ny, amp=0.5):
    """A sponge of the reference's kind for the shear-layer grid: spg rises
    towards the far field (j = ny), spg2 is a Gaussian band in x; both
    (nx, ny) Fortran arrays."""
    import numpy as np

    x = np.linspace(0.0, 1.0, nx)
    y = np.linspace(0.0, 1.0, ny)
    spg = np.asfortranarray(amp * np.outer(np.ones(nx), y ** 3))
    spg2 = np.asfortranarray(0.3 * amp * np.outer(np.exp(-((x - 0.25) / 0.1) ** 2), np.ones(ny)))
    return spg, spg2

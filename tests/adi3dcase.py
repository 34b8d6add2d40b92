"""The 3D-step oracle harness, re-exported for the tests."""
from oracle.adi3d import A3Grid, A3Ops, Oracle3D, _lib, ptr  # noqa: F401

"""Test cases for the line solvers: seeded systems in the reference layouts,
and runners for the oracle, the translated reference and the GPU library.

Systems follow the isolated batched solve workload: real and imaginary parts
of every block entry uniform in [-1, 1], diagonal blocks + 10*I, right-hand
side uniform in [-1, 1] (normal for the full-size workload).
"""
import numpy as np

import oracle

SOLVERS = ["penta2bc", "penta1bc", "cpenta2bc", "cpenta1bc", "penta2p", "penta1p", "cpenta2p", "cpenta1p"]


def info(solver):
    return dict(complex=solver.startswith("c"), layout=1 if "1" in solver else 2, periodic=solver.endswith("p"))


def shapes(solver, rows, nsys):
    lay = info(solver)["layout"]
    mat = (5, 5, 5, rows, nsys) if lay == 2 else (5, 5, 5, nsys, rows)
    rhs = (5, rows, nsys) if lay == 2 else (5, nsys, rows)
    per = (2, 5, 5, rows, nsys) if lay == 2 else (2, 5, 5, nsys, rows)
    return mat, rhs, per


def make_case(solver, rows, nsys, seed, normal_rhs=False):
    """rows = n for boundary solvers, np = n+1 for periodic ones."""
    c = info(solver)
    rng = np.random.default_rng(seed)
    ms, rs, ps = shapes(solver, rows, nsys)

    def u(shape):
        a = rng.uniform(-1.0, 1.0, shape)
        if c["complex"]:
            a = a + 1j * rng.uniform(-1.0, 1.0, shape)
        return a

    mat = u(ms)
    mat[2] += 10.0 * np.eye(5)[:, :, None, None]
    if normal_rhs:
        rhs = rng.standard_normal(rs) + (1j * rng.standard_normal(rs) if c["complex"] else 0)
    else:
        rhs = u(rs)
    dt = np.complex128 if c["complex"] else np.float64
    case = dict(solver=solver, rows=rows, nsys=nsys, mat=np.asfortranarray(mat, dtype=dt),
                rhs=np.asfortranarray(rhs, dtype=dt))
    if c["periodic"]:
        case["per"] = np.zeros(ps, dt, order="F")
        case["per2"] = np.zeros(ps, dt, order="F") if c["complex"] else np.zeros((6, 5, 5, nsys), dt, order="F")
    return case


def copy(case):
    return {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in case.items()}


def dims(case):
    c = info(case["solver"])
    return (case["rows"], case["nsys"]) if c["layout"] == 2 else (case["nsys"], case["rows"])


def run_oracle(case, code=2, flags=oracle.COMPAT_PERIODIC_SLOT):
    """Runs the restated oracle in place on a copy; returns the copy."""
    out = copy(case)
    c = info(case["solver"])
    O, p = oracle.orc(), oracle.ptr
    lay, rows, nsys = c["layout"], case["rows"], case["nsys"]
    if not c["periodic"] and not c["complex"]:
        rc = O.orc_penta_bc(lay, rows, nsys, p(out["mat"]), p(out["rhs"]))
    elif not c["periodic"]:
        rc = O.orc_cpenta_bc(lay, rows, nsys, p(out["mat"]), p(out["rhs"]), code, flags)
    elif not c["complex"]:
        rc = O.orc_penta_p(lay, rows, nsys, p(out["mat"]), p(out["rhs"]), p(out["per"]), flags)
    else:
        rc = O.orc_cpenta_p(lay, rows, nsys, p(out["mat"]), p(out["rhs"]), p(out["per"]), p(out["per2"]), code, flags)
    assert rc == 0, rc
    return out


def run_ref(case, code=2):
    """Runs the translated reference (single pass in line order) on a copy,
    or returns None where it was not built."""
    R = oracle.ref()
    if R is None:
        return None
    out = copy(case)
    c = info(case["solver"])
    p = oracle.ptr
    f = getattr(R, "ref_" + case["solver"])
    d = dims(case)
    if not c["periodic"] and not c["complex"]:
        f(d[0], d[1], 5, p(out["mat"]), p(out["rhs"]))
    elif not c["periodic"]:
        f(d[0], d[1], 5, p(out["mat"]), p(out["rhs"]), code)
    elif not c["complex"]:
        f(d[0], d[1], 5, p(out["mat"]), p(out["rhs"]), p(out["per"]), p(out["per2"]))
    else:
        f(d[0], d[1], 5, p(out["mat"]), p(out["rhs"]), p(out["per"]), p(out["per2"]), code)
    return out


def run_gpu(case, code=2, device=None):
    """Runs the GPU library on a copy: host arrays (device=None) or CUDA
    tensors on `device`."""
    import lns3d_gb300 as g

    out = copy(case)
    c = info(case["solver"])
    fn = getattr(g, case["solver"])
    d = dims(case)
    args = [out["mat"], out["rhs"]]
    names = ["mat", "rhs"]
    if c["periodic"]:
        names += ["per", "per2"]
        args += [out["per"], out["per2"]]
    if device is not None:
        import torch

        args = [torch.from_numpy(out[k].ravel(order="F")).to(device) for k in names]
    extra = [code] if c["complex"] else []
    fn(d[0], d[1], 5, *args, *extra)
    if device is not None:
        for k, a in zip(names, args):
            out[k] = a.cpu().numpy().reshape(out[k].shape, order="F")
    return out


def relerr(a, b):
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))

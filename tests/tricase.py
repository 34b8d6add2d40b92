"""Seeded cases of the block-tridiagonal line solvers of the second-order
implicit path (src/nsolve{1,2}{bc,p}.f90) and their runners: the oracle
(oracle/tri_oracle.c), the translated reference (oracle/_ref) and the GPU
entry points (lns_solve{1,2}{bc,p}).

Layouts are the reference's: "2" solvers mat(3,5,5,rows,nsys),
rhs(5,rows,nsys); "1" solvers mat(3,5,5,nsys,rows), rhs(5,nsys,rows);
boundary solvers add bc(14,5,5,nsys); periodic solvers take np = rows
(row np repeats row 1) and the scratch per(5,5,np,nsys), per2(2,5,5,nsys).
"""
import ctypes

import numpy as np

SOLVERS = ["solve2bc", "solve1bc", "solve2p", "solve1p"]


def info(solver):
    return {"layout": 2 if solver[5] == "2" else 1, "periodic": solver.endswith("p")}


def make_case(solver, rows, nsys, seed=0):
    c = info(solver)
    rng = np.random.default_rng(seed)
    shp = (3, 5, 5, rows, nsys) if c["layout"] == 2 else (3, 5, 5, nsys, rows)
    mat = rng.uniform(-1.0, 1.0, shp)
    mat[1] += 10.0 * np.eye(5)[:, :, None, None]
    rhs = rng.standard_normal((5, rows, nsys) if c["layout"] == 2 else (5, nsys, rows))
    case = {"solver": solver, "rows": rows, "nsys": nsys, "mat": np.asfortranarray(mat),
            "rhs": np.asfortranarray(rhs)}
    if not c["periodic"]:
        case["bc"] = np.asfortranarray(rng.uniform(-0.5, 0.5, (14, 5, 5, nsys)))
    return case


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def run_ref(case):
    """The reference's own solver sources (translated): solution in rhs."""
    import oracle

    L = oracle.ref()
    s, rows, nsys = case["solver"], case["rows"], case["nsys"]
    mat = case["mat"].copy(order="F")
    rhs = case["rhs"].copy(order="F")
    fn = getattr(L, "ref_" + s)
    a, b = (rows, nsys) if info(s)["layout"] == 2 else (nsys, rows)
    if info(s)["periodic"]:
        per = np.zeros((5, 5, rows, nsys), order="F")
        per2 = np.zeros((2, 5, 5, nsys), order="F")
        fn(a, b, 5, _p(mat), _p(rhs), _p(per), _p(per2))
    else:
        bc = case["bc"].copy(order="F")
        fn(a, b, 5, _p(mat), _p(rhs), _p(bc))
    return rhs


def run_oracle(case, lib=None):
    import oracle

    L = lib or oracle.orc()
    s, rows, nsys = case["solver"], case["rows"], case["nsys"]
    rhs = case["rhs"].copy(order="F")
    lay = info(s)["layout"]
    if info(s)["periodic"]:
        rc = L.orc_tri_p(lay, rows, nsys, _p(case["mat"]), _p(rhs))
    else:
        rc = L.orc_tri_bc(lay, rows, nsys, _p(case["mat"]), _p(rhs), _p(case["bc"]))
    assert rc == 0, rc
    return rhs


def dense_line(case, iv):
    """The line's matrix as a dense (5n, 5n) array (n unknown rows), from
    the block table of the reference solvers (oracle/tri_oracle.c)."""
    s, rows = case["solver"], case["rows"]
    c = info(s)
    per = c["periodic"]
    n = rows - 1 if per else rows
    A = np.zeros((5 * n, 5 * n))

    def blk(k, t):
        m = case["mat"]
        return m[k - 1, :, :, t - 1, iv] if c["layout"] == 2 else m[k - 1, :, :, iv, t - 1]

    def bcb(j):
        return case["bc"][j - 1, :, :, iv]

    def put(t, col, B):
        if per:
            col = (col - 1) % n + 1
        A[5 * (t - 1):5 * t, 5 * (col - 1):5 * col] += B

    for t in range(1, n + 1):
        if per:
            for k in (1, 2, 3):
                put(t, t + k - 2, blk(k, t))
            continue
        table = {1: [(1, "m", 2), (2, "m", 3), (3, "b", 1), (4, "b", 2), (5, "b", 3)],
                 2: [(1, "m", 1), (2, "m", 2), (3, "m", 3), (4, "b", 4), (5, "b", 5)],
                 3: [(1, "b", 7), (2, "m", 1), (3, "m", 2), (4, "m", 3), (5, "b", 6)],
                 n - 2: [(n - 4, "b", 8), (n - 3, "m", 1), (n - 2, "m", 2), (n - 1, "m", 3), (n, "b", 9)],
                 n - 1: [(n - 4, "b", 10), (n - 3, "b", 11), (n - 2, "m", 1), (n - 1, "m", 2), (n, "m", 3)],
                 n: [(n - 4, "b", 12), (n - 3, "b", 13), (n - 2, "b", 14), (n - 1, "m", 1), (n, "m", 2)]}
        ent = table.get(t, [(t - 1, "m", 1), (t, "m", 2), (t + 1, "m", 3)])
        for col, kind, j in ent:
            put(t, col, blk(j, t) if kind == "m" else bcb(j))
    return A


def line_rhs(case, a, iv):
    """The n-row right-hand side of line iv from a rhs array."""
    s, rows = case["solver"], case["rows"]
    n = rows - 1 if info(s)["periodic"] else rows
    x = a[:, :n, iv] if info(s)["layout"] == 2 else a[:, iv, :n]
    return x.reshape(-1, order="F")

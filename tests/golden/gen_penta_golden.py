#!/usr/bin/env python3
"""Generates tests/golden/penta_<solver>.npz: seeded inputs and the outputs
of the reference's own solver sources (translated to C by
oracle/f77sub2c.py and built into oracle/_ref/libref_penta.so), run in one
thread so that the complex boundary solvers' mis-indexed row (src/cpenta1bc.f:675,
src/cpenta2bc.f:676) is deterministic.

Run in a container that has the reference tree:
    make -C oracle && OMP_NUM_THREADS=1 python tests/golden/gen_penta_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import pentacase  # noqa: E402

CASES = {  # solver: (rows, nsys); rows = np for periodic solvers
    "penta2bc": (9, 2), "penta1bc": (8, 3), "cpenta2bc": (8, 2), "cpenta1bc": (9, 2),
    "penta2p": (10, 2), "penta1p": (9, 3), "cpenta2p": (9, 2), "cpenta1p": (10, 2),
}


def main():
    assert os.environ.get("OMP_NUM_THREADS") == "1", "run with OMP_NUM_THREADS=1"
    for k, (solver, (rows, nsys)) in enumerate(sorted(CASES.items())):
        case = pentacase.make_case(solver, rows, nsys, seed=1000 + k)
        info = pentacase.info(solver)
        data = {"rows": rows, "nsys": nsys, "mat_in": case["mat"], "rhs_in": case["rhs"]}
        if info["complex"]:
            fac = pentacase.run_ref(case, code=0)
            data["mat_factored"] = fac["mat"]
            if info["periodic"]:
                data["per_factored"], data["per2_factored"] = fac["per"], fac["per2"]
            full = pentacase.run_ref(case, code=2)
        else:
            full = pentacase.run_ref(case)
        data["rhs_out"] = full["rhs"]
        np.savez_compressed(os.path.join(HERE, "penta_%s.npz" % solver), **data)
        print(solver, rows, nsys)


if __name__ == "__main__":
    main()

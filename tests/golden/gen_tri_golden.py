#!/usr/bin/env python3
"""Generates tests/golden/tri_<solver>.npz: seeded inputs and the outputs of
the reference's own block-tridiagonal solver sources (src/nsolve{1,2}{bc,p}.f90,
translated to C by oracle/f77sub2c.py into oracle/_ref/libref_penta.so).

Run in a container that has the reference tree:
    make -C oracle && python tests/golden/gen_tri_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import tricase  # noqa: E402

CASES = {"solve2bc": (10, 2), "solve1bc": (9, 3), "solve2p": (11, 2), "solve1p": (10, 3)}


def main():
    for k, (solver, (rows, nsys)) in enumerate(sorted(CASES.items())):
        case = tricase.make_case(solver, rows, nsys, seed=2000 + k)
        data = {"rows": rows, "nsys": nsys, "mat_in": case["mat"], "rhs_in": case["rhs"],
                "rhs_out": tricase.run_ref(case)}
        if "bc" in case:
            data["bc_in"] = case["bc"]
        np.savez_compressed(os.path.join(HERE, "tri_%s.npz" % solver), **data)
        print(solver, rows, nsys)


if __name__ == "__main__":
    main()

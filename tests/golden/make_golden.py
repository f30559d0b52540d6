"""Generates the committed golden fixtures of tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py

The reference (Julia) cannot run in this environment, so the fixtures pin the
oracle restatement: the KernelMatrix products of examples/Kernel.jl's point
families and kernels, and of the n=2048 interleaved grid, with their dense FP64
products and tree statistics.  Tests check the oracle and the GPU library
against these files.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402

KERNELS = {"cauchy": O.CAUCHY, "coulomb": O.COULOMB, "coulombprime": O.COULOMB_PRIME, "log": O.LOG}


def case(kernel, x, y, box, seed):
    b = np.random.default_rng(seed).standard_normal(len(y))
    H = O.OracleKernelMatrix(KERNELS[kernel], x, y, *box)
    u = H @ b
    ud = O.kernel_dense(KERNELS[kernel], x, y) @ b
    st = H.stats()
    return dict(x=x, y=y, box=np.array(box), b=b, u=u, u_dense=ud,
                stats=np.array([st["bary"], st["dense"], st["depth"], st["stored_values"]]))


def main():
    out = {}
    x, y = O.grid_points(2048)
    out["grid2048_cauchy"] = case("cauchy", x, y, (1.0, 0.0, 1.0, 0.0), 0)
    for fam in ("chebyshev", "quadratic"):
        x, y, box = O.example_points(fam, 1000)
        for k in KERNELS:
            out[f"{fam}1000_{k}"] = case(k, x, y, box, 1)
    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
        rel = np.linalg.norm(d["u"] - d["u_dense"]) / np.linalg.norm(d["u_dense"])
        print(f"{name}: stats {d['stats'].tolist()} rel vs dense {rel:.2e}")


if __name__ == "__main__":
    main()

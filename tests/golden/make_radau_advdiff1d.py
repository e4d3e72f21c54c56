"""Writes tests/golden/radau_advdiff1d.npy: the comparison solution of the 1D
solver benchmark (benchmarks/benchmark_solver_comparison.py:67-121), SciPy Radau
(rtol 1e-6, atol 1e-8) on the periodic FD semi-discretisation of
u_t = 0.01 u_xx - u_x, N = 1024, u0 = exp(-100 (x - 0.5)^2), t in [0, 10].

Usage: python tests/golden/make_radau_advdiff1d.py   (about 20 s of CPU time)
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import fftcn  # noqa: E402

if __name__ == "__main__":
    u0 = fftcn.solver_comparison_ic(1024)
    ref, n_out = fftcn.radau_advdiff_1d(u0, 0.01, 1.0, 10.0)
    print("Radau output times:", n_out)
    np.save(os.path.join(HERE, "radau_advdiff1d.npy"), ref)

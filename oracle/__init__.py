"""CPU oracle for the moljax method-of-lines step path.

TEST INFRASTRUCTURE ONLY.  This package is a NumPy FP64 restatement of the
reference moljax algorithms (gogipav14/moljax, JAX).  It exists so that the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
can check the CUDA path against an independent implementation.  The product
package ``moljax_gb300`` never imports it; nothing under ``oracle/`` is
shipped or measured as the product.

Every function cites the reference file:line it restates.  Parity is pinned
against the reference's own published numbers (see ``tests/golden``):
the FFT-CN error table of ``benchmarks/results/precision_fp32_fp64.json``
and ``benchmarks/results/scipy_comparison.json``, plus the known-answer
assertions of the reference test-suite (Helmholtz residuals, FD symbol zero
mode, IMEX pure-diffusion decay, fixed-dt == manual Strang steps, ...).
"""

from oracle import mol, fftcn, imex  # noqa: F401

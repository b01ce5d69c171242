"""CPU oracle for the PyFlow projection step (TEST INFRASTRUCTURE ONLY).

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may import
it.  The GPU package (``pyflow_solver_gb300``) never routes through it and
fails loudly when its CUDA library is missing.

Contents
--------
ops      NumPy restatement of the reference's array operators
         (coherent gradient/divergence/Laplacian, central divergence,
         QUICK and upwind advection).
xsum     Exactly rounded dot products and sums (order independent), the
         "twin" reductions that the CUDA kernels reproduce bit for bit.
cg       Restatement of the preconditioned CG sequence of
         ``scipy.sparse.linalg.cg`` (SciPy, pinned 1.13.1 by the reference's
         pyproject.toml:20; 1.18.1 installed) with a pluggable dot product.
step     Restatement of ``step`` / ``solve_pressure_poisson`` /
         ``SimulationDriver.run`` of the reference.
workloads  Seeded generators of the benchmark configurations.

Parity is pinned: in ``reductions='numpy'`` mode the oracle reproduces the
reference bit for bit on the platform that generated the golden fixtures
(``tests/golden/make_golden.py`` runs the reference itself); in
``reductions='exact'`` mode every dot/sum is exactly rounded, which is the
order-independent form the CUDA path matches bit for bit on any platform.
"""

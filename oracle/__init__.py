"""CPU FP64 oracle for the jax-fem hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in numpy/scipy (plus torch.func on the CPU in float64
where the reference uses JAX forward/reverse-mode AD), the algorithm of
deepmodeling/jax-fem's hot path:

  * basis tables and quadrature          jax_fem/basis.py:19-250
  * per-cell geometry (shape grads, JxW)  jax_fem/fe.py:112-218
  * Dirichlet / boundary-face selection   jax_fem/fe.py:220-322
  * COO index build and PETSc AIJ pattern jax_fem/problem.py:86-107, jax_fem/solver.py:469-529
  * cell / mass / surface kernels         jax_fem/problem.py:189-356
  * residual scatter and element tangents jax_fem/problem.py:359-460
  * BC row elimination, Newton loop       jax_fem/solver.py:290-421, 1112-1356
  * linear solvers (jax bicgstab rule)    jax_fem/solver.py:63-134, 261-284
  * implicit adjoint (ad_wrapper)         jax_fem/solver.py:1362-1455

It is the checker, never the thing measured or shipped: only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import it.  The
product package never imports it and has no CPU fallback.

Pinning: the restatement is checked against the reference's own FEniCSx gold
fixtures (tests/golden/*.npz, extracted from the reference's
tests/benchmarks/*/fenicsx/ by tests/golden/make_golden.py) at the tolerances
the reference's tests use (decimal 5 / 3 / 4).  The CSR pattern, assembled
values and adjoint gradients have no fixture in the reference; they are pinned
by the restatement itself, AD cross-checks and central finite differences.
"""

"""CPU oracle for the jax_lbm D3Q19 time-step hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped package imports this
directory; only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline / reference arm use it, and only as the checker or as the
timed CPU restatement -- never as the thing measured on the GPU.

What it is: an op-for-op restatement of the reference's pure-JAX solver in
PyTorch on the CPU (float32 or float64, differentiable with autograd so it
stands in for ``jax.grad``).  The reference itself (JAX/XLA) cannot run in
this environment.  Every function cites the reference file:line it follows.

Pinning: the restatement is pinned to the reference's own published values
(``tests/test_oracle_pins.py``): the FP64 AD/FD table (d(sum f_eq)/d rho = 64,
d rho_bar/dU = 0.611238, Bouzidi dCd/dr = 93.33275), the Poiseuille profile,
the drag-coefficient and projected-area known answers, and the per-op unit
properties of the reference test-suite.
"""

"""CPU oracle: a plain numpy restatement of tincr's linear-response excited-state path.

TEST INFRASTRUCTURE ONLY.  Nothing in the `tincr_gb300` package imports this folder; only the
tests, `__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` use it, and only as the
checker (or, in the bench, as the timed CPU baseline).  The GPU product path never routes through
it.

Each function cites the tincr source (file:line inside the tincr project) it restates.  The
restatement keeps tincr's order of operations and data layouts (q_ov[A, i*v + a], occupied-major
CI vectors, [3N, n_orb, n_orb] derivative tensors) so that its outputs can be compared one to one.

Parity anchors (golden data under tests/golden/):
* gamma / gamma_lr and their gradients against tincr's tests/data fixtures (1e-15);
* water TDA energies from explicit S, orbital energies and coefficients (known-answer test of
  `not_refactored_tests/solver.rs`, 1e-10) and the 2x2 active-space TDA known answer (1e-14);
* Davidson against dense diagonalisation (tincr's `tda/system.rs:105-159` design);
* analytic gradients against central finite differences of the excitation energy
  (tincr's `gradients/numerical.rs` design).
"""

"""CPU oracle for the probabilistic IVP hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
directory.  It is used by ``tests/``, by ``__graft_entry__.smoke()`` as the
checker, and by ``bench.py``'s CPU-baseline / reference arm.

The Python modules restate, in PyTorch float64 on the CPU, the reference
algorithm of pnkraemer/probdiffeq for the per-step hot path: the
integrated-Wiener-process prior, TS0/TS1 linearisation, the QR-based
square-root Kalman update (``revert_conditional``), calibration, the
residual-based error estimate, the I/PI controllers, the adaptive rejection
loop with checkpoints, the filter / fixed-point / fixed-interval strategies,
and the log-marginal-likelihood.  Every function cites the reference
``file:line`` it follows (paths relative to the reference project root).

The reference is JAX code; JAX is not installed on the build or the GPU
machines, so the reference itself cannot run.  The restatement is pinned to
the reference's own known-answer tests and equivalence tests (see
``tests/test_oracle_*.py``), to closed-form results, and to a
high-accuracy classical ODE solver (scipy DOP853), which is what the
reference's own accuracy tests compare against.  One exception: the
log-marginal-likelihood's values and gradients are parity unpinned by the
reference, whose tests only check that they are finite; here they are
pinned by internal consistency only (PyTorch reverse mode through the
restatement against central finite differences, and forward-mode and
adjoint kernels against both).

``oracle/port`` holds a plain-C float64 port of the isotropic TS0 adaptive
solver (the ensemble configuration) used as the timed CPU baseline.
"""

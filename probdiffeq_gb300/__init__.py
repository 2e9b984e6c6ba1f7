"""GB300-native probabilistic IVP solvers (sm_103a).

A from-scratch implementation of the per-step hot path of probabilistic ODE
solvers (pnkraemer/probdiffeq): integrated-Wiener-process prediction, TS0/TS1
linearisation, the QR-based square-root Kalman update, calibration, the
residual-based error estimate and adaptive step control, batched over many
independent IVP instances in hand-written CUDA kernels.

Public modules:
  * ``probdiffeq_gb300.ivpsolve`` / ``probdiffeq_gb300.probdiffeq`` -- the
    reference's constructor and solve API, lowered to one native call;
  * ``probdiffeq_gb300.ensemble`` -- batched solves on tensors;
  * ``probdiffeq_gb300.autograd`` -- the LML kernel as a torch.autograd.Function;
  * ``probdiffeq_gb300.replicas`` -- sharding independent instances over ranks;
  * ``probdiffeq_gb300._native`` -- the ctypes binding of ``include/pdq.h``.
"""

from . import _native  # noqa: F401

__all__ = ["_native"]

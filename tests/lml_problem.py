"""The LML-gradient configuration shared by tests and the benchmark (the
generators live in ``probdiffeq_gb300.configs``; these are their names in the
tests)."""

from probdiffeq_gb300.configs import FHN_STD as STD  # noqa: F401
from probdiffeq_gb300.configs import FHN_THETA_STAR as THETA_STAR  # noqa: F401
from probdiffeq_gb300.configs import FHN_U0 as U0  # noqa: F401
from probdiffeq_gb300.configs import _fhn as fhn  # noqa: F401
from probdiffeq_gb300.configs import fhn_observations as observations  # noqa: F401
from probdiffeq_gb300.configs import fhn_theta_samples as theta_samples  # noqa: F401

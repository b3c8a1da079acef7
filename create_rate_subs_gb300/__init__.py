"""GB300 (sm_103a) evaluation of the species and reaction rates that
kyleniemeyer/create_rate_subs generates as straight-line code.

Front end (host, no GPU needed): ``mech_interpret.read_mech``,
``mechanism.Mechanism``, ``create_rate_subs.create_rate_subs`` / the CLI
(``python -m create_rate_subs_gb300``).  Evaluation (GPU):
``rates.RateSubs`` over libcrs (include/crs.h).
"""

from .mech_interpret import MechanismError, read_mech, read_thermo  # noqa: F401
from .mechanism import Mechanism  # noqa: F401

__all__ = ["read_mech", "read_thermo", "MechanismError", "Mechanism"]

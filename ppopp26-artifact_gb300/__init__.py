"""GB300-native Fr prover operators (NTT/INTT, coset LDE, grand product,
evaluation, division by X - z) behind the reference's operator interface.

The directory name is not a Python identifier; load it with
``__graft_entry__.load_package()`` (module name ``ppopp26_artifact_gb300``).
"""
from . import ppfr  # noqa: F401
from .ppfr import (LDE_COEFFS, LDE_EVALS, LDE_SPREAD, PPError, div_xplusc_, evaluate,  # noqa: F401
                   gp_perm, gp_prefix_, intt, launch_count, lde, ntt, random_fr)

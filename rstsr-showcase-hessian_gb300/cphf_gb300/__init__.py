"""cphf_gb300 -- GB300 CPHF/CPKS response path (RI-J, RI-K, XC response, block Krylov).

Python face of ``libcphf.so`` (C ABI in ``include/cphf.h``).  ``Context`` mirrors the
reference crate's plugin and driver methods; ``synth`` builds seeded synthetic systems.
"""

from .api import (Config, Context, CphfError, KrylovNotConverged, Stats, LIB_PATH, EXPORTS,  # noqa: F401
                  load_library)
from . import synth  # noqa: F401


def build(force=False):
    """Compile libcphf.so for sm_103a (nvcc) next to this package."""
    from . import _build
    return _build.build(force=force)

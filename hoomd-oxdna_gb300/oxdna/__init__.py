"""oxDNA / oxRNA force hot path on GB300 (sm_103a).

The same Python surface as the reference HOOMD plugin (``oxdna.forces``,
``oxdna.model.dna1|dna2|rna2``, ``oxdna.io``) over a native CUDA engine
(``liboxdna_gb300.so``, C ABI in ``include/oxdna_gb300.h``). ``oxdna.runtime``
stands in for the HOOMD-blue simulation objects the reference runs inside.
"""

from . import _abi  # noqa: F401
from . import io  # noqa: F401
from . import forces  # noqa: F401
from . import runtime  # noqa: F401
from . import model  # noqa: F401

from .version import version  # noqa: F401

__all__ = ["io", "forces", "model", "runtime", "version"]

"""oxDNA model variants: oxDNA1, oxDNA2 and oxRNA2 over the same force engine."""

from . import dna1  # noqa: F401
from . import dna2  # noqa: F401
from . import rna2  # noqa: F401

__all__ = ["dna1", "dna2", "rna2"]

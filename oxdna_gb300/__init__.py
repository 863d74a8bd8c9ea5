"""oxdna_gb300: GB300-native oxDNA2 MD hot path (forces, Verlet lists, integrator, thermostats).

The compute path is liboxgb.so (hand-written CUDA for sm_103a behind the C ABI of
include/oxgb.h); this package holds its Python front end and the host-side file formats.
"""

from ._abi import OxgbError, lib, library_path  # noqa: F401
from .md import MDSystem, dna2_settings, md_settings  # noqa: F401

__all__ = ["OxgbError", "lib", "library_path", "MDSystem", "dna2_settings", "md_settings"]

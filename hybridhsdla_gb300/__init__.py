"""GB300-native (sm_103a) FLAPW Hamiltonian/overlap generation.

The compute path is ``libhsdla_gb300.so`` (C ABI in ``include/hsdla.h``); this
package holds its in-tree build (``build``), the Python mirror of the reference
entry point (``api``) and the seeded input generator (``synth``).
"""
from . import synth  # noqa: F401

__all__ = ["synth", "api", "build"]

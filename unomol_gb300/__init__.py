"""unomol_gb300: GB300-native (sm_103a) direct two-electron Fock build for unomol.

The CUDA library (libunomol_gb300.so, C ABI in include/unomol_gb300.h) replaces unomol's
TwoElectronInts; this package holds its Python binding, a mirror of the reference's Basis reader, and
the synthetic molecules of the benchmark workloads.
"""
from .basis import Basis, full_to_packed, packed_to_full  # noqa: F401

__all__ = ["Basis", "full_to_packed", "packed_to_full"]

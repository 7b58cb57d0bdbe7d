"""gbsym -- GB300-native sparse triangular-solve executor.

A from-scratch sm_103a implementation of the triangular-solve path of
sympiler/sympiler: the CSR/CSC SpTRSV executors (serial, level-set and LBC
scheduled), the SpMV they pair with, the ILU0/IC0 producers and the
PCG/GMRES drivers around them, behind a C ABI (``include/gbsym.h``) that
keeps the reference's signatures.

* ``sympiler_gb300.sym_lib`` -- the reference's function names over numpy
  host arrays (drop-in semantics).
* ``sympiler_gb300.plans``   -- device-resident plans over torch tensors.
* ``sympiler_gb300.matgen``  -- seeded synthetic operators.
"""
from ._lib import GbsymError, lib  # noqa: F401

__all__ = ["GbsymError", "lib"]

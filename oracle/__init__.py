"""TEST INFRASTRUCTURE ONLY: the CPU oracle (comd_oracle.c) and the compiled
reference (oracle/_ref) behind one ctypes interface.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
load this package, to check results; the GB300 library never calls it.
"""
from .oracle import (KIND_EAM_CHEBY, KIND_EAM_TABLE, KIND_LJ, Oracle, RefCentro, RefLib, build,
                     oracle_lib, ref_centro, ref_lib)

__all__ = ["Oracle", "RefLib", "RefCentro", "oracle_lib", "ref_lib", "ref_centro", "build", "KIND_EAM_TABLE",
           "KIND_EAM_CHEBY", "KIND_LJ"]

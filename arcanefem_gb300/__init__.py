"""arcanefem_gb300: GB300-native (sm_103a) node-wise P1 assembly and Krylov solve.

The compute lives in libafem_gb300.so (C ABI: include/afem_gb300.h).  This
package holds its Python binding and a host-side mirror of ArcaneFEM's
BSRFormat / DoFLinearSystem interfaces (:mod:`arcanefem_gb300.fem`).
"""
from ._capi import AfemError, LIB_PATH, lib  # noqa: F401

__all__ = ["AfemError", "LIB_PATH", "lib"]

"""GB300-native (sm_103a) seminaive spherical harmonic transform with S2kit's memo-path API.

`s2kit_gb300.api` mirrors the reference C interface (FSTSemiMemo, InvFSTSemiMemo, FZTSemiMemo,
ConvOn2SphereSemiMemo, DLTSemi, table builders, ...) over the C ABI of libs2kit_gb300.so, and
adds the batched device-pointer `Plan` API.
"""
from . import api  # noqa: F401
from ._lib import LIB_PATH, S2GError, load  # noqa: F401

__all__ = ["api", "load", "LIB_PATH", "S2GError"]

"""tapkee_gb300 -- GB300 (sm_103a) local-neighborhood operator for Tapkee's
KLLE / KLTSA methods: brute-force kNN, LLE weights, LTSA tangent bases and the
alignment matrix M in CSR, behind a C ABI (include/tapkee_gb300.h).
"""
from . import datasets  # noqa: F401
from ._capi import library_path  # noqa: F401
from .api import (  # noqa: F401
    CancelledError,
    Context,
    DeviceError,
    EigendecompositionError,
    LocalOperator,
    MissedParameterError,
    MultipleParameterError,
    NoDataError,
    NotEnoughMemoryError,
    ParametersInitializedState,
    TapkeeError,
    TapkeeOutput,
    UnsupportedMethodError,
    WrongParameterError,
    default_context,
    embed,
    smallest_eigenvectors,
    with_,
)

__version__ = "0.1.0"

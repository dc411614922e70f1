"""GB300-native rawspec spectrometer core.

The compute path is the native library rawspec_gb300/lib/librawspec.so
(hand-written sm_103a CUDA behind the C interface of include/rawspec.h);
`rawspec_gb300.api` is its ctypes mirror.
"""
from .api import (  # noqa: F401
    MAX_OUTPUTS,
    RAWSPEC_FORWARD_FFT,
    RAWSPEC_INVERSE_FFT,
    RawspecContext,
    Spectrometer,
    load_library,
)

__all__ = ["MAX_OUTPUTS", "RAWSPEC_FORWARD_FFT", "RAWSPEC_INVERSE_FFT", "RawspecContext", "Spectrometer",
           "load_library"]

"""GB300 (sm_103a) implementation of GenPK's power-spectrum hot path.

CIC deposit -> FP32 r2c FFT (own z, y and x passes for power-of-two grids of
64-512 cells per side, cuFFT otherwise) -> fused CIC deconvolution + log-k
shell binning, plus the adjoint of a P(k) loss, behind the C ABI in
include/genpk_gb300.h.  See genpk_gb300.api for the Python mirror.
"""
from .api import (Batch, Context, GenPKError, fieldize, geometry, invwindow,  # noqa: F401
                  powerspectrum)

__all__ = ["Batch", "Context", "GenPKError", "fieldize", "geometry", "invwindow",
           "powerspectrum"]

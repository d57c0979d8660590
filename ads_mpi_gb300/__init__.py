"""GB300 implementation of the IGA-ADS explicit time step (macwozni/ADS_MPI).

The CUDA kernels and the C-ABI live in ``csrc/`` and are built into
``libadsgpu.so`` by ``build.py``; ``ads.ADS`` mirrors the reference's
initialize / Step / Cleanup over that C-ABI.
"""
from .ads import (ADS, ADSError, FORM_HEAT, FORM_OIL, FORM_PROJECT, PREC_FP64, PREC_MIXED, PREC_MIXED_FAST,  # noqa: F401
                  REORDER_FOR_X, REORDER_FOR_Y, REORDER_FOR_Z, axis_setup, fma_peak, load, lib_path, write_vti)

"""GB300-native multi-pass PIV (drop-in for openpiv-python-gpu's PIV path).

Modules mirror the reference package: ``gpu_process`` (piv_gpu, PIVGPU),
``gpu_validation`` (ValidationGPU, ReplacementGPU), ``gpu_smoothn``
(SmoothnGPU). The compute runs in libpiv_gb300.so (hand-written sm_103a CUDA).
"""

import numpy as np

# Default data types (the reference's openpiv_gpu/__init__.py:1-5).
DTYPE_i = np.int64
DTYPE_f = np.float64
DTYPE_c = np.complex128

"""dtcf_gb300 -- GB300-native node-local contraction path for DTCF-style
coupled-cluster workloads.

The product is the CUDA library ``libgbx.so`` (sources in ``csrc/``, C ABI in
``include/gbx.h``).  This package loads it with ctypes and mirrors the
reference's leaf interface in Python for tests and drivers.  There is no CPU
fallback: importing ``lib()`` fails loudly when the library is missing.
"""
from ._lib import lib, check, GbxError, LIB_PATH  # noqa: F401
from .leaves import (  # noqa: F401
    transpose, transpose_blocks, dltc_transpose, local_contraction, dltc_compute,
    create_big_matrix, create_big_matrix_nl, revert_big_matrix, grouped_gemm_f64, split_gemm,
)

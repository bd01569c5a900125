"""tbsla_gb300: GB300-native (sm_103a) SpMV / a_axpx_ / PageRank path of TBSLA.

The product is the shared library ``libtbsla_gb300.so`` (CUDA kernels, the
C ABI of include/tbsla_gb300.h, the drop-in ``tbsla::cpp::Matrix*`` classes
and the reference's ``C_CPP_*`` ABI).  This package builds it
(:mod:`tbsla_gb300.build`) and binds its C ABI for Python callers
(:mod:`tbsla_gb300.capi`, which loads the library on first use).
"""
from . import build, capi  # noqa: F401

__all__ = ["build", "capi"]

"""GB300 (sm_103a) implementation of the filter-diagonalisation path of the
semi-empirical pseudopotential method (the reference's filter/ program).

The work happens in libsep_gb300.so (CUDA kernels + C ABI, include/sep_gb300.h);
this package is a thin ctypes binding over it plus synthetic-input helpers.
Nothing here computes on the CPU in place of the library: if the library is
missing, every call raises.
"""
from .binding import (  # noqa: F401
    Batch,
    Context,
    SepError,
    coefficients,
    device_count,
    filter_chunk_plan,
    form_factor_backward,
    form_factor_table,
    hermitian_lowest,
    ksqr,
    lib,
    start_states,
)

__all__ = ["Batch", "Context", "SepError", "coefficients", "device_count", "filter_chunk_plan",
           "form_factor_backward", "form_factor_table",
           "hermitian_lowest", "ksqr",
           "lib", "start_states"]

"""GB300-native (sm_103a) state-vector backend for QCS.

The product is the shared library ``libqcs_gb300.so`` (CUDA kernels, the C ABI
of ``include/qcs_cuda.h`` and the public QCS API of ``include/qcs.h``); this
package holds its sources, its build script and thin ctypes bindings.
"""
from . import workloads  # noqa: F401

__all__ = ["workloads", "capi", "build"]

"""GB300-native type-1/type-2 NUFFT library with the cuFINUFFT v1.3 interface.

The compute path is ``lib/libcufinufft.so`` (hand-written sm_103a kernels plus
cuFFT), reached through the C ABI in ``include/cufinufft.h``.  This package
holds its build script and the ctypes/Python interface that mirrors the
reference's ``cufinufft`` Python package.  The library is loaded on first use
of ``cufinufft`` (so ``cufinufft_gb300.build`` can run before it exists).
"""

__all__ = ["cufinufft", "cufinufft_batch"]


def __getattr__(name):
    if name in ("cufinufft", "cufinufft_batch"):
        from cufinufft_gb300 import _interface
        cls = getattr(_interface, name)
        globals()[name] = cls
        return cls
    raise AttributeError(name)

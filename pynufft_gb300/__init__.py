"""pynufft_gb300: PyNUFFT's min-max NUFFT on one GB300 (sm_103a).

``NUFFT`` is a drop-in for the reference ``pynufft.NUFFT`` (plan / forward /
adjoint / selfadjoint / solve and the six stage methods); the transforms run
as hand-written CUDA kernels plus cuFFT through the C ABI of
``libpynufft_gb300.so`` (include/pynufft_gb300.h).
"""
from .nufft import NUFFT

__version__ = '0.1.0'
__all__ = ['NUFFT']

"""ctypes binding of libpynufft_gb300.so (the C ABI in include/pynufft_gb300.h).

The shared library is built in-tree by ``pynufft_gb300.build``.  There is no
CPU fallback: if the library is missing or fails to load, importing the
operator raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int64, c_void_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libpynufft_gb300.so')

NUFFT_OK = 0
NUFFT_EINVAL = 1
NUFFT_EOM_NONFINITE = 2
NUFFT_ENOMEM = 3
NUFFT_ECUDA = 4
NUFFT_ECUFFT = 5
NUFFT_ENOPOINTS = 6
NUFFT_ECG_BREAKDOWN = 7
NUFFT_EUNSUPPORTED = 8
NUFFT_ETIMEOUT = 9
NUFFT_FLAG_DETERMINISTIC = 1
NUFFT_FLAG_OWN_FFT = 2
NUFFT_FLAG_CUFFT = 4
NUFFT_FFT_CUFFT, NUFFT_FFT_CUFFT_PRUNED, NUFFT_FFT_OWN_PRUNED, NUFFT_FFT_OWN_COILS = 0, 1, 2, 3
NUFFT_K2Y_ZTEAM, NUFFT_K2Y_POINT, NUFFT_K2Y_TILE, NUFFT_K2Y_TILE_POINT = 1, 2, 3, 4
NUFFT_Y2K_ZTEAM, NUFFT_Y2K_POINT, NUFFT_Y2K_GLOBAL = 1, 2, 3

# every symbol the header declares, with (restype, argtypes)
SIGNATURES = {
    'nufft_last_error': (c_char_p, []),
    'nufft_version': (c_char_p, []),
    'nufft_axis_params': (c_int, [c_int, c_int, c_int, POINTER(c_float), c_int, POINTER(c_float),
                                  POINTER(c_int), POINTER(c_double), POINTER(c_double)]),
    'nufft_plan_set_alpha': (c_int, [c_void_p, c_int, POINTER(c_float), c_int]),
    'nufft_plan_create': (c_int, [c_int, POINTER(c_int), POINTER(c_int), POINTER(c_int), c_int,
                                  c_int, c_int, POINTER(c_void_p)]),
    'nufft_set_points': (c_int, [c_void_p, POINTER(c_int64), c_void_p, c_int, c_void_p]),
    'nufft_plan_destroy': (c_int, [c_void_p]),
    'nufft_plan_set_bins': (c_int, [c_void_p, POINTER(c_int), c_int]),
    'nufft_plan_info': (c_int, [c_void_p, POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]),
    'nufft_plan_transform_kind': (c_int, [c_void_p, POINTER(c_int)]),
    'nufft_plan_set_methods': (c_int, [c_void_p, c_int, c_int]),
    'nufft_x2xx': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_xx2k': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_k2y': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_y2k': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_k2xx': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_xx2x': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_forward': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_adjoint': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_selfadjoint': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_k2y2k': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_solve_cg': (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_double, c_double,
                               POINTER(c_int), c_void_p]),
    'nufft_solve_l1tvols': (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_double, c_void_p]),
    'nufft_plan_check': (c_int, [c_void_p, c_void_p]),
    'nufft_mapped_pointer': (c_int, [c_void_p, POINTER(c_void_p)]),
    'nufft_selftest_bounded_wait': (c_int, [c_int, POINTER(c_int)]),
    'nufft_plan_kernel_timing': (c_int, [c_void_p, c_int]),
    'nufft_plan_kernel_times': (c_int, [c_void_p, POINTER(c_double), POINTER(c_int),
                                        POINTER(c_double), POINTER(c_int)]),
    'nufft_forward_dom': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_set_sense': (c_int, [c_void_p, c_void_p, c_int, c_void_p]),
    'nufft_y2k_exact_static': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_forward_one2many': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    'nufft_adjoint_many2one': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
}

_lib = None


class NufftError(RuntimeError):
    """A status code other than NUFFT_OK returned by the C ABI."""

    def __init__(self, code: int, msg: str):
        super().__init__(f'[{code}] {msg}')
        self.code = code


def load(path: str = LIB_PATH):
    """Load the shared library (once) and attach the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f'{path} is missing: build it with `python -m pynufft_gb300.build` '
            '(pynufft_gb300 has no CPU fallback)')
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int, what: str = ''):
    if code != NUFFT_OK:
        msg = load().nufft_last_error().decode(errors='replace')
        if code == NUFFT_EINVAL:
            raise ValueError(f'{what}: {msg}')
        if code == NUFFT_EOM_NONFINITE:
            raise ValueError(f'{what}: {msg}')
        if code == NUFFT_EUNSUPPORTED:
            raise NotImplementedError(f'{what}: {msg}')
        if code == NUFFT_ENOMEM:
            raise MemoryError(f'{what}: {msg}')
        raise NufftError(code, f'{what}: {msg}')


def int_array(vals):
    arr = (c_int * 3)(*([int(v) for v in vals] + [1] * (3 - len(vals))))
    return arr

"""C ABI checks that need no GPU: the library loads, exports every function
include/pynufft_gb300.h declares, and its host-side plan numerics
(nufft_axis_params) agree with the reference's fixtures."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import PLAN_CASES, ROOT, load_golden

HEADER = os.path.join(ROOT, 'include', 'pynufft_gb300.h')


def _declared():
    src = open(HEADER).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(nufft_[a-z0-9_]+)\s*\(', src)))


def test_library_exports_every_declared_symbol():
    from pynufft_gb300 import _lib
    lib = _lib.load()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    # the Python binding attaches a signature to each of them
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)
    assert b'sm_103a' in lib.nufft_version()


def test_python_constants_match_the_header():
    """Every NUFFT_* integer constant the Python binding mirrors has the
    header's value (status codes, plan flags, method and transform kinds)."""
    from pynufft_gb300 import _lib
    src = re.sub(r'/\*.*?\*/', '', open(HEADER).read(), flags=re.S)
    defs = {m.group(1): int(m.group(2))
            for m in re.finditer(r'#define\s+(NUFFT_[A-Z0-9_]+)\s+(-?\d+)', src)}
    mirrored = [n for n in dir(_lib) if n.startswith('NUFFT_') and isinstance(getattr(_lib, n), int)]
    assert len(mirrored) >= 15
    for n in mirrored:
        assert n in defs, n
        assert getattr(_lib, n) == defs[n], (n, getattr(_lib, n), defs[n])


def _axis(N, J, K, alpha_in=None):
    from pynufft_gb300 import _lib
    lib = _lib.load()
    a = (ctypes.c_float * 16)()
    L = ctypes.c_int()
    sn = (ctypes.c_double * N)()
    T = (ctypes.c_double * (J * J))()
    ain, Lin = None, 0
    if alpha_in is not None:
        ain = (ctypes.c_float * 16)(*([float(v) for v in alpha_in] + [0.0] * (16 - len(alpha_in))))
        Lin = len(alpha_in) - 1
    _lib.check(lib.nufft_axis_params(N, J, K, ain, Lin, a, ctypes.byref(L), sn, T))
    return (np.frombuffer(a, np.float32)[:L.value + 1].copy(), np.frombuffer(sn).copy(),
            np.frombuffer(T).reshape(J, J).copy())


@pytest.mark.parametrize('case', PLAN_CASES)
def test_axis_params_match_reference(case):
    """Given the reference's coefficients (which the Python plan layer
    reproduces with the same complex64 solve), the C++ host numerics derive the
    reference's sn and T."""
    from pynufft_gb300.plan_params import alpha_fit
    g = load_golden(case)
    Nd, Kd, Jd = g['Nd'], g['Kd'], g['Jd']
    sn_full = np.ones(())
    for d in range(len(Nd)):
        ref_a = g[f'alpha{d}']
        a_py, L = alpha_fit(int(Nd[d]), int(Jd[d]), int(Kd[d]))
        assert np.array_equal(a_py, ref_a)
        a, sn, T = _axis(int(Nd[d]), int(Jd[d]), int(Kd[d]), ref_a)
        assert np.array_equal(a, ref_a)
        np.testing.assert_allclose(T, g[f'T{d}'], rtol=1e-9, atol=1e-9 * np.abs(g[f'T{d}']).max())
        shp = [1] * len(Nd)
        shp[d] = int(Nd[d])
        sn_full = sn_full * sn.reshape(shp)
    np.testing.assert_allclose(sn_full, g['sn'].real, rtol=2e-6)


def test_axis_params_rejects_bad_sizes():
    from pynufft_gb300 import _lib
    lib = _lib.load()
    a = (ctypes.c_float * 16)()
    L = ctypes.c_int()
    sn = (ctypes.c_double * 8)()
    T = (ctypes.c_double * 400)()
    assert lib.nufft_axis_params(8, 17, 16, None, 0, a, ctypes.byref(L), sn, T) == _lib.NUFFT_EINVAL
    assert lib.nufft_axis_params(32, 6, 16, None, 0, a, ctypes.byref(L), sn, T) == _lib.NUFFT_EINVAL
    assert b'J' in lib.nufft_last_error()


def test_plan_argument_errors_match_reference():
    """helper.plan raises TypeError for non-tuple shapes and KeyError for
    mismatched lengths (src/_helper/helper.py:644-654)."""
    from pynufft_gb300.nufft import NUFFT
    with pytest.raises(TypeError):
        NUFFT._check_shapes([256, 256], (512, 512), (6, 6))
    with pytest.raises(TypeError):
        NUFFT._check_shapes((256, 256), [512, 512], (6, 6))
    with pytest.raises(TypeError):
        NUFFT._check_shapes((256, 256), (512, 512), 6)
    with pytest.raises(KeyError):
        NUFFT._check_shapes((256, 256), (512, 512), (6,))


def test_null_plan_is_rejected_without_gpu():
    from pynufft_gb300 import _lib
    lib = _lib.load()
    assert lib.nufft_forward(None, None, None, None) == _lib.NUFFT_EINVAL
    assert lib.nufft_plan_destroy(None) == _lib.NUFFT_OK


@pytest.mark.parametrize('case', PLAN_CASES)
def test_axis_params_own_fit_close_to_reference(case):
    """Without the reference's coefficients the C++ fit (truncated SVD at the
    float32 cutoff) gives an interpolator whose scaling factor stays within
    1e-5 relative of the reference's."""
    g = load_golden(case)
    Nd, Kd, Jd = g['Nd'], g['Kd'], g['Jd']
    sn_full = np.ones(())
    for d in range(len(Nd)):
        a, sn, T = _axis(int(Nd[d]), int(Jd[d]), int(Kd[d]))
        shp = [1] * len(Nd)
        shp[d] = int(Nd[d])
        sn_full = sn_full * sn.reshape(shp)
    assert np.linalg.norm(sn_full - g['sn'].real) / np.linalg.norm(g['sn'].real) < 1e-5

"""Plan-time cosine-series coefficients of the Kaiser-Bessel scaling fit.

The reference fits 1/KB_ft with an (L+1)-term cosine series by a complex64
least-squares solve, ``numpy.linalg.lstsq(X, b, rcond=-1)``
(src/_helper/helper.py:910-958).  Its basis is ill-conditioned (cond ~1e10),
so the float32 rank cutoff of that solve, not its arithmetic, decides the
coefficients; repeating the same complex64 solve here reproduces them exactly
and hence the reference's interpolator.  This is O(N * L) host work per
axis, once per plan; all per-point work runs on the GPU.
"""
from __future__ import annotations

import numpy as np
import scipy.special

_KB_BEST_RATIO = {2: 2.5, 3: 2.27, 4: 2.31, 5: 2.34, 6: 2.32, 7: 2.32, 8: 2.35,
                  9: 2.34, 10: 2.34, 11: 2.35, 12: 2.34, 13: 2.35, 14: 2.35,
                  15: 2.35, 16: 2.33}


def kb_shape(J: int, K_over_N: float) -> float:
    """Kaiser-Bessel shape (src/_helper/helper.py:961-997)."""
    if K_over_N != 2:
        return 2.34 * J
    if J in _KB_BEST_RATIO:
        return J * _KB_BEST_RATIO[J]
    keys = np.array(sorted(_KB_BEST_RATIO))
    return J * _KB_BEST_RATIO[int(keys[np.argmin(np.abs(keys - J))])]


def kb_ft(u, J: int, alpha: float):
    """J sin(z)/z / I0(alpha), z^2 = (pi J u)^2 - alpha^2: the m = 0, d = 1
    Kaiser-Bessel transform of src/_helper/helper.py:1000-1012."""
    w = (np.pi * J * np.asarray(u, dtype=np.float64)) ** 2 - alpha ** 2
    z = np.sqrt(np.abs(w))
    with np.errstate(invalid='ignore', divide='ignore'):
        s = np.where(w > 0, np.sin(z) / z, np.where(w < 0, np.sinh(z) / z, 1.0))
    return J * s / scipy.special.iv(0, alpha)


def alpha_fit(N: int, J: int, K: int):
    """-> (alpha float32[L+1], L) exactly as the reference's complex64 fit."""
    L = 13 if N > 40 else int(np.ceil(N / 3))
    nlist = np.arange(N) * 1.0 - (N - 1.0) / 2.0
    if J > 1:
        target = 1.0 / kb_ft(nlist / K, J, kb_shape(J, K / N))
    else:
        target = np.ones(N)
    X = np.cos(np.outer(2 * np.pi / K * nlist, np.arange(L + 1))).astype(np.complex64)
    b = np.conj(target).reshape(N, 1).astype(np.complex64)
    coef = np.linalg.lstsq(np.nan_to_num(X), np.nan_to_num(b), rcond=-1)[0][:, 0]
    alpha = coef.copy()
    if J > 1:
        alpha[1:] = alpha[1:] / 2.0
    else:
        alpha[0] = 1.0
        alpha[1:] = 0.0
    return np.real(alpha).astype(np.float32), L

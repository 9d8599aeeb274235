"""Oracle: a CPU restatement of PyNUFFT's numpy min-max NUFFT path.

TEST INFRASTRUCTURE ONLY.  This module is the checker for the CUDA path: the
parity tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs import
it; the product package never does.

It restates, in numpy/scipy, the algorithm of the reference package
(pynufft 2025.2.1); every function names the reference lines it follows:

* plan numerics                 src/_helper/helper.py:620-802
* Kaiser-Bessel fit / scaling   src/_helper/helper.py:910-1050
* min-max interpolator          src/_helper/helper.py:606-618, 1060-1117, 148-210
* CSR interpolation matrix      src/_helper/helper.py:285-311, 449-480
* the six stages + solve('cg')  nufft/_nufft_class_methods_cpu.py:27-362,
                                linalg/solve_cpu.py:256-288
* exact NUDFT                   linalg/nudft_cpu.py:27-41, 92-103

Dtypes follow the reference on numpy >= 2: the scaling factor is stored as
complex64, the oversampled FFT runs in complex64, the CSR holds complex128, so
``k2y``/``y2k`` return complex128 and ``k2xx`` runs its inverse FFT at the
precision of its input before cropping into complex64.

The oracle is pinned against outputs of the reference itself
(``tests/golden/make_golden.py`` imports the reference, writes the fixtures,
and ``tests/test_oracle_golden.py`` checks this module against them) and
against the exact-NDFT known-answer vectors shipped with the reference
(``tests/tmp2d_{1,2,3}_.mat``, converted to ``tests/golden/ndft_known_answer.npz``).
"""
from __future__ import annotations

import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.linalg
import scipy.sparse
import scipy.special

# Kaiser-Bessel "best" alpha/J ratios for K/N == 2 (src/_helper/helper.py:972-987).
_KB_BEST_RATIO = {2: 2.5, 3: 2.27, 4: 2.31, 5: 2.34, 6: 2.32, 7: 2.32, 8: 2.35,
                  9: 2.34, 10: 2.34, 11: 2.35, 12: 2.34, 13: 2.35, 14: 2.35,
                  15: 2.35, 16: 2.33}


# --------------------------------------------------------------------------
# plan-time numerics
# --------------------------------------------------------------------------
def kb_shape(J: int, K_over_N: float) -> float:
    """Kaiser-Bessel shape parameter (src/_helper/helper.py:961-997)."""
    if K_over_N != 2:
        return 2.34 * J
    if J in _KB_BEST_RATIO:
        return J * _KB_BEST_RATIO[J]
    keys = np.array(sorted(_KB_BEST_RATIO))
    return J * _KB_BEST_RATIO[int(keys[np.argmin(np.abs(keys - J))])]


def kb_ft(u, J: int, alpha: float):
    """Fourier transform of the KB window, order m=0, d=1
    (src/_helper/helper.py:1000-1012)."""
    u = np.asarray(u) * (1.0 + 0.0j)
    z = np.sqrt((2 * np.pi * (J / 2) * u) ** 2.0 - alpha ** 2.0)
    nu = 0.5
    y = ((2 * np.pi) ** 0.5) * (J / 2) / scipy.special.iv(0, alpha) \
        * scipy.special.jv(nu, z) / (z ** nu)
    return np.real(y)


def alpha_beta_fit(N: int, J: int, K: int):
    """Cosine-series fit of 1/KB_ft (src/_helper/helper.py:910-958).

    Returns ``(alpha, beta)``; ``alpha`` is float32 of length L+1 because the
    reference solves the least-squares problem in complex64.
    """
    beta = 1
    Nmid = (N - 1.0) / 2.0
    L = 13 if N > 40 else int(np.ceil(N / 3))
    nlist = np.arange(N) * 1.0 - Nmid
    if J > 1:
        sn_kaiser = 1.0 / kb_ft(nlist / K, J, kb_shape(J, K / N))
    else:
        sn_kaiser = np.ones(N)
    gam = 2 * np.pi / K
    X = np.cos(np.outer(beta * gam * nlist, np.arange(L + 1)))
    X = np.asarray(X, dtype=np.complex64)
    rhs = np.asarray(np.conj(sn_kaiser).reshape(N, 1), dtype=np.complex64)
    coef = np.linalg.lstsq(np.nan_to_num(X), np.nan_to_num(rhs), rcond=-1)[0]
    alpha = coef[:, 0].copy()
    if J > 1:
        alpha[1:] = alpha[1:] / 2.0
    else:
        alpha[0] = 1.0
        alpha[1:] = 0.0
    return np.real(alpha).astype(np.float32), beta


def scale_axis(N: int, K: int, alpha, beta) -> np.ndarray:
    """Per-axis image-domain scaling factor, real part
    (src/_helper/helper.py:1015-1036, 558-584, 780)."""
    alpha = np.asarray(alpha)
    L = alpha.size - 1
    n = np.arange(N, dtype=np.float64)
    Nmid = (N - 1) / 2.0
    sn = np.zeros(N, dtype=np.complex128)
    ph = 1j * (2 * np.pi / K) * (n - Nmid) * beta
    for l1 in range(-L, L + 1):
        sn = sn + alpha[abs(l1)].astype(np.float64) * np.exp(ph * l1)
    return sn.real


def minmax_T(N: int, J: int, K: int, alpha, beta) -> np.ndarray:
    """T = pinv(CSSC), the J x J min-max normal matrix
    (src/_helper/helper.py:1060-1083).  alpha products are formed in float32
    first, as the reference does with its float32 coefficient array."""
    alpha = np.asarray(alpha, dtype=np.float32)
    L = alpha.size - 1
    j1, j2 = np.mgrid[1:J + 1, 1:J + 1]
    overlap = (j2 - j1).astype(np.float64)
    cssc = np.zeros((J, J))
    for l1 in range(-L, L + 1):
        for l2 in range(-L, L + 1):
            a12 = np.float32(alpha[abs(l1)] * alpha[abs(l2)])
            cssc = cssc + np.float64(a12) * np.sinc((overlap + beta * (l1 - l2)) / (K / N))
    return scipy.linalg.pinv(cssc)


def minmax_axis(om_d, N: int, J: int, K: int, alpha, beta, T=None):
    """Per-axis interpolation coefficients and grid indices.

    Follows min_max/nufft_r/OMEGA_u/OMEGA_k/nufft_offset
    (src/_helper/helper.py:606-618, 1086-1117, 148-210, 900-907).
    Returns ``ud`` (M x J complex128, already conjugated as in the reference's
    CSR) and ``kd`` (M x J int64 grid indices along this axis, mod K).
    """
    om_d = np.asarray(om_d, dtype=np.float64).ravel()
    if T is None:
        T = minmax_T(N, J, K, alpha, beta)
    alpha = np.asarray(alpha, dtype=np.float32)
    L = alpha.size - 1
    gam = 2.0 * np.pi / K
    koff = np.floor(om_d / gam - J / 2.0)
    dk = om_d / gam - koff
    arg = np.add.outer(-np.arange(1, J + 1) * 1.0, dk)            # J x M
    r = np.zeros(arg.shape)
    for l1 in range(-L, L + 1):
        r = r + np.float64(alpha[abs(l1)]) * np.sinc((arg + l1 * beta) / (K / N))
    c = T.dot(r)
    u = np.exp(1j * gam * (N - 1.0) / 2.0 * arg) * c * np.exp(-1j * om_d * N / 2.0)
    ud = u.T.conj()
    kd = np.mod(np.add.outer(np.arange(1, J + 1), koff.astype(np.int64)), K).T
    return ud, kd


def interp_csr(om, Nd, Kd, Jd, params=None):
    """The M x prod(Kd) complex128 interpolation matrix
    (src/_helper/helper.py:449-480 Khatri-Rao, 285-311 create_csr).
    Row m, entry (j_0..j_{d-1}) with the last axis fastest."""
    om = np.asarray(om, dtype=np.float64)
    M, d = om.shape
    if params is None:
        params = [alpha_beta_fit(Nd[i], Jd[i], Kd[i]) for i in range(d)]
    uu = None
    kk = None
    for i in range(d):
        a, b = params[i]
        ud, kd = minmax_axis(om[:, i], Nd[i], Jd[i], Kd[i], a, b)
        stride = int(np.prod(Kd[i + 1:])) if i < d - 1 else 1
        kd = kd * stride
        if uu is None:
            uu, kk = ud, kd
        else:
            uu = np.einsum('mi,mj->mij', uu, ud).reshape(M, -1)
            kk = (kk[:, :, None] + kd[:, None, :]).reshape(M, -1)
    P = int(np.prod(Jd))
    indptr = np.arange(0, (M + 1) * P, P, dtype=np.int64)
    return scipy.sparse.csr_matrix((uu.ravel(), kk.ravel(), indptr),
                                   shape=(M, int(np.prod(Kd))))


def check_plan_args(Nd, Kd, Jd):
    """Argument checks of helper.plan (src/_helper/helper.py:644-654)."""
    if type(Nd) != tuple:
        raise TypeError('Nd must be tuple, e.g. (256, 256)')
    if type(Kd) != tuple:
        raise TypeError('Kd must be tuple, e.g. (512, 512)')
    if type(Jd) != tuple:
        raise TypeError('Jd must be tuple, e.g. (6, 6)')
    if len(Nd) != len(Kd) or len(Nd) != len(Jd):
        raise KeyError('Nd, Kd, Jd must be in the same length, e.g. '
                       'Nd=(256,256),Kd=(512,512),Jd=(6,6)')


# --------------------------------------------------------------------------
# the operator
# --------------------------------------------------------------------------
class OracleNUFFT:
    """numpy restatement of the reference ``NUFFT`` CPU backend
    (nufft/_nufft_class_methods_cpu.py:27-362).

    ``batch`` follows the deprecated device class (linalg/nufft_hsa.py:203-228):
    x is Nd+(B,), k is Kd+(B,), y is (M,B); each coil is an independent
    single-coil transform sharing the plan.
    """

    def plan(self, om, Nd, Kd, Jd, batch=None, threads=1, build_threads=None):
        """``threads``: host threads of the sparse products and FFTs (1 = the
        reference's single-threaded numpy/scipy calls).  ``build_threads``
        (default ``threads``): threads that build the CSR matrices, on row
        chunks whose stacked result is identical to the one-piece build."""
        check_plan_args(Nd, Kd, Jd)
        self.Nd, self.Kd, self.Jd = Nd, Kd, Jd
        self.ndims = len(Nd)
        self.batch = batch
        self.threads = int(threads)
        om = np.asarray(om, dtype=np.float64)
        self.M = om.shape[0]
        self.params = [alpha_beta_fit(Nd[i], Jd[i], Kd[i]) for i in range(self.ndims)]
        self.snd = [scale_axis(Nd[i], Kd[i], *self.params[i]) for i in range(self.ndims)]
        sn = np.ones(())
        for i, s in enumerate(self.snd):
            shp = [1] * self.ndims
            shp[i] = s.size
            sn = sn * s.reshape(shp)
        self.sn = np.asarray(sn.real.astype(np.complex64), order='C')
        nb = int(build_threads or self.threads)
        if nb <= 1 or self.M < 2 * 65536:
            self.sp = interp_csr(om, Nd, Kd, Jd, self.params)
            self.spH = self.sp.getH().tocsr()
        else:
            edges = np.linspace(0, self.M, 4 * nb + 1).astype(np.int64)
            spans = [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]

            def part(ab):
                a, b = ab
                sp = interp_csr(om[a:b], Nd, Kd, Jd, self.params)
                return sp, sp.getH().tocsr()
            with ThreadPoolExecutor(nb) as ex:
                parts = list(ex.map(part, spans))
            self.sp = scipy.sparse.vstack([p[0] for p in parts], format='csr')
            self.spH = scipy.sparse.hstack([p[1] for p in parts], format='csr')
        self._row_chunks = None
        return 0

    # ---- helpers for the (optional) threaded sparse products -------------
    def _chunks(self, n):
        t = max(1, self.threads)
        edges = np.linspace(0, n, t + 1).astype(np.int64)
        return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]

    def _matvec(self, A, v):
        if self.threads <= 1:
            return A.dot(v)
        if self._row_chunks is None:
            self._row_chunks = {}
        key = id(A)
        if key not in self._row_chunks:
            self._row_chunks[key] = [(a, b, A[a:b]) for a, b in self._chunks(A.shape[0])]
        parts = self._row_chunks[key]
        out = np.empty(A.shape[0], dtype=np.result_type(A.dtype, v.dtype))

        def work(p):
            a, b, sub = p
            out[a:b] = sub.dot(v)
        with ThreadPoolExecutor(len(parts)) as ex:
            list(ex.map(work, parts))
        return out

    def _fftn(self, a, inverse=False):
        if self.threads <= 1:
            return np.fft.ifftn(a) if inverse else np.fft.fftn(a)
        import scipy.fft
        f = scipy.fft.ifftn if inverse else scipy.fft.fftn
        return f(a, workers=self.threads)

    # ---- single-coil stages (nufft/_nufft_class_methods_cpu.py) -----------
    def _x2xx1(self, x):              # :224-230
        return x * self.sn

    def _xx2k1(self, xx):             # :232-249 (+ preindex_copy, helper.py:830-881)
        out = np.zeros(self.Kd, dtype=np.complex64)
        out[tuple(slice(0, n) for n in self.Nd)] = xx
        return self._fftn(out)

    def _k2y1(self, k):               # :273-288
        return self._matvec(self.sp, np.reshape(k, (-1,)))

    def _y2k1(self, y):               # :290-314
        return np.reshape(self._matvec(self.spH, y), self.Kd)

    def _k2xx1(self, k):              # :316-329
        k = self._fftn(k, inverse=True)
        xx = np.zeros(self.Nd, dtype=np.complex64)
        xx[...] = k[tuple(slice(0, n) for n in self.Nd)]
        return xx

    # ---- batch-aware public stages ----------------------------------------
    def _per_coil(self, fn, a, lead_shape):
        if self.batch is None:
            return fn(a)
        outs = [fn(a[..., b]) for b in range(a.shape[-1])]
        return np.stack(outs, axis=-1)

    def x2xx(self, x):
        if self.batch is None:
            return self._x2xx1(x)
        return x * self.sn[..., None]

    def xx2x(self, xx):               # :346-351 (same multiply as x2xx)
        return self.x2xx(xx)

    def xx2k(self, xx):
        return self._per_coil(self._xx2k1, xx, self.Nd)

    def k2y(self, k):
        return self._per_coil(self._k2y1, k, self.Kd)

    def y2k(self, y):
        return self._per_coil(self._y2k1, y, (self.M,))

    def k2xx(self, k):
        return self._per_coil(self._k2xx1, k, self.Kd)

    def forward(self, x):             # :168-179
        return self.k2y(self.xx2k(self.x2xx(x)))

    def adjoint(self, y):             # :181-193
        return self.xx2x(self.k2xx(self.y2k(y)))

    def k2y2k(self, k):               # :353-362
        return self.y2k(self.k2y(k))

    def selfadjoint(self, x):         # :201-214
        return self.xx2x(self.k2xx(self.k2y2k(self.xx2k(self.x2xx(x)))))

    # ---- SENSE coil operators (linalg/nufft_cpu.py:177-203)
    def forward_one2many(self, x, maps):
        """forward(x[..., None] * maps): image Nd -> (M, B)."""
        return np.stack([self._k2y1(self._xx2k1(self._x2xx1(x * maps[..., b])))
                         for b in range(maps.shape[-1])], axis=-1)

    def adjoint_many2one(self, y, maps):
        """mean over coils of conj(maps) * adjoint(y)."""
        xs = [self._x2xx1(self._k2xx1(self._y2k1(y[:, b]))) * np.conj(maps[..., b])
              for b in range(maps.shape[-1])]
        return np.mean(np.stack(xs, axis=-1), axis=-1)

    def density_pipe(self, maxiter):
        """Pipe's density compensation weights (linalg/solve_cpu.py:165-183):
        W <- W / forward(adjoint(W)), W0 = 1, single coil."""
        W = np.ones(self.M, dtype=np.complex64)
        for _ in range(maxiter):
            E = self._k2y1(self._xx2k1(self._x2xx1(self._x2xx1(self._k2xx1(self._y2k1(W))))))
            W = W / E
        return W

    def l1tvols(self, y, maxiter, rho):
        """solve(y, 'L1TVOLS', maxiter, rho): split-Bregman L1-TV least squares
        (linalg/solve_cpu.py:42-163), mu = 1, lambda = rho, single coil, in the
        reference's complex64 / float32 arithmetic.  The k-space preconditioner
        is mu |xx2k(adjoint(1))| - lambda fftn(periodic Laplacian stencil)
        (_create_kspace_sampling_density :24-40, helper.create_laplacian_kernel
        src/_helper/helper.py:11-44); D_d x = x[n - e_d] - x[n] and its
        transpose v[n + e_d] - v[n] (cDiff with helper.indxmap_diff :46-70)."""
        nd = len(self.Nd)
        lmbd = rho * 1.0
        w = np.abs(self._xx2k1(self.adjoint(np.ones(self.M, np.complex64))))
        lap = np.zeros(self.Kd, np.complex64)
        lap[(0,) * nd] = -2.0 * nd
        for d in range(nd):
            for s in (1, -1):
                idx = [0] * nd
                idx[d] = s
                lap[tuple(idx)] = 1
        uker = w - lmbd * np.fft.fftn(lap)
        ahy = self.adjoint(y)
        x = np.zeros_like(ahy)
        ahyk = np.zeros_like(ahy)
        dd = [np.zeros(self.Nd, np.complex64) for _ in range(nd)]
        bb = [np.zeros(self.Nd, np.complex64) for _ in range(nd)]
        for _ in range(maxiter):
            rhs = ahyk.copy()
            for d in range(nd):
                v = dd[d] - bb[d]
                rhs += lmbd * (np.roll(v, -1, axis=d) - v)
            x = self._k2xx1((self._xx2k1(rhs) + 1e-7) / (uker + 1e-7))
            zz = [np.roll(x, 1, axis=d) - x for d in range(nd)]
            st = [zz[d] + bb[d] for d in range(nd)]
            s = np.zeros(self.Nd, np.float32)
            for d in range(nd):
                s = np.hypot(np.hypot(st[d].real, st[d].imag), s)
            s = s + np.float32(1e-5)
            th = 1.0 / lmbd
            r = (s > th) * (s - th) / s
            for d in range(nd):
                dd[d] = st[d] * r
                bb[d] += zz[d] - dd[d]
            ahyk = ahyk - (self.selfadjoint(x) - ahy)
        return x

    def solve(self, y, solver='cg', maxiter=None, rtol=1e-5, atol=0.0,
              return_info=False, solver_kw=None, operator_dtype=None):
        """solve(y, 'cg', maxiter): CG on the k-space normal operator spH.sp,
        x0 = 0, then k2xx(k) / sn (linalg/solve_cpu.py:256-288).  The CG
        recursion restates scipy.sparse.linalg.cg (scipy 1.18.1,
        sparse/linalg/_isolve/iterative.py) without a preconditioner."""
        if solver == 'dc':
            # linalg/solve_cpu.py:202-225: x = adjoint(W * y)
            W = self.density_pipe(maxiter)
            return self.adjoint(W * y if self.batch is None else W[:, None] * y)
        if solver in ('lsqr', 'lsmr'):
            # linalg/solve_cpu.py:226-251: scipy lsqr/lsmr on sp, then k2xx(k)/sn
            import scipy.sparse.linalg as sla
            fn = sla.lsqr if solver == 'lsqr' else sla.lsmr
            kw = dict(atol=atol, btol=atol) if solver == 'lsqr' else dict(atol=atol, btol=atol)
            k = fn(self.sp, np.asarray(y).ravel(), maxiter=maxiter, **kw)[0] \
                if solver == 'lsmr' else fn(self.sp, np.asarray(y).ravel(), iter_lim=maxiter, **kw)[0]
            xx = self._k2xx1(np.reshape(k, self.Kd))
            return xx / self.sn
        if solver in ('bicg', 'bicgstab', 'gmres', 'lgmres'):
            # linalg/solve_cpu.py:253-288: the scipy routine on the Hermitian
            # normal operator spH.sp (k2y2k), b = y2k(y), then k2xx(k) / sn
            import scipy.sparse.linalg as sla
            n = int(np.prod(self.Kd))

            def spHsp(v):
                return self._matvec(self.spH, self._matvec(self.sp, v))
            A = sla.LinearOperator((n, n), matvec=spHsp, rmatvec=spHsp, dtype=np.complex128)
            b = np.reshape(self._y2k1(y), (-1,))
            kw = dict(rtol=rtol, atol=atol, maxiter=maxiter, **(solver_kw or {}))
            k, info = getattr(sla, solver)(A, b, **kw)
            xx = self._k2xx1(np.reshape(k, self.Kd))
            return (xx / self.sn, info) if return_info else xx / self.sn
        if solver != 'cg':
            raise NotImplementedError(solver)

        def one(yc):
            b = np.reshape(self._y2k1(yc), (-1,))
            x, it = cg_restated(lambda v: self._matvec(self.spH, self._matvec(self.sp, v)),
                                b, maxiter=maxiter, rtol=rtol, atol=atol,
                                operator_dtype=operator_dtype)
            xx = self._k2xx1(np.reshape(x, self.Kd))
            return xx / self.sn, it

        if self.batch is None:
            x, it = one(y)
            return (x, it) if return_info else x
        outs = [one(y[:, b]) for b in range(y.shape[1])]
        x = np.stack([o[0] for o in outs], axis=-1)
        return (x, [o[1] for o in outs]) if return_info else x


class ChunkedOracleNUFFT(OracleNUFFT):
    """The reference numpy path planned on row chunks of ``om``, for point
    sets whose full CSR does not fit in host memory (a 3D J=6 plan holds
    216 complex128 entries per point, twice with ``spH``).

    Rows of the interpolation matrix are independent, so ``k2y`` is the
    concatenation of each chunk's ``sp . k`` and ``y2k`` the sum of each
    chunk's ``spH . y`` (nufft/_nufft_class_methods_cpu.py:273-314); the
    FFT and scaling stages are the unchunked ones.  A chunk's CSR is built
    when it is used and dropped afterwards.  ``k2y_rows`` evaluates only the
    selected rows (one CSR of those rows).
    """

    def plan(self, om, Nd, Kd, Jd, batch=None, threads=1, chunk=1_000_000):
        check_plan_args(Nd, Kd, Jd)
        self.Nd, self.Kd, self.Jd = Nd, Kd, Jd
        self.ndims = len(Nd)
        self.batch = batch
        self.threads = int(threads)
        self.om = np.asarray(om, dtype=np.float64)
        self.M = self.om.shape[0]
        self.chunk = int(chunk)
        self.params = [alpha_beta_fit(Nd[i], Jd[i], Kd[i]) for i in range(self.ndims)]
        self.snd = [scale_axis(Nd[i], Kd[i], *self.params[i]) for i in range(self.ndims)]
        sn = np.ones(())
        for i, s in enumerate(self.snd):
            shp = [1] * self.ndims
            shp[i] = s.size
            sn = sn * s.reshape(shp)
        self.sn = np.asarray(sn.real.astype(np.complex64), order='C')
        self._row_chunks = None
        return 0

    def _csr(self, a, b):
        return interp_csr(self.om[a:b], self.Nd, self.Kd, self.Jd, self.params)

    def _k2y1(self, k):
        kv = np.reshape(k, (-1,))
        out = np.empty(self.M, dtype=np.complex128)
        for a in range(0, self.M, self.chunk):
            b = min(self.M, a + self.chunk)
            out[a:b] = self._csr(a, b).dot(kv)
        return out

    def _y2k1(self, y):
        acc = np.zeros(int(np.prod(self.Kd)), dtype=np.complex128)
        for a in range(0, self.M, self.chunk):
            b = min(self.M, a + self.chunk)
            acc += self._csr(a, b).getH().dot(y[a:b])
        return np.reshape(acc, self.Kd)

    def k2y_rows(self, k, rows):
        """k2y at the selected rows only: (len(rows),) or (len(rows), B)."""
        rows = np.asarray(rows)
        sp = interp_csr(self.om[rows], self.Nd, self.Kd, self.Jd, self.params)
        if self.batch is None:
            return sp.dot(np.reshape(k, (-1,)))
        return np.stack([sp.dot(np.reshape(k[..., b], (-1,))) for b in range(k.shape[-1])], -1)

    def forward_rows(self, x, rows):
        """forward(x) at the selected rows: k = xx2k(x2xx(x)) on the full
        grid, then the interpolation rows."""
        return self.k2y_rows(self.xx2k(self.x2xx(x)), rows)


def cg_restated(matvec, b, maxiter=None, rtol=1e-5, atol=0.0, operator_dtype=None):
    """Conjugate gradients with scipy.sparse.linalg.cg's recursion and stopping
    rule (x0 = 0; stop when ||r|| < max(atol, rtol*||b||) at the top of an
    iteration).  Returns (x, iterations_run).

    ``operator_dtype`` (e.g. numpy.complex64) rounds the operator's input and
    output to that type, everything else staying complex128: the recursion
    as run with a single-precision operator.  Tests use it to measure how far
    any float32 operator's CG iterates drift from the complex128 ones."""
    b = np.asarray(b)
    bnrm2 = np.linalg.norm(b)
    tol = max(float(atol), float(rtol) * float(bnrm2))
    x = np.zeros_like(b)
    if bnrm2 == 0:
        return b, 0
    if maxiter is None:
        maxiter = b.size * 10
    r = b.copy()
    rho_prev = None
    p = None
    for it in range(maxiter):
        if np.linalg.norm(r) < tol:
            return x, it
        rho = np.vdot(r, r)
        if it > 0:
            p = r + (rho / rho_prev) * p
        else:
            p = r.copy()
        if operator_dtype is None:
            q = matvec(p)
        else:
            q = matvec(p.astype(operator_dtype).astype(b.dtype)).astype(operator_dtype).astype(b.dtype)
        alpha = rho / np.vdot(p, q)
        x = x + alpha * p
        r = r - alpha * q
        rho_prev = rho
    return x, maxiter


# --------------------------------------------------------------------------
# exact NUDFT on subsets (linalg/nudft_cpu.py:27-41, 92-103)
# --------------------------------------------------------------------------
def _centred_grid(Nd):
    return [np.arange(n, dtype=np.float64) - n / 2 for n in Nd]


def nudft_forward_rows(x, om, rows=None):
    """y_m = sum_n x_n exp(-i om_m . (n - N/2)) for the selected rows, FP64.

    Separable per axis: the innermost image axis is contracted for all rows by
    one matrix product, the others by per-row weighted sums, so memory is
    O(prod(Nd[:-1]) * rows) and the heavy step runs in BLAS."""
    x = np.asarray(x, dtype=np.complex128)
    om = np.asarray(om, dtype=np.float64)
    if rows is not None:
        om = om[np.asarray(rows)]
    Nd = x.shape
    nd = len(Nd)
    grids = _centred_grid(Nd)
    F = [np.exp(-1j * np.outer(om[:, d], grids[d])) for d in range(nd)]   # R x N_d
    out = np.empty(om.shape[0], dtype=np.complex128)
    step = 512
    for s in range(0, om.shape[0], step):
        e = min(om.shape[0], s + step)
        # (prod(Nd[:-1]), N_last) @ (N_last, R) -> rows last
        t = x.reshape(-1, Nd[-1]) @ F[-1][s:e].T
        for d in range(nd - 2, -1, -1):
            t = t.reshape(-1, Nd[d], e - s)
            t = np.einsum('anr,rn->ar', t, F[d][s:e])
        out[s:e] = t.reshape(e - s)
    return out


def nudft_adjoint_pixels(y, om, Nd, pixels, chunk=65536):
    """x_n = sum_m y_m exp(+i om_m . (n - N/2)) at the selected flat pixel
    indices (C order), FP64, unnormalised, summed over chunks of points.  The
    reference NUFFT adjoint equals this divided by prod(Kd).  y may carry a
    trailing coil axis (M, B); the result is then (pixels, B)."""
    y = np.asarray(y, dtype=np.complex128)
    om = np.asarray(om, dtype=np.float64)
    idx = np.unravel_index(np.asarray(pixels), Nd)
    cen = np.stack([idx[d] - Nd[d] / 2 for d in range(len(Nd))], 1)   # P x d
    out = np.zeros((len(pixels),) + y.shape[1:], dtype=np.complex128)
    for s in range(0, om.shape[0], chunk):
        e = min(om.shape[0], s + chunk)
        out += np.exp(1j * (cen @ om[s:e].T)) @ y[s:e]
    return out


def rel_l2(a, b) -> float:
    a = np.asarray(a).astype(np.complex128).ravel()
    b = np.asarray(b).astype(np.complex128).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))

"""Solvers other than 'cg' for ``NUFFT.solve`` (linalg/solve_cpu.py:185-288).

Every operator application is the GPU NUFFT (k2y / y2k / forward / adjoint
through the C ABI); the vectors stay on the device and the few scalars of
each iteration are read back to drive the recursion.

* 'dc'   Pipe's density compensation (linalg/solve_cpu.py:165-183, 202-225):
         W0 = 1, W <- W / forward(adjoint(W)) for maxiter rounds, then
         x = adjoint(W * y).
* 'lsqr' / 'lsmr'  min ||sp k - y|| over the oversampled grid k with the
         reference's operator pair (k2y, y2k) (linalg/solve_cpu.py:226-251),
         x = k2xx(k) / sn.  LSQR follows Paige & Saunders (ACM TOMS 8, 1982)
         and LSMR follows Fong & Saunders (SISC 33, 2011), with damp = 0 and
         the published stopping tests (atol, btol, conlim).
* 'bicg' / 'bicgstab' / 'gmres' / 'lgmres'  the Krylov solvers the reference
         runs on the Hermitian k-space normal operator spH.sp = k2y2k with
         b = y2k(y) (linalg/solve_cpu.py:253-288), then x = k2xx(k) / sn.
         The recursions, defaults (x0 = 0, rtol 1e-5, atol 0, gmres restart
         20, lgmres inner_m 30 / outer_k 3) and stopping tests are those of
         scipy.sparse.linalg 1.18, which the reference calls; the vectors are
         complex128 on the device, the operator is the complex64 GPU NUFFT,
         and the small Hessenberg / Givens algebra runs on the host.
"""
from __future__ import annotations

import math


def solve(nufft, y, solver, *args, maxiter=None, **kwargs):
    if solver in ('cgs', 'qmr', 'minres'):
        raise TypeError(solver + ' requires real symmetric matrix')
    if solver == 'dc':
        it = maxiter if maxiter is not None else (args[0] if args else kwargs.get('maxiter', 10))
        return density_compensated_adjoint(nufft, y, int(it))
    if solver in ('lsqr', 'lsmr'):
        iters = kwargs.pop('iter_lim', None) or maxiter or (args[0] if args else None)
        fn = lsqr if solver == 'lsqr' else lsmr
        return fn(nufft, y, iter_lim=iters, **kwargs)
    if solver in KRYLOV:
        return normal_krylov(nufft, y, solver, *args, maxiter=maxiter, **kwargs)
    raise NotImplementedError(f"solver {solver!r} is not available; use 'cg', 'dc', 'lsqr', "
                              "'lsmr', 'bicg', 'bicgstab', 'gmres', 'lgmres' or 'L1TVOLS'")


def _dev(nufft, a, kind):
    d, how = nufft._in(a, kind)
    return d, how


def pipe_density(nufft, maxiter: int):
    """Density compensation weights (M,) for the planned points (single coil)."""
    import torch
    if nufft.batch is not None:
        raise NotImplementedError("'dc' weights are computed on a single-coil plan")
    W = torch.ones(nufft.M, dtype=torch.complex64, device=nufft.device)
    for _ in range(maxiter):
        E = nufft.forward(nufft.adjoint(W))
        W = W / E
    return W


def density_compensated_adjoint(nufft, y, maxiter: int):
    d, how = _dev(nufft, y, 'y')
    W = pipe_density(nufft, maxiter)
    return nufft._out(nufft.adjoint(W * d), how)


def _norm(v):
    import torch
    return float(torch.linalg.vector_norm(v))


def _finish(nufft, k, how):
    xx = nufft.k2xx(k.reshape(nufft._shape('k')))
    import torch
    sn = torch.from_numpy(nufft.sn).to(nufft.device)
    if nufft.batch is not None:
        sn = sn[..., None]
    return nufft._out(xx / sn, how)


def lsqr(nufft, y, iter_lim=None, atol=1e-6, btol=1e-6, conlim=1e8, return_info=False):
    """LSQR on A = k2y (grid -> samples), A^H = y2k."""
    import torch
    if nufft.batch is not None or nufft.ninst > 1:
        raise NotImplementedError('lsqr runs on single-coil, single-instance plans')
    b, how = _dev(nufft, y, 'y')
    n = nufft.Kdprod
    iter_lim = 2 * n if iter_lim is None else int(iter_lim)
    A = lambda v: nufft.k2y(v.reshape(nufft.Kd))
    AH = lambda u: nufft.y2k(u).reshape(-1)
    x = torch.zeros(n, dtype=torch.complex64, device=nufft.device)
    u = b.clone()
    beta = bnorm = _norm(u)
    if beta == 0:
        return _finish(nufft, x, how)
    u = u / beta
    v = AH(u)
    alpha = _norm(v)
    if alpha > 0:
        v = v / alpha
    w = v.clone()
    rhobar, phibar = alpha, beta
    anorm = acond = ddnorm = xxnorm = res2 = 0.0
    z = 0.0
    cs2, sn2 = -1.0, 0.0
    ctol = 1.0 / conlim if conlim > 0 else 0.0
    itn = 0
    istop = 0
    if alpha * beta == 0:
        return _finish(nufft, x, how)
    while itn < iter_lim:
        itn += 1
        u = A(v) - alpha * u
        beta = _norm(u)
        if beta > 0:
            u = u / beta
            anorm = math.sqrt(anorm ** 2 + alpha ** 2 + beta ** 2)
            v = AH(u) - beta * v
            alpha = _norm(v)
            if alpha > 0:
                v = v / alpha
        rho = math.hypot(rhobar, beta)
        c, s = rhobar / rho, beta / rho
        theta = s * alpha
        rhobar = -c * alpha
        phi = c * phibar
        phibar = s * phibar
        t1, t2 = phi / rho, -theta / rho
        dk = w / rho
        x = x + t1 * w
        w = v + t2 * w
        ddnorm += _norm(dk) ** 2
        # estimate ||x|| and cond(A) for the stopping tests
        delta = sn2 * rho
        gambar = -cs2 * rho
        rhs = phi - delta * z
        zbar = rhs / gambar
        xnorm = math.sqrt(xxnorm + zbar ** 2)
        gamma = math.hypot(gambar, theta)
        cs2, sn2 = gambar / gamma, theta / gamma
        z = rhs / gamma
        xxnorm += z ** 2
        acond = anorm * math.sqrt(ddnorm)
        rnorm = phibar
        arnorm = alpha * abs(c) * phibar        # ||A^H r|| = alpha_{k+1} |c_k| phibar_{k+1}
        test1 = rnorm / bnorm
        test2 = arnorm / (anorm * rnorm) if anorm * rnorm > 0 else 0.0
        test3 = 1.0 / acond if acond > 0 else 0.0
        rtol = btol + atol * anorm * xnorm / bnorm
        if test3 <= ctol:
            istop = 3
        if test2 <= atol:
            istop = 2
        if test1 <= rtol:
            istop = 1
        if istop:
            break
    out = _finish(nufft, x, how)
    return (out, itn, istop) if return_info else out


def lsmr(nufft, y, iter_lim=None, atol=1e-6, btol=1e-6, conlim=1e8, return_info=False):
    """LSMR on A = k2y (grid -> samples), A^H = y2k (damp = 0)."""
    import torch
    if nufft.batch is not None or nufft.ninst > 1:
        raise NotImplementedError('lsmr runs on single-coil, single-instance plans')
    b, how = _dev(nufft, y, 'y')
    n = nufft.Kdprod
    iter_lim = min(M_or(nufft), n) if iter_lim is None else int(iter_lim)
    A = lambda v: nufft.k2y(v.reshape(nufft.Kd))
    AH = lambda u: nufft.y2k(u).reshape(-1)
    u = b.clone()
    normb = beta = _norm(u)
    x = torch.zeros(n, dtype=torch.complex64, device=nufft.device)
    if beta == 0:
        return _finish(nufft, x, how)
    u = u / beta
    v = AH(u)
    alpha = _norm(v)
    if alpha > 0:
        v = v / alpha
    itn = 0
    zetabar = alpha * beta
    alphabar = alpha
    rho = rhobar = cbar = 1.0
    sbar = 0.0
    h = v.clone()
    hbar = torch.zeros_like(x)
    # quantities for the norm estimates
    betadd = beta
    betad = 0.0
    rhodold = 1.0
    tautildeold = 0.0
    thetatilde = 0.0
    zeta = 0.0
    d = 0.0
    normA2 = alpha ** 2
    maxrbar, minrbar = 0.0, 1e100
    ctol = 1.0 / conlim if conlim > 0 else 0.0
    istop = 0
    if alpha * beta == 0:
        return _finish(nufft, x, how)
    while itn < iter_lim:
        itn += 1
        u = A(v) - alpha * u
        beta = _norm(u)
        if beta > 0:
            u = u / beta
            v = AH(u) - beta * v
            alpha = _norm(v)
            if alpha > 0:
                v = v / alpha
        chat, shat, alphahat = 1.0, 0.0, alphabar      # damp = 0
        rhoold = rho
        rho = math.hypot(alphahat, beta)
        c, s = alphahat / rho, beta / rho
        thetanew = s * alpha
        alphabar = c * alpha
        rhobarold = rhobar
        zetaold = zeta
        thetabar = sbar * rho
        rhotemp = cbar * rho
        rhobar = math.hypot(cbar * rho, thetanew)
        cbar, sbar = cbar * rho / rhobar, thetanew / rhobar
        zeta = cbar * zetabar
        zetabar = -sbar * zetabar
        hbar = h - (thetabar * rho / (rhoold * rhobarold)) * hbar
        x = x + (zeta / (rho * rhobar)) * hbar
        h = v - (thetanew / rho) * h
        # ||r|| estimate
        betaacute = chat * betadd
        betacheck = -shat * betadd
        betahat = c * betaacute
        betadd = -s * betaacute
        thetatildeold = thetatilde
        rhotildeold = math.hypot(rhodold, thetabar)
        ctildeold, stildeold = rhodold / rhotildeold, thetabar / rhotildeold
        thetatilde = stildeold * rhobar
        rhodold = ctildeold * rhobar
        betad = -stildeold * betad + ctildeold * betahat
        tautildeold = (zetaold - thetatildeold * tautildeold) / rhotildeold
        taud = (zeta - thetatilde * tautildeold) / rhodold
        d = d + betacheck ** 2
        normr = math.sqrt(d + (betad - taud) ** 2 + betadd ** 2)
        normA2 = normA2 + beta ** 2
        normA = math.sqrt(normA2)
        normA2 = normA2 + alpha ** 2
        maxrbar = max(maxrbar, rhobarold)
        if itn > 1:
            minrbar = min(minrbar, rhobarold)
        condA = max(maxrbar, rhotemp) / min(minrbar, rhotemp)
        normar = abs(zetabar)
        normx = _norm(x)
        test1 = normr / normb
        test2 = normar / (normA * normr) if normA * normr > 0 else float('inf')
        test3 = 1.0 / condA
        t1 = test1 / (1 + normA * normx / normb)
        rtol = btol + atol * normA * normx / normb
        if 1 + test3 <= 1:
            istop = 6
        if 1 + test2 <= 1:
            istop = 5
        if 1 + t1 <= 1:
            istop = 4
        if test3 <= ctol:
            istop = 3
        if test2 <= atol:
            istop = 2
        if test1 <= rtol:
            istop = 1
        if istop:
            break
    out = _finish(nufft, x, how)
    return (out, itn, istop) if return_info else out


def M_or(nufft):
    return int(nufft.M[0])


# --------------------------------------------------------------------------
# Krylov solvers on the normal operator (linalg/solve_cpu.py:253-288)
# --------------------------------------------------------------------------
_EPS = 2.220446049250313e-16      # complex128 machine epsilon (scipy's x dtype)


def _vdot(a, b):
    import torch
    return complex(torch.vdot(a, b))


def _nrm(v):
    import torch
    return float(torch.linalg.vector_norm(v))


def normal_krylov(nufft, y, solver, x0=None, *, maxiter=None, rtol=None, atol=0.0,
                  return_info=False, **kw):
    """solve(y, solver) for solver in bicg / bicgstab / gmres / lgmres: the
    scipy routine of that name on A = k2y2k (Hermitian), b = y2k(y), then
    x = k2xx(k) / sn.  Returns x (and scipy's info code with return_info)."""
    import torch
    if nufft.batch is not None or nufft.ninst > 1:
        raise NotImplementedError(solver + ' runs on single-coil, single-instance plans')
    if rtol is None:
        rtol = kw.pop('tol', 1e-5)
    yd, how = _dev(nufft, y, 'y')
    dev = nufft.device
    Kd = nufft.Kd

    def A(v):
        return nufft.k2y2k(v.to(torch.complex64).reshape(Kd)).reshape(-1).to(torch.complex128)
    b = nufft.y2k(yd).reshape(-1).to(torch.complex128)
    if x0 is None:
        x = torch.zeros_like(b)
    else:
        x0 = x0 if isinstance(x0, torch.Tensor) else torch.from_numpy(__import__('numpy').asarray(x0))
        x = x0.to(dev, torch.complex128).reshape(-1).clone()
    fn = KRYLOV[solver]
    x, info = fn(A, b, x, rtol=float(rtol), atol=float(atol), maxiter=maxiter, **kw)
    out = _finish(nufft, x.to(torch.complex64), how)
    return (out, info) if return_info else out


def _bicg(A, b, x, rtol, atol, maxiter):
    """scipy.sparse.linalg.bicg; A^H = A here, so rmatvec is A again."""
    bnrm2 = _nrm(b)
    atol = max(atol, rtol * bnrm2)
    if bnrm2 == 0:
        return b, 0
    if maxiter is None:
        maxiter = b.numel() * 10
    rhotol = _EPS ** 2
    rho_prev = p = ptilde = None
    r = b - A(x) if bool(x.any()) else b.clone()
    rtilde = r.clone()
    for it in range(maxiter):
        if _nrm(r) < atol:
            return x, 0
        rho = _vdot(rtilde, r)
        if abs(rho) < rhotol:
            return x, -10
        if it > 0:
            beta = rho / rho_prev
            p = p * beta + r
            ptilde = ptilde * beta.conjugate() + rtilde
        else:
            p = r.clone()
            ptilde = rtilde.clone()
        q = A(p)
        qtilde = A(ptilde)
        rv = _vdot(ptilde, q)
        if rv == 0:
            return x, -11
        alpha = rho / rv
        x = x + alpha * p
        r = r - alpha * q
        rtilde = rtilde - alpha.conjugate() * qtilde
        rho_prev = rho
    return x, maxiter


def _bicgstab(A, b, x, rtol, atol, maxiter):
    """scipy.sparse.linalg.bicgstab."""
    bnrm2 = _nrm(b)
    atol = max(atol, rtol * bnrm2)
    if bnrm2 == 0:
        return b, 0
    if maxiter is None:
        maxiter = b.numel() * 10
    rhotol = omegatol = _EPS ** 2
    rho_prev = omega = alpha = p = v = None
    r = b - A(x) if bool(x.any()) else b.clone()
    rtilde = r.clone()
    for it in range(maxiter):
        if _nrm(r) < atol:
            return x, 0
        rho = _vdot(rtilde, r)
        if abs(rho) < rhotol:
            return x, -10
        if it > 0:
            if abs(omega) < omegatol:
                return x, -11
            beta = (rho / rho_prev) * (alpha / omega)
            p = (p - omega * v) * beta + r
        else:
            p = r.clone()
        v = A(p)
        rv = _vdot(rtilde, v)
        if rv == 0:
            return x, -11
        alpha = rho / rv
        r = r - alpha * v
        s = r
        if _nrm(s) < atol:
            return x + alpha * p, 0
        t = A(s)
        omega = _vdot(t, s) / _vdot(t, t)
        x = x + alpha * p + omega * s
        r = r - omega * t
        rho_prev = rho
    return x, maxiter


def _gmres(A, b, x, rtol, atol, maxiter, restart=None):
    """scipy.sparse.linalg.gmres (restarted, modified Gram-Schmidt, Givens
    rotations from LAPACK zlartg, scipy's inner-tolerance control)."""
    import numpy as np
    import torch
    from scipy.linalg import get_lapack_funcs
    n = b.numel()
    bnrm2 = _nrm(b)
    atol = max(atol, rtol * bnrm2)
    if bnrm2 == 0:
        return b, 0
    if maxiter is None:
        maxiter = n * 10
    restart = min(20 if restart is None else int(restart), n)
    ptol_max_factor = 1.0
    ptol = bnrm2 * min(ptol_max_factor, atol / bnrm2)
    presid = 0.0
    lartg = get_lapack_funcs('lartg', dtype=np.complex128)
    V = torch.empty((restart + 1, n), dtype=torch.complex128, device=b.device)
    h = np.zeros((restart, restart + 1), dtype=np.complex128)
    givens = np.zeros((restart, 2), dtype=np.complex128)
    rnorm = None
    for it in range(maxiter):
        if it == 0:
            r = b - A(x) if bool(x.any()) else b.clone()
            if _nrm(r) < atol:
                return x, 0
        tmp = _nrm(r)
        V[0] = r * (1 / tmp)
        S = np.zeros(restart + 1, dtype=np.complex128)
        S[0] = tmp
        breakdown = False
        for col in range(restart):
            w = A(V[col])
            h0 = _nrm(w)
            for k in range(col + 1):
                t = _vdot(V[k], w)
                h[col, k] = t
                w = w - t * V[k]
            h1 = _nrm(w)
            h[col, col + 1] = h1
            V[col + 1] = w
            if h1 <= _EPS * h0:
                h[col, col + 1] = 0
                breakdown = True
            else:
                V[col + 1] *= (1 / h1)
            for k in range(col):
                c, s = givens[k, 0], givens[k, 1]
                n0, n1 = h[col, [k, k + 1]]
                h[col, [k, k + 1]] = [c * n0 + s * n1, -s.conj() * n0 + c * n1]
            c, s, mag = lartg(h[col, col], h[col, col + 1])
            givens[col, :] = [c, s]
            h[col, [col, col + 1]] = mag, 0
            tmp = -np.conjugate(s) * S[col]
            S[[col, col + 1]] = [c * S[col], tmp]
            presid = abs(tmp)
            if presid <= ptol or breakdown:
                break
        if h[col, col] == 0:
            S[col] = 0
        yv = np.zeros(col + 1, dtype=np.complex128)
        yv[:] = S[:col + 1]
        for k in range(col, 0, -1):
            if yv[k] != 0:
                yv[k] /= h[k, k]
                yv[:k] -= yv[k] * h[k, :k]
        if yv[0] != 0:
            yv[0] /= h[0, 0]
        x = x + torch.from_numpy(yv).to(b.device) @ V[:col + 1]
        r = b - A(x)
        rnorm = _nrm(r)
        if rnorm <= atol:
            break
        elif breakdown:
            break
        elif presid <= ptol:
            ptol_max_factor = max(_EPS, 0.25 * ptol_max_factor)
        else:
            ptol_max_factor = min(1.0, 1.5 * ptol_max_factor)
        ptol = presid * min(ptol_max_factor, atol / rnorm)
    return x, (0 if rnorm <= atol else maxiter)


def _fgmres(A, v0, m, atol, outer_v):
    """The FGMRES Arnoldi process of scipy's LGMRES (augmentation vectors
    appended), H kept in QR form updated by scipy.linalg.qr_insert."""
    import numpy as np
    import torch
    from scipy.linalg import lstsq, qr_insert
    vs = [v0]
    zs = []
    m = m + len(outer_v)
    Q = np.ones((1, 1), dtype=np.complex128)
    R = np.zeros((1, 0), dtype=np.complex128)
    breakdown = False
    res = np.nan
    for j in range(m):
        if j >= m - len(outer_v):
            z, w = outer_v[j - (m - len(outer_v))]
        else:
            z, w = vs[-1], None
        w = A(z) if w is None else w.clone()
        w_norm = _nrm(w)
        hcur = np.zeros(j + 2, dtype=np.complex128)
        for i, v in enumerate(vs):
            a = _vdot(v, w)
            hcur[i] = a
            w = w - a * v
        hcur[i + 1] = _nrm(w)
        with np.errstate(over='ignore', divide='ignore'):
            a = 1 / hcur[-1]
        if np.isfinite(a):
            w = w * a
        if not (hcur[-1] > _EPS * w_norm):
            breakdown = True
        vs.append(w)
        zs.append(z)
        Q2 = np.zeros((j + 2, j + 2), dtype=np.complex128, order='F')
        Q2[:j + 1, :j + 1] = Q
        Q2[j + 1, j + 1] = 1
        R2 = np.zeros((j + 2, j), dtype=np.complex128, order='F')
        R2[:j + 1, :] = R
        Q, R = qr_insert(Q2, R2, hcur, j, which='col', overwrite_qru=True, check_finite=False)
        res = abs(Q[0, -1])
        if res < atol or breakdown:
            break
    if not np.isfinite(R[j, j]):
        raise np.linalg.LinAlgError()
    yv, _, _, _ = lstsq(R[:j + 1, :j + 1], Q[0, :j + 1].conj())
    return Q, R, vs, zs, yv, res


def _lgmres(A, b, x, rtol, atol, maxiter, inner_m=30, outer_k=3, outer_v=None,
            store_outer_Av=True, prepend_outer_v=False):
    """scipy.sparse.linalg.lgmres (augmentation vectors appended)."""
    import numpy as np
    import torch
    if prepend_outer_v:
        raise NotImplementedError('lgmres: prepend_outer_v=True is not supported')
    if maxiter is None:
        maxiter = 1000
    if outer_v is None:
        outer_v = []
    b_norm = _nrm(b)
    atol = max(atol, rtol * b_norm)
    if b_norm == 0:
        return b, 0
    ptol_max_factor = 1.0
    for k_outer in range(maxiter):
        r_outer = A(x) - b
        r_norm = _nrm(r_outer)
        if r_norm <= max(atol, rtol * b_norm):
            break
        v0 = -r_outer
        inner_res_0 = _nrm(v0)
        v0 = v0 * (1.0 / inner_res_0)
        ptol = min(ptol_max_factor, max(atol, rtol * b_norm) / r_norm)
        try:
            Q, R, vs, zs, yv, pres = _fgmres(A, v0, inner_m, ptol, outer_v)
            yv = yv * inner_res_0
            if not np.isfinite(yv).all():
                raise np.linalg.LinAlgError()
        except np.linalg.LinAlgError:
            return x, k_outer + 1
        if pres > ptol:
            ptol_max_factor = min(1.0, 1.5 * ptol_max_factor)
        else:
            ptol_max_factor = max(1e-16, 0.25 * ptol_max_factor)
        dx = zs[0] * complex(yv[0])
        for w, yc in zip(zs[1:], yv[1:]):
            dx = dx + w * complex(yc)
        nx = _nrm(dx)
        if nx > 0:
            if store_outer_Av:
                q = Q.dot(R.dot(yv))
                ax = vs[0] * complex(q[0])
                for v, qc in zip(vs[1:], q[1:]):
                    ax = ax + v * complex(qc)
                outer_v.append((dx / nx, ax / nx))
            else:
                outer_v.append((dx / nx, None))
        while len(outer_v) > outer_k:
            del outer_v[0]
        x = x + dx
    else:
        return x, maxiter
    return x, 0


KRYLOV = {'bicg': _bicg, 'bicgstab': _bicgstab, 'gmres': _gmres, 'lgmres': _lgmres}

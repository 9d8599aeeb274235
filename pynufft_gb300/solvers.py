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
    raise NotImplementedError(f"solver {solver!r} is not available; use 'cg', 'dc', 'lsqr' or 'lsmr'")


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

"""Generate the golden fixtures in this directory from the reference itself.

Run where a checkout of the reference (pynufft 2025.2.1) is available, giving
its location with --reference or the PYNUFFT_REFERENCE environment variable:

    python tests/golden/make_golden.py --reference /path/to/pynufft [groups...]

It imports the reference package read-only through a symlink
(<tmp>/refpkg/pynufft -> the checkout, no bytecode written), runs the
reference numpy ``NUFFT`` on seeded synthetic inputs and writes ``*.npz``
fixtures next to this script.  The GPU machine never runs this script; it only
reads the fixtures.

Cases (all seeds fixed):
  plan_*.npz   small 1D/2D/3D, odd and anisotropic plans: om, inputs, the
               reference's per-stage outputs, forward/adjoint/selfadjoint,
               solve('cg', maxiter=5), sn, alpha, T and ud/kd tables.
  radial_c1.npz  2D radial 256 spokes x 512 samples, Nd 256^2, Kd 512^2,
               Jd 6^2: reference forward at 4096 sampled rows and adjoint at
               4096 sampled pixels (inputs regenerated from their seeds).
  cg_c1.npz    solve(y, 'cg', maxiter=20) of the reference on the radial_c1
               plan, y = complex Gaussian samples (seed 100, the radial_c1
               adjoint input): the full complex64 image.
  ndft_known_answer.npz  the exact-NDFT vectors shipped with the reference
               (tests/tmp2d_{1,2,3}_.mat: image fhat, points x, NDFT f2) and
               the reference's own J=6, K=2N forward at om = 2*pi*x.
  l1tvols.npz  solve(y, 'L1TVOLS', maxiter, rho) of the reference on a 2D
               radial plan (Nd 32^2) and a 3D random plan (Nd 12^3), y the
               reference forward of a disk phantom plus 1% noise.

Pass case groups (plans, radial, cg, ndft, l1tvols) to regenerate only those.
"""
from __future__ import annotations

import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = None   # the reference checkout, from --reference or PYNUFFT_REFERENCE


def _import_reference():
    import tempfile
    os.environ['PYTHONDONTWRITEBYTECODE'] = '1'
    sys.dont_write_bytecode = True
    pkgdir = os.path.join(tempfile.gettempdir(), 'refpkg')
    os.makedirs(pkgdir, exist_ok=True)
    link = os.path.join(pkgdir, 'pynufft')
    if os.path.islink(link) and os.readlink(link) != REF:
        os.unlink(link)
    if not os.path.islink(link):
        os.symlink(REF, link)
    sys.path.insert(0, pkgdir)
    warnings.filterwarnings('ignore')
    import pynufft
    from pynufft.src._helper import helper
    return pynufft, helper


def radial_c1_om():
    """256 spokes x 512 samples, angles k*pi/256, radius linspace(-pi, pi, 512, endpoint=False)."""
    ang = np.arange(256) * np.pi / 256
    rad = np.linspace(-np.pi, np.pi, 512, endpoint=False)
    om = np.empty((256 * 512, 2))
    om[:, 0] = (np.cos(ang)[:, None] * rad[None, :]).ravel()
    om[:, 1] = (np.sin(ang)[:, None] * rad[None, :]).ravel()
    return om


def cplx(rng, shape, dtype=np.complex64):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)


PLAN_CASES = {
    # name: (Nd, Kd, Jd, M, om range (x pi), seed)
    'plan_1d': ((64,), (128,), (6,), 300, 1.0, 11),
    'plan_2d': ((32, 32), (64, 64), (6, 6), 1000, 1.0, 12),
    'plan_2d_odd': ((21, 30), (42, 48), (5, 6), 600, 1.5, 13),
    'plan_3d': ((12, 12, 12), (24, 24, 24), (6, 6, 6), 800, 1.0, 14),
    'plan_3d_aniso': ((12, 20, 16), (24, 30, 32), (4, 6, 5), 400, 1.0, 15),
    'plan_2d_grid': ((24, 24), (48, 48), (4, 4), 0, 1.0, 16),
    'plan_2d_J8': ((40, 40), (80, 80), (8, 8), 500, 1.0, 17),
}


def grid_points(Kd, rng):
    """Points exactly on oversampled-grid nodes, at +-pi and at 0."""
    k = rng.integers(-Kd[0], Kd[0], size=(200, 2))
    om = 2 * np.pi * k / np.array(Kd)
    edge = np.array([[np.pi, np.pi], [-np.pi, -np.pi], [0.0, 0.0], [np.pi, -np.pi],
                     [-np.pi, 0.0], [1e-15, -1e-15], [2 * np.pi / Kd[0], 0.0]])
    return np.vstack([om, edge])


def make_plan_case(pynufft, helper, name, Nd, Kd, Jd, M, rng_scale, seed):
    rng = np.random.default_rng(seed)
    if name == 'plan_2d_grid':
        om = grid_points(Kd, rng)
    else:
        om = rng.uniform(-np.pi * rng_scale, np.pi * rng_scale, (M, len(Nd)))
    M = om.shape[0]
    A = pynufft.NUFFT()
    A.plan(om, Nd, Kd, Jd)
    x = cplx(rng, Nd)
    y = cplx(rng, (M,))
    k = cplx(rng, Kd)
    out = dict(om=om, Nd=np.array(Nd), Kd=np.array(Kd), Jd=np.array(Jd), x=x, y=y, k=k)
    out['sn'] = A.sn
    out['x2xx'] = A.x2xx(x)
    out['xx2k'] = A.xx2k(out['x2xx'])
    out['k2y'] = A.k2y(k)
    out['y2k'] = A.y2k(y)
    out['k2xx'] = A.k2xx(k)
    out['xx2x'] = A.xx2x(x)
    out['forward'] = A.forward(x)
    out['adjoint'] = A.adjoint(y)
    out['selfadjoint'] = A.selfadjoint(x)
    out['solve_cg5'] = A.solve(y, 'cg', maxiter=5)
    for d in range(len(Nd)):
        a, b = helper.nufft_alpha_kb_fit(Nd[d], Jd[d], Kd[d])
        out[f'alpha{d}'] = np.asarray(a).ravel()
        out[f'T{d}'] = helper.nufft_T(Nd[d], Jd[d], Kd[d], a, b)
        ud = helper.min_max(Nd[d], Jd[d], Kd[d], a, b, om[:, d], True)
        kd = helper.OMEGA_k(Jd[d], Kd[d], om[:, d], Kd, d, len(Nd), True).T
        out[f'ud{d}'] = ud
        out[f'kd{d}'] = np.rint(kd).astype(np.int64)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)
    print(name, 'M =', M)


def make_radial_c1(pynufft):
    om = radial_c1_om()
    Nd, Kd, Jd = (256, 256), (512, 512), (6, 6)
    A = pynufft.NUFFT()
    A.plan(om, Nd, Kd, Jd)
    x = cplx(np.random.default_rng(0), Nd)
    y = cplx(np.random.default_rng(100), (om.shape[0],))
    yf = A.forward(x)
    xa = A.adjoint(y)
    rng = np.random.default_rng(101)
    rows = np.sort(rng.choice(om.shape[0], 4096, replace=False))
    pix = np.sort(rng.choice(Nd[0] * Nd[1], 4096, replace=False))
    np.savez_compressed(os.path.join(HERE, 'radial_c1.npz'), rows=rows, forward_rows=yf[rows],
                        pixels=pix, adjoint_pixels=xa.ravel()[pix],
                        forward_norm=np.linalg.norm(yf), adjoint_norm=np.linalg.norm(xa))
    print('radial_c1')


def make_cg_c1(pynufft):
    """solve(y, 'cg', maxiter=20) on the 2D radial plan (Nd 256^2, Kd 512^2, Jd 6^2)."""
    om = radial_c1_om()
    A = pynufft.NUFFT()
    A.plan(om, (256, 256), (512, 512), (6, 6))
    y = cplx(np.random.default_rng(100), (om.shape[0],))
    x = A.solve(y, 'cg', maxiter=20)
    np.savez_compressed(os.path.join(HERE, 'cg_c1.npz'), maxiter=20, y_seed=100,
                        x=np.asarray(x, dtype=np.complex64))
    print('cg_c1')


def make_ndft_known_answer(pynufft):
    import scipy.io
    fhat = None
    out = {}
    for i in (1, 2, 3):
        d = scipy.io.loadmat(os.path.join(REF, 'tests', f'tmp2d_{i}_.mat'))
        if fhat is None:
            fhat = d['fhat']
            out['fhat'] = fhat
        assert np.array_equal(fhat, d['fhat'])
        out[f'x{i}'] = d['x']
        out[f'f2_{i}'] = d['f2'].ravel()
        A = pynufft.NUFFT()
        A.plan(2 * np.pi * d['x'], (256, 256), (512, 512), (6, 6))
        out[f'ref_forward_{i}'] = A.forward(fhat.astype(np.complex64))
    np.savez_compressed(os.path.join(HERE, 'ndft_known_answer.npz'), **out)
    print('ndft_known_answer')


def disk_phantom(Nd, rng):
    """Piecewise-constant image of 6 random disks/ellipses (complex amplitudes)."""
    grids = np.meshgrid(*[np.arange(n) - n / 2 for n in Nd], indexing='ij')
    x = np.zeros(Nd, np.complex64)
    for _ in range(6):
        c = rng.uniform(-0.3, 0.3, len(Nd)) * np.array(Nd)
        a = rng.uniform(0.08, 0.3, len(Nd)) * np.array(Nd)
        inside = sum(((g - ci) / ai) ** 2 for g, ci, ai in zip(grids, c, a)) <= 1
        x[inside] += complex(rng.standard_normal(), rng.standard_normal())
    return x


def make_l1tvols(pynufft):
    """solve(y, 'L1TVOLS', maxiter, rho) on 2D radial and 3D random plans."""
    out = {}
    rng = np.random.default_rng(11)
    ang = np.arange(48) * np.pi / 48
    rad = np.linspace(-np.pi, np.pi, 64, endpoint=False)
    om2 = np.stack([(np.cos(ang)[:, None] * rad).ravel(), (np.sin(ang)[:, None] * rad).ravel()], 1)
    om3 = rng.uniform(-np.pi, np.pi, (6000, 3))
    for tag, om, Nd, Kd, Jd, it, rho in (('2d', om2, (32, 32), (64, 64), (6, 6), 6, 0.1),
                                         ('3d', om3, (12, 12, 12), (24, 24, 24), (6, 6, 6), 4, 0.5)):
        A = pynufft.NUFFT()
        A.plan(om, Nd, Kd, Jd)
        x = disk_phantom(Nd, rng)
        y = A.forward(x).astype(np.complex64)
        y = (y + 0.01 * np.abs(y).mean() * cplx(rng, y.shape)).astype(np.complex64)
        out[f'om_{tag}'] = om
        out[f'geom_{tag}'] = np.array([Nd, Kd, Jd])
        out[f'y_{tag}'] = y
        out[f'maxiter_{tag}'] = it
        out[f'rho_{tag}'] = rho
        out[f'x_{tag}'] = A.solve(y, 'L1TVOLS', maxiter=it, rho=rho)
    np.savez_compressed(os.path.join(HERE, 'l1tvols.npz'), **out)
    print('l1tvols')


def main():
    global REF
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split('\n')[0])
    ap.add_argument('--reference', default=os.environ.get('PYNUFFT_REFERENCE'),
                    help='path of the reference checkout (default: $PYNUFFT_REFERENCE)')
    ap.add_argument('groups', nargs='*')
    args = ap.parse_args()
    if not args.reference or not os.path.isdir(args.reference):
        ap.error('give the reference checkout with --reference or PYNUFFT_REFERENCE')
    REF = os.path.abspath(args.reference)
    pynufft, helper = _import_reference()
    only = args.groups
    if not only or 'plans' in only:
        for name, args in PLAN_CASES.items():
            make_plan_case(pynufft, helper, name, *args)
    if not only or 'radial' in only:
        make_radial_c1(pynufft)
    if not only or 'cg' in only:
        make_cg_c1(pynufft)
    if not only or 'ndft' in only:
        make_ndft_known_answer(pynufft)
    if not only or 'l1tvols' in only:
        make_l1tvols(pynufft)


if __name__ == '__main__':
    main()

"""The oracle (a numpy restatement of the reference) against fixtures that the
reference itself produced (tests/golden/make_golden.py), and against the
exact-NDFT known-answer vectors shipped with the reference."""
import numpy as np
import pytest

from conftest import PLAN_CASES, load_golden
from oracle.nufft_oracle import (ChunkedOracleNUFFT, OracleNUFFT, alpha_beta_fit, interp_csr,
                                 minmax_T, nudft_adjoint_pixels, nudft_forward_rows, rel_l2)


def _tup(a):
    return tuple(int(v) for v in a)


@pytest.mark.parametrize('case', PLAN_CASES)
def test_oracle_matches_reference_stages(case):
    g = load_golden(case)
    Nd, Kd, Jd = _tup(g['Nd']), _tup(g['Kd']), _tup(g['Jd'])
    O = OracleNUFFT()
    O.plan(g['om'], Nd, Kd, Jd)
    assert np.array_equal(O.sn, g['sn'])
    for d in range(len(Nd)):
        a, b = alpha_beta_fit(Nd[d], Jd[d], Kd[d])
        assert np.array_equal(a, g[f'alpha{d}'])
        np.testing.assert_allclose(minmax_T(Nd[d], Jd[d], Kd[d], a, b), g[f'T{d}'], rtol=1e-12, atol=1e-9)
    checks = {
        'x2xx': O.x2xx(g['x']), 'xx2k': O.xx2k(g['x2xx']), 'k2y': O.k2y(g['k']),
        'y2k': O.y2k(g['y']), 'k2xx': O.k2xx(g['k']), 'xx2x': O.xx2x(g['x']),
        'forward': O.forward(g['x']), 'adjoint': O.adjoint(g['y']),
        'selfadjoint': O.selfadjoint(g['x']), 'solve_cg5': O.solve(g['y'], 'cg', maxiter=5),
    }
    for k, v in checks.items():
        assert v.dtype == g[k].dtype, (k, v.dtype, g[k].dtype)
        assert rel_l2(v, g[k]) < 1e-12, (k, rel_l2(v, g[k]))


@pytest.mark.parametrize('case', ['plan_2d', 'plan_3d_aniso', 'plan_2d_grid'])
def test_oracle_tables_match_reference_ud_kd(case):
    g = load_golden(case)
    Nd, Kd, Jd = _tup(g['Nd']), _tup(g['Kd']), _tup(g['Jd'])
    from oracle.nufft_oracle import minmax_axis
    for d in range(len(Nd)):
        a, b = alpha_beta_fit(Nd[d], Jd[d], Kd[d])
        ud, kd = minmax_axis(g['om'][:, d], Nd[d], Jd[d], Kd[d], a, b)
        stride = int(np.prod(Kd[d + 1:])) if d < len(Nd) - 1 else 1
        np.testing.assert_allclose(ud, g[f'ud{d}'], rtol=0, atol=1e-13)
        assert np.array_equal(kd * stride, g[f'kd{d}'])


def test_oracle_ndft_known_answer():
    """tests/tmp2d_{1,2,3}_.mat: f2 is the exact NDFT of fhat at x; the reference
    (J=6, K=2N) scores 3.0e-6 / 5.2e-6 / 4.6e-6 on them."""
    g = load_golden('ndft_known_answer')
    fhat = g['fhat'].astype(np.complex64)
    for i in (1, 2, 3):
        om = 2 * np.pi * g[f'x{i}']
        O = OracleNUFFT()
        O.plan(om, (256, 256), (512, 512), (6, 6))
        y = O.forward(fhat)
        assert rel_l2(y, g[f'ref_forward_{i}']) < 1e-12
        err = rel_l2(y, g[f'f2_{i}'])
        assert err < 1e-5, err
        # the FP64 NUDFT restatement reproduces f2 to round-off
        rows = np.arange(0, 1000, 37)
        yd = nudft_forward_rows(g['fhat'], om, rows)
        assert rel_l2(yd, g[f'f2_{i}'][rows]) < 1e-12


def test_oracle_radial_c1_fixture():
    from tests_util import radial_c1_om
    g = load_golden('radial_c1')
    om = radial_c1_om()
    O = OracleNUFFT()
    O.plan(om, (256, 256), (512, 512), (6, 6))
    x = _cplx(np.random.default_rng(0), (256, 256))
    y = _cplx(np.random.default_rng(100), (om.shape[0],))
    yf = O.forward(x)
    xa = O.adjoint(y)
    assert rel_l2(yf[g['rows']], g['forward_rows']) < 1e-12
    assert rel_l2(xa.ravel()[g['pixels']], g['adjoint_pixels']) < 1e-12
    np.testing.assert_allclose(np.linalg.norm(yf), g['forward_norm'], rtol=1e-12)


def _cplx(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def test_nudft_subset_against_dense():
    rng = np.random.default_rng(3)
    Nd = (6, 5, 4)
    om = rng.uniform(-np.pi, np.pi, (40, 3))
    x = _cplx(rng, Nd)
    grid = np.indices(Nd).reshape(3, -1).T - np.array(Nd) / 2
    A = np.exp(-1j * om @ grid.T)
    np.testing.assert_allclose(nudft_forward_rows(x, om), A @ x.ravel(), rtol=1e-12, atol=1e-12)
    y = _cplx(rng, (40,))
    pix = np.array([0, 7, 33, 119])
    np.testing.assert_allclose(nudft_adjoint_pixels(y, om, Nd, pix), (A.conj().T @ y)[pix],
                               rtol=1e-12, atol=1e-12)


def test_oracle_batch_is_per_coil_loop():
    rng = np.random.default_rng(4)
    om = rng.uniform(-np.pi, np.pi, (300, 2))
    O1 = OracleNUFFT(); O1.plan(om, (16, 16), (32, 32), (6, 6))
    OB = OracleNUFFT(); OB.plan(om, (16, 16), (32, 32), (6, 6), batch=3)
    x = _cplx(rng, (16, 16, 3))
    yb = OB.forward(x)
    for b in range(3):
        assert np.array_equal(yb[:, b], O1.forward(x[..., b]))


def test_oracle_adjoint_identity():
    rng = np.random.default_rng(5)
    om = rng.uniform(-np.pi, np.pi, (500, 2))
    O = OracleNUFFT(); O.plan(om, (20, 24), (40, 48), (6, 6))
    x = _cplx(rng, (20, 24)).astype(np.complex128)
    y = _cplx(rng, (500,)).astype(np.complex128)
    lhs = np.vdot(O.forward(x), y)
    rhs = np.prod((40, 48)) * np.vdot(x, O.adjoint(y))
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


@pytest.mark.parametrize('tag', ['2d', '3d'])
def test_oracle_l1tvols_matches_reference(tag):
    """The oracle's split-Bregman L1-TV restatement reproduces the
    reference's solve(y, 'L1TVOLS', maxiter, rho) (linalg/solve_cpu.py:42-163)."""
    g = load_golden('l1tvols')
    Nd, Kd, Jd = [tuple(int(v) for v in r) for r in g[f'geom_{tag}']]
    O = OracleNUFFT()
    O.plan(g[f'om_{tag}'], Nd, Kd, Jd)
    x = O.l1tvols(g[f'y_{tag}'], int(g[f'maxiter_{tag}']), float(g[f'rho_{tag}']))
    assert rel_l2(x, g[f'x_{tag}']) < 1e-6


def test_oracle_cg_c1_fixture():
    """solve(y, 'cg', maxiter=20) on the 2D radial plan (256^2 / 512^2, J 6):
    the oracle's restatement of scipy's CG against the reference's own
    result (complex64 output, so ~1e-7 is rounding)."""
    from tests_util import radial_c1_om
    g = load_golden('cg_c1')
    om = radial_c1_om()
    O = OracleNUFFT()
    O.plan(om, (256, 256), (512, 512), (6, 6))
    y = _cplx(np.random.default_rng(int(g['y_seed'])), (om.shape[0],))
    x, it = O.solve(y, 'cg', maxiter=int(g['maxiter']), return_info=True)
    assert it == 20
    assert rel_l2(x, g['x']) < 1e-6, rel_l2(x, g['x'])


@pytest.mark.parametrize('batch', [None, 3])
def test_chunked_oracle_equals_the_full_plan(batch):
    """Planning on row chunks (forward concatenates, adjoint sums the chunks'
    spH . y) gives the unchunked oracle's results bit for bit, and the
    row-subset forward equals those rows of the full forward."""
    rng = np.random.default_rng(6)
    Nd, Kd, Jd = (10, 12, 8), (20, 24, 16), (6, 6, 6)
    om = rng.uniform(-np.pi, np.pi, (2300, 3))
    O = OracleNUFFT()
    O.plan(om, Nd, Kd, Jd, batch=batch)
    C = ChunkedOracleNUFFT()
    C.plan(om, Nd, Kd, Jd, batch=batch, chunk=600)
    tail = () if batch is None else (batch,)
    x = _cplx(rng, Nd + tail)
    y = _cplx(rng, (2300,) + tail)
    assert np.array_equal(C.forward(x), O.forward(x))
    assert np.array_equal(C.adjoint(y), O.adjoint(y))
    rows = np.array([0, 599, 600, 1777, 2299])
    assert np.array_equal(C.forward_rows(x, rows), O.forward(x)[rows])


def test_nudft_adjoint_pixels_with_coils():
    rng = np.random.default_rng(8)
    Nd = (5, 6, 4)
    om = rng.uniform(-np.pi, np.pi, (70, 3))
    y = _cplx(rng, (70, 3))
    pix = np.array([1, 50, 119])
    got = nudft_adjoint_pixels(y, om, Nd, pix, chunk=16)
    for b in range(3):
        np.testing.assert_allclose(got[:, b], nudft_adjoint_pixels(y[:, b], om, Nd, pix),
                                   rtol=1e-12, atol=1e-12)

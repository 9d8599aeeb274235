"""Plans of 8 or more coils: forward / adjoint / selfadjoint through the
coil-team kernels, the adjoint of 3D plans and of 2D plans with a multiple
of 32 coils gridding by register rows straight into coil-major spectra
(interp_cm.cuh), the others through the coil-team tile.  Against the oracle
(one single-coil reference transform per coil, linalg/nufft_hsa.py:203-228
batch semantics) at 1e-5 relative L2, for 2D and 3D, J in {4, 6, 8}, 8 to 32
coils, one or several instances, clustered points (bins split into several
sub-problems), both gridding modes; the deterministic mode bitwise
repeatable, on one plan and across plans of the same points."""
import numpy as np
import pytest

from oracle.nufft_oracle import OracleNUFFT, rel_l2
from tests_util import cplx

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _points(rng, M, ndim):
    """Uniform points plus a dense cluster near the k-space centre (bins of
    more than one sub-problem) and a few on the +-pi edges (wrapped tiles)."""
    om = rng.uniform(-np.pi, np.pi, (M, ndim))
    om[: M // 2] = rng.normal(0.0, 0.05, (M // 2, ndim))
    om[-4:] = np.pi * np.array([[1.0], [-1.0], [0.999], [-0.999]])
    return om


CASES = [((24, 20), (48, 40), 6, 8), ((24, 20), (48, 40), 4, 32), ((20, 24), (40, 48), 8, 16),
         ((24, 20), (48, 40), 6, 24), ((12, 14, 10), (24, 28, 20), 6, 8),
         ((12, 14, 10), (24, 28, 20), 4, 32), ((10, 10, 10), (20, 20, 20), 8, 16)]


@pytest.mark.parametrize('Nd,Kd,J,B', CASES)
@pytest.mark.parametrize('det', [False, True])
def test_coil_major_transforms_match_oracle(Nd, Kd, J, B, det):
    from pynufft_gb300 import NUFFT
    rng = np.random.default_rng(81)
    M = 3000
    Jd = (J,) * len(Nd)
    om = _points(rng, M, len(Nd))
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd, batch=B, deterministic=det)
    O = OracleNUFFT()
    O.plan(om, Nd, Kd, Jd, batch=B)
    x = cplx(rng, Nd + (B,))
    y = cplx(rng, (M, B))
    ef = rel_l2(A.forward(x), O.forward(x))
    xa = A.adjoint(y)
    ea = rel_l2(xa, O.adjoint(y))
    es = rel_l2(A.selfadjoint(x), O.selfadjoint(x))
    assert max(ef, ea, es) < TOL, (ef, ea, es)
    if det:
        assert np.array_equal(xa, A.adjoint(y))
    A.check()


@pytest.mark.parametrize('ndim,B', [(2, 8), (3, 8), (2, 32)])
def test_coil_major_many_instances_match_oracle(ndim, B):
    from pynufft_gb300 import NUFFT
    rng = np.random.default_rng(82)
    Nd, Kd = ((24, 20), (48, 40)) if ndim == 2 else ((12, 12, 10), (24, 24, 20))
    Jd = (6,) * ndim
    Ms = [900, 1, 2500]
    oms = [_points(rng, m, ndim) if m > 8 else rng.uniform(-np.pi, np.pi, (m, ndim)) for m in Ms]
    A = NUFFT(0)
    A.plan_many(oms, Nd, Kd, Jd, batch=B)
    x = cplx(rng, (len(Ms),) + Nd + (B,))
    y = cplx(rng, (sum(Ms), B))
    yf = A.forward(x)
    xa = A.adjoint(y)
    off = 0
    for i, om in enumerate(oms):
        O = OracleNUFFT()
        O.plan(om, Nd, Kd, Jd, batch=B)
        sl = slice(off, off + Ms[i])
        assert rel_l2(yf[sl], O.forward(x[i])) < TOL, i
        assert rel_l2(xa[i], O.adjoint(y[sl])) < TOL, i
        off += Ms[i]


@pytest.mark.parametrize('Nd,Kd,J,B', [((12, 14, 10), (24, 28, 20), 6, 8),
                                       ((24, 20), (48, 40), 6, 32),
                                       ((24, 20), (48, 40), 6, None)])
def test_deterministic_plans_of_the_same_points_agree_bitwise(Nd, Kd, J, B):
    """Two deterministic plans of the same points (planned separately, so
    their binning ran twice) give bitwise equal adjoints, y2k stages and
    10-iteration CG solves: a bin's points are ranked by index, not in the
    order threads reached the bin, so the row gridding's fixed-order float
    sums are the same on every plan."""
    from pynufft_gb300 import NUFFT
    rng = np.random.default_rng(82)
    M = 4000
    om = _points(rng, M, len(Nd))
    y = cplx(rng, (M,) + (() if B is None else (B,)))
    out = []
    for _ in range(2):
        A = NUFFT(0)
        A.plan(om, Nd, Kd, (J,) * len(Nd), batch=B, deterministic=True)
        out.append((A.adjoint(y), A.y2k(y), A.solve(y, 'cg', maxiter=10)))
        A.check()
        A.release()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize('det', [False, True])
def test_empty_and_ragged_coil_plans(det):
    """Edge cases of the coil paths: a 3D 8-coil and a 2D 32-coil plan with
    no points (forward gives (0, B), adjoint and y2k zeros, CG zeros); a
    single point; and a many-instance coil plan whose middle instance has
    no points while its neighbours match the oracle."""
    from pynufft_gb300 import NUFFT
    rng = np.random.default_rng(83)
    for Nd, Kd, B in (((12, 14, 10), (24, 28, 20), 8), ((24, 20), (48, 40), 32)):
        Jd = (6,) * len(Nd)
        A = NUFFT(0)
        A.plan(np.zeros((0, len(Nd))), Nd, Kd, Jd, batch=B, deterministic=det)
        assert A.forward(cplx(rng, Nd + (B,))).shape == (0, B)
        y0 = np.zeros((0, B), np.complex64)
        assert not np.any(A.adjoint(y0)) and not np.any(A.y2k(y0))
        assert not np.any(A.solve(y0, 'cg', maxiter=3))
        A.check()
        om = rng.uniform(-np.pi, np.pi, (1, len(Nd)))
        A.plan(om, Nd, Kd, Jd, batch=B, deterministic=det)
        O = OracleNUFFT()
        O.plan(om, Nd, Kd, Jd, batch=B)
        x, y = cplx(rng, Nd + (B,)), cplx(rng, (1, B))
        assert rel_l2(A.forward(x), O.forward(x)) < TOL
        assert rel_l2(A.adjoint(y), O.adjoint(y)) < TOL
    Nd, Kd, Jd, B = (12, 14, 10), (24, 28, 20), (6, 6, 6), 8
    oms = [rng.uniform(-np.pi, np.pi, (700, 3)), np.zeros((0, 3)), _points(rng, 900, 3)]
    A = NUFFT(0)
    A.plan_many(oms, Nd, Kd, Jd, batch=B, deterministic=det)
    x = cplx(rng, (3,) + Nd + (B,))
    y = cplx(rng, (1600, B))
    yf, xa = A.forward(x), A.adjoint(y)
    assert yf.shape == (1600, B) and not np.any(xa[1])
    for i, (a, b) in ((0, (0, 700)), (2, (700, 1600))):
        O = OracleNUFFT()
        O.plan(oms[i], Nd, Kd, Jd, batch=B)
        assert rel_l2(yf[a:b], O.forward(x[i])) < TOL
        assert rel_l2(xa[i], O.adjoint(y[a:b])) < TOL
    A.check()

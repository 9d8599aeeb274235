"""GPU parity: the CUDA path (through the C ABI) against the reference's own
outputs (golden fixtures), the oracle, and the exact NDFT.

Tolerance: 1e-5 relative L2 against the reference's numpy NUFFT on the same
inputs; float32 gridding/FFT typically lands at 1e-7..1e-6.  Every test
states the bound it asserts.
"""
import numpy as np
import pytest

from conftest import PLAN_CASES, load_golden
from oracle.nufft_oracle import (OracleNUFFT, nudft_adjoint_pixels, nudft_forward_rows,
                                 rel_l2)

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _tup(a):
    return tuple(int(v) for v in a)


@pytest.fixture(scope='module')
def NUFFT():
    import torch
    assert torch.cuda.is_available()
    from pynufft_gb300 import NUFFT as N
    return N


def cplx(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize('case', PLAN_CASES)
def test_stages_match_reference(NUFFT, case):
    g = load_golden(case)
    Nd, Kd, Jd = _tup(g['Nd']), _tup(g['Kd']), _tup(g['Jd'])
    A = NUFFT(0)
    assert A.plan(g['om'], Nd, Kd, Jd) == 0
    np.testing.assert_allclose(A.sn, g['sn'], rtol=3e-7)   # float32 sn, 1 ulp
    got = {
        'x2xx': A.x2xx(g['x']), 'xx2k': A.xx2k(g['x2xx']), 'k2y': A.k2y(g['k']),
        'y2k': A.y2k(g['y']), 'k2xx': A.k2xx(g['k']), 'xx2x': A.xx2x(g['x']),
        'forward': A.forward(g['x']), 'adjoint': A.adjoint(g['y']),
        'selfadjoint': A.selfadjoint(g['x']),
    }
    errs = {k: rel_l2(v, g[k]) for k, v in got.items()}
    for k, v in got.items():
        assert v.shape == g[k].shape, k
        assert v.dtype == np.complex64, k
    assert max(errs.values()) < TOL, errs


@pytest.mark.parametrize('case', ['plan_2d', 'plan_3d', 'plan_1d'])
def test_solve_cg_matches_reference(NUFFT, case):
    """solve(y, 'cg', maxiter=5): float32 vectors with FP64 scalars against
    scipy's complex128 CG.  At 5 iterations the recursion barely amplifies
    the operator's float32 rounding (the oracle with a complex64-rounded
    operator lands ~5e-8 from the reference here), so the parity bar holds."""
    g = load_golden(case)
    A = NUFFT(0)
    A.plan(g['om'], _tup(g['Nd']), _tup(g['Kd']), _tup(g['Jd']))
    x, it = A.solve(g['y'], 'cg', maxiter=5, return_info=True)
    assert it == 5
    assert rel_l2(x, g['solve_cg5']) < TOL, rel_l2(x, g['solve_cg5'])


def test_radial_c1_matches_reference(NUFFT):
    from pynufft_gb300.trajectories import radial_2d
    g = load_golden('radial_c1')
    om = radial_2d(256, 512)
    A = NUFFT(0)
    A.plan(om, (256, 256), (512, 512), (6, 6))
    x = cplx(np.random.default_rng(0), (256, 256))
    y = cplx(np.random.default_rng(100), (om.shape[0],))
    yf = A.forward(x)
    xa = A.adjoint(y)
    assert rel_l2(yf[g['rows']], g['forward_rows']) < TOL
    assert rel_l2(xa.ravel()[g['pixels']], g['adjoint_pixels']) < TOL
    assert abs(np.linalg.norm(yf) / g['forward_norm'] - 1) < 1e-6


def test_ndft_known_answer(NUFFT):
    """The reference scores 3.0e-6 / 5.2e-6 / 4.6e-6 against the exact NDFT
    vectors of tests/tmp2d_{1,2,3}_.mat; the GPU path must stay within 1e-5
    of the exact NDFT and within 1e-5 of the reference."""
    g = load_golden('ndft_known_answer')
    fhat = g['fhat'].astype(np.complex64)
    for i in (1, 2, 3):
        A = NUFFT(0)
        A.plan(2 * np.pi * g[f'x{i}'], (256, 256), (512, 512), (6, 6))
        y = A.forward(fhat)
        e_exact = rel_l2(y, g[f'f2_{i}'])
        e_ref = rel_l2(y, g[f'ref_forward_{i}'])
        assert e_exact < 1e-5 and e_ref < TOL, (i, e_exact, e_ref)


@pytest.mark.parametrize('Nd,Kd,Jd,B', [((24, 20), (48, 40), (6, 6), 2),
                                        ((16, 16), (32, 32), (6, 6), 8),
                                        ((16, 16), (32, 32), (4, 4), 32),
                                        ((10, 12, 8), (20, 24, 16), (6, 6, 6), 3),
                                        ((64,), (128,), (6,), 5)])
def test_batch_matches_per_coil_oracle(NUFFT, Nd, Kd, Jd, B):
    rng = np.random.default_rng(7)
    M = 700
    om = rng.uniform(-np.pi, np.pi, (M, len(Nd)))
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd, batch=B)
    O = OracleNUFFT()
    O.plan(om, Nd, Kd, Jd, batch=B)
    x = cplx(rng, Nd + (B,))
    y = cplx(rng, (M, B))
    k = cplx(rng, Kd + (B,))
    assert rel_l2(A.forward(x), O.forward(x)) < TOL
    assert rel_l2(A.adjoint(y), O.adjoint(y)) < TOL
    assert rel_l2(A.k2y(k), O.k2y(k)) < TOL
    assert rel_l2(A.y2k(y), O.y2k(y)) < TOL
    assert rel_l2(A.xx2k(x), O.xx2k(x)) < TOL
    assert rel_l2(A.k2xx(k), O.k2xx(k)) < TOL


@pytest.mark.parametrize('B', [None, 2])
def test_many_instances_match_oracle(NUFFT, B):
    rng = np.random.default_rng(8)
    Nd, Kd, Jd = (20, 20), (40, 40), (6, 6)
    Ms = [300, 1, 1200, 57, 800]
    oms = [rng.uniform(-np.pi, np.pi, (m, 2)) for m in Ms]
    A = NUFFT(0)
    A.plan_many(oms, Nd, Kd, Jd, batch=B)
    tail = () if B is None else (B,)
    x = cplx(rng, (len(Ms),) + Nd + tail)
    y = cplx(rng, (sum(Ms),) + tail)
    yf = A.forward(x)
    xa = A.adjoint(y)
    off = 0
    for i, om in enumerate(oms):
        O = OracleNUFFT()
        O.plan(om, Nd, Kd, Jd, batch=B)
        sl = slice(off, off + Ms[i])
        assert rel_l2(yf[sl], O.forward(x[i])) < TOL
        assert rel_l2(xa[i], O.adjoint(y[sl])) < TOL
        off += Ms[i]


@pytest.mark.parametrize('B', [4, 8, 32])
def test_deterministic_gridding_is_bitwise_reproducible(NUFFT, B):
    """Exact fixed-point gridding, for lanes-per-point (B < 8) and coil-team
    (B >= 8) kernels alike: repeated calls are bitwise equal and match the
    oracle."""
    from pynufft_gb300.trajectories import radial_2d
    rng = np.random.default_rng(9)
    om = radial_2d(64, 128)       # dense centre: many contributions per cell
    y = cplx(rng, (om.shape[0], B))
    A = NUFFT(0)
    A.plan(om, (64, 64), (128, 128), (6, 6), batch=B, deterministic=True)
    k1 = A.y2k(y)
    k2 = A.y2k(y)
    x1 = A.adjoint(y)
    x2 = A.adjoint(y)
    assert np.array_equal(k1, k2) and np.array_equal(x1, x2)
    O = OracleNUFFT()
    O.plan(om, (64, 64), (128, 128), (6, 6), batch=B)
    assert rel_l2(k1, O.y2k(y)) < 1e-6
    assert rel_l2(x1, O.adjoint(y)) < TOL


def test_adjoint_identity(NUFFT):
    """<A x, y> = prod(Kd) <x, A^H y> (the reference adjoint carries 1/prod(Kd))."""
    rng = np.random.default_rng(10)
    for Nd, Kd, Jd in [((40, 36), (80, 72), (6, 6)), ((16, 12, 20), (32, 24, 40), (6, 6, 6))]:
        M = 3000
        om = rng.uniform(-np.pi, np.pi, (M, len(Nd)))
        A = NUFFT(0)
        A.plan(om, Nd, Kd, Jd)
        x = cplx(rng, Nd)
        y = cplx(rng, (M,))
        lhs = np.vdot(A.forward(x).astype(np.complex128), y)
        rhs = np.prod(Kd) * np.vdot(x.astype(np.complex128), A.adjoint(y))
        assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_torch_tensor_inputs_stay_on_device(NUFFT):
    import torch
    rng = np.random.default_rng(11)
    om = rng.uniform(-np.pi, np.pi, (500, 2))
    A = NUFFT(0)
    A.plan(torch.from_numpy(om).cuda(), (32, 32), (64, 64), (6, 6))
    x = cplx(rng, (32, 32))
    xt = torch.from_numpy(x).cuda()
    yt = A.forward(xt)
    assert isinstance(yt, torch.Tensor) and yt.is_cuda and yt.dtype == torch.complex64
    xp = torch.from_numpy(x).pin_memory()
    yp = A.forward(xp)
    assert isinstance(yp, torch.Tensor) and not yp.is_cuda
    np.testing.assert_array_equal(yt.cpu().numpy(), yp.numpy())
    np.testing.assert_array_equal(A.forward(x), yp.numpy())


def test_errors_are_reported(NUFFT):
    rng = np.random.default_rng(12)
    A = NUFFT(0)
    om = rng.uniform(-np.pi, np.pi, (100, 2))
    om[17, 1] = np.nan
    with pytest.raises(ValueError):
        A.plan(om, (16, 16), (32, 32), (6, 6))
    with pytest.raises(TypeError):
        A.plan(om, [16, 16], (32, 32), (6, 6))
    with pytest.raises(KeyError):
        A.plan(om, (16, 16), (32, 32), (6,))
    with pytest.raises(ValueError):        # Jd > Kd
        A.plan(rng.uniform(-1, 1, (10, 1)), (4,), (4,), (6,))
    A.plan(rng.uniform(-np.pi, np.pi, (100, 2)), (16, 16), (32, 32), (6, 6))
    with pytest.raises(ValueError):
        A.forward(np.zeros((16, 15), np.complex64))
    with pytest.raises(ValueError):
        A.adjoint(np.zeros((99,), np.complex64))


def test_single_point_and_far_out_points(NUFFT):
    """M = 1, and points far outside [-pi, pi) wrap modulo the grid exactly as
    the reference's mod-K indexing does."""
    rng = np.random.default_rng(13)
    Nd, Kd, Jd = (20, 24), (40, 48), (6, 6)
    x = cplx(rng, Nd)
    for om in [np.array([[0.3, -2.0]]), rng.uniform(-40.0, 40.0, (64, 2))]:
        A = NUFFT(0)
        A.plan(om, Nd, Kd, Jd)
        O = OracleNUFFT()
        O.plan(om, Nd, Kd, Jd)
        y = cplx(rng, (om.shape[0],))
        assert rel_l2(A.forward(x), O.forward(x)) < TOL
        assert rel_l2(A.adjoint(y), O.adjoint(y)) < TOL


def test_empty_trajectory(NUFFT):
    A = NUFFT(0)
    A.plan(np.zeros((0, 2)), (16, 16), (32, 32), (6, 6))
    assert A.forward(np.ones((16, 16), np.complex64)).shape == (0,)
    x = A.adjoint(np.zeros((0,), np.complex64))
    assert x.shape == (16, 16) and not np.any(x)


def test_forward_dom_is_the_trajectory_derivative(NUFFT):
    """dy/dom_d from forward_dom against central differences of the exact
    NUDFT (FP64, h = 1e-4)."""
    rng = np.random.default_rng(14)
    Nd, Kd, Jd = (24, 24), (48, 48), (6, 6)
    om = rng.uniform(-3.0, 3.0, (200, 2))
    x = cplx(rng, Nd)
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd)
    dy = A.forward_dom(x)
    h = 1e-4
    for d in range(2):
        e = np.zeros(2)
        e[d] = h
        fd = (nudft_forward_rows(x, om + e) - nudft_forward_rows(x, om - e)) / (2 * h)
        assert rel_l2(dy[d], fd) < 1e-5, rel_l2(dy[d], fd)


def test_full_size_3d_against_exact_nudft(NUFFT):
    """3D 128^3 / 256^3 / J6 at M = 2,000,000 uniform points: forward rows and
    adjoint pixels against the FP64 NUDFT on subsets, plus the adjoint
    identity at full size."""
    from pynufft_gb300.trajectories import ellipsoids, uniform
    Nd, Kd, Jd = (128, 128, 128), (256, 256, 256), (6, 6, 6)
    om = uniform(2_000_000, 3, seed=1)
    x = ellipsoids(Nd, 32, seed=2)
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd)
    y = A.forward(x)
    rows = np.random.default_rng(15).choice(om.shape[0], 512, replace=False)
    assert rel_l2(y[rows], nudft_forward_rows(x, om, rows)) < 1e-5
    rng = np.random.default_rng(16)
    yr = cplx(rng, (om.shape[0],))
    xa = A.adjoint(yr)
    pix = rng.choice(int(np.prod(Nd)), 64, replace=False)
    ref = nudft_adjoint_pixels(yr, om, Nd, pix) / np.prod(Kd)
    assert rel_l2(xa.ravel()[pix], ref) < 1e-5
    lhs = np.vdot(y.astype(np.complex128), yr)
    rhs = np.prod(Kd) * np.vdot(x.astype(np.complex128), xa)
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


@pytest.mark.parametrize('case', ['plan_1d', 'plan_2d', 'plan_3d', 'plan_3d_aniso', 'plan_2d_J8'])
@pytest.mark.parametrize('k2y,y2k', [('tile', 'zteam'), ('zteam', 'point'), ('point', 'global'),
                                     ('tile_point', 'point')])
def test_every_lane_mapping_matches_reference(NUFFT, case, k2y, y2k):
    g = load_golden(case)
    A = NUFFT(0)
    A.plan(g['om'], _tup(g['Nd']), _tup(g['Kd']), _tup(g['Jd']))
    A.set_methods(k2y, y2k)
    assert rel_l2(A.k2y(g['k']), g['k2y']) < TOL
    assert rel_l2(A.y2k(g['y']), g['y2k']) < TOL
    assert rel_l2(A.forward(g['x']), g['forward']) < TOL
    assert rel_l2(A.adjoint(g['y']), g['adjoint']) < TOL
    A.check()   # no kernel gave up a bounded wait for its bulk copies


@pytest.mark.parametrize('bins', [(4, 4), (16, 8), (64, 64)])
def test_bin_shapes_do_not_change_results(NUFFT, bins):
    g = load_golden('plan_2d')
    A = NUFFT(0)
    A.plan(g['om'], (32, 32), (64, 64), (6, 6), bins=bins, max_sub_points=64)
    assert rel_l2(A.y2k(g['y']), g['y2k']) < TOL
    assert rel_l2(A.k2y(g['k']), g['k2y']) < TOL


def test_autotune_picks_a_setting_and_keeps_results(NUFFT, tmp_path, monkeypatch):
    """The autotuner re-plans with the fastest candidate and caches it; the
    transform is unchanged."""
    from pynufft_gb300 import autotune
    monkeypatch.setattr(autotune, 'CACHE', str(tmp_path / 'tune.json'))
    g = load_golden('plan_3d')
    A = NUFFT(0)
    A.plan(g['om'], (12, 12, 12), (24, 24, 24), (6, 6, 6), autotune=True)
    assert autotune.cached(A) is not None and A.tuned['ms'] > 0
    assert rel_l2(A.forward(g['x']), g['forward']) < TOL
    assert rel_l2(A.adjoint(g['y']), g['adjoint']) < TOL
    B = NUFFT(0)
    B.plan(g['om'], (12, 12, 12), (24, 24, 24), (6, 6, 6), autotune=True)   # from the cache
    assert B.tuned == A.tuned


def test_replan_same_geometry_matches_fresh_plan(NUFFT):
    """plan() again with the same geometry keeps the plan and replaces only
    the points (and drops the captured CG graphs, which hold the old
    tables): results equal a fresh plan's."""
    rng = np.random.default_rng(21)
    Nd, Kd, Jd = (24, 20), (48, 40), (6, 6)
    om1 = rng.uniform(-np.pi, np.pi, (1500, 2))
    om2 = rng.uniform(-np.pi, np.pi, (2300, 2))
    x = cplx(rng, Nd)
    A = NUFFT(0)
    A.plan(om1, Nd, Kd, Jd)
    y1 = cplx(rng, (1500,))
    A.solve(y1, 'cg', maxiter=3)
    A.plan(om2, Nd, Kd, Jd)
    B = NUFFT(0)
    B.plan(om2, Nd, Kd, Jd)
    assert np.array_equal(A.forward(x), B.forward(x))
    y2 = cplx(rng, (2300,))
    assert rel_l2(A.adjoint(y2), B.adjoint(y2)) < 1e-6
    assert rel_l2(A.solve(y2, 'cg', maxiter=3), B.solve(y2, 'cg', maxiter=3)) < 1e-5


@pytest.mark.parametrize('case', ['plan_1d', 'plan_2d', 'plan_2d_odd', 'plan_3d', 'plan_2d_J8'])
def test_interpolator_tables_at_float_precision(NUFFT, case):
    """The per-point coefficient tables (FP64 per-axis table + cubic
    interpolation, stored complex64) reproduce the reference's complex128
    interpolator to float32 precision: k2y against the reference within 1e-6
    relative L2, an order of magnitude inside the 1e-5 parity bar."""
    g = load_golden(case)
    A = NUFFT(0)
    A.plan(g['om'], _tup(g['Nd']), _tup(g['Kd']), _tup(g['Jd']))
    assert rel_l2(A.k2y(g['k']), g['k2y']) < 1e-6


def test_cg_on_many_instances_and_coils_matches_oracle(NUFFT):
    """solve(y, 'cg') on a plan of several instances and coils runs one
    independent CG system per (instance, coil), with its own scalars and its
    own stopping test: each matches the oracle's CG on that instance and coil,
    and an all-zero system stops at once with x = 0."""
    rng = np.random.default_rng(31)
    Nd, Kd, Jd, B = (16, 18), (32, 36), (6, 6), 2
    Ms = [700, 1100, 400]
    oms = [rng.uniform(-np.pi, np.pi, (m, 2)) for m in Ms]
    A = NUFFT(0)
    A.plan_many(oms, Nd, Kd, Jd, batch=B)
    y = cplx(rng, (sum(Ms), B))
    y[Ms[0]:Ms[0] + Ms[1], 1] = 0          # instance 1, coil 1: b = 0
    x, it = A.solve(y, 'cg', maxiter=4, return_info=True)
    assert it == 4 and x.shape == (3,) + Nd + (B,)
    off = 0
    for i, om in enumerate(oms):
        O = OracleNUFFT()
        O.plan(om, Nd, Kd, Jd, batch=B)
        xo = O.solve(y[off:off + Ms[i]], 'cg', maxiter=4)
        for b in range(B):
            if i == 1 and b == 1:
                assert not np.any(x[i][..., b])
            else:
                assert rel_l2(x[i][..., b], xo[..., b]) < TOL
        off += Ms[i]


@pytest.mark.parametrize('B', [None, 4, 8])
def test_pinned_host_images_match_device_tensors(NUFFT, B):
    """Pinned CPU tensors: for one coil the image kernels read and write them
    in place through their device mapping (no copies), for several coils they
    go through copies; results equal the device-tensor path and the returned
    tensors are pinned CPU tensors."""
    import torch
    rng = np.random.default_rng(41)
    Nd, Kd, Jd = (24, 20, 16), (48, 40, 32), (6, 6, 6)
    M = 3000
    om = rng.uniform(-np.pi, np.pi, (M, 3))
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd, batch=B)
    tail = () if B is None else (B,)
    x = torch.from_numpy(cplx(rng, Nd + tail)).pin_memory()
    y = torch.from_numpy(cplx(rng, (M,) + tail)).pin_memory()
    k = torch.from_numpy(cplx(rng, Kd + tail)).pin_memory()
    xd, yd, kd = x.cuda(), y.cuda(), k.cuda()
    for name, arg, argd in [('forward', x, xd), ('adjoint', y, yd), ('selfadjoint', x, xd),
                            ('x2xx', x, xd), ('xx2x', x, xd), ('xx2k', x, xd), ('k2xx', k, kd)]:
        got = getattr(A, name)(arg)
        ref = getattr(A, name)(argd).cpu()
        assert not got.is_cuda and got.is_pinned(), name
        assert rel_l2(got.numpy(), ref.numpy()) < 1e-6, name


def test_bounded_wait_runs_out_and_the_context_stays_usable(NUFFT):
    """The bounded mbarrier wait of the bulk-copy kernels ends when its bytes
    never arrive (a self-test kernel arms 16 bytes that no copy delivers),
    reports it, and the GPU keeps working; a plan's own flag stays clear."""
    import ctypes
    from pynufft_gb300 import _lib
    L = _lib.load()
    t = ctypes.c_int(0)
    _lib.check(L.nufft_selftest_bounded_wait(1000, ctypes.byref(t)), 'selftest')
    assert t.value == 1
    g = load_golden('plan_2d')
    A = NUFFT(0)
    A.plan(g['om'], _tup(g['Nd']), _tup(g['Kd']), _tup(g['Jd']))
    assert rel_l2(A.forward(g['x']), g['forward']) < TOL
    A.check()


@pytest.mark.parametrize('Nd,Kd,Jd', [((10, 11, 9), (20, 23, 19), (5, 4, 6)),     # odd K, mixed J
                                      ((12, 10, 14), (24, 20, 28), (3, 7, 5)),
                                      ((30, 26), (61, 52), (7, 5))])
def test_odd_grids_and_mixed_J_match_oracle(NUFFT, Nd, Kd, Jd):
    """Grids whose innermost extent is odd take the thread-loaded tile path
    (no bulk copies), and unequal J per axis the guarded tap loops: both
    match the oracle for every stage."""
    rng = np.random.default_rng(51)
    M = 2500
    om = rng.uniform(-np.pi, np.pi, (M, len(Nd)))
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd)
    O = OracleNUFFT()
    O.plan(om, Nd, Kd, Jd)
    x = cplx(rng, Nd)
    y = cplx(rng, (M,))
    k = cplx(rng, Kd)
    assert rel_l2(A.k2y(k), O.k2y(k)) < TOL
    assert rel_l2(A.y2k(y), O.y2k(y)) < TOL
    assert rel_l2(A.forward(x), O.forward(x)) < TOL
    assert rel_l2(A.adjoint(y), O.adjoint(y)) < TOL
    A.check()


def test_kernel_timing_counts_the_launches(NUFFT):
    """nufft_plan_kernel_timing with period n brackets the 1st, (n+1)-th ...
    k2y / y2k kernel launches with CUDA events: period 1 times every launch,
    period 3 over five forward+adjoint pairs times launches 1 and 4."""
    import ctypes
    g = load_golden('plan_3d')
    A = NUFFT(0)
    A.plan(g['om'], _tup(g['Nd']), _tup(g['Kd']), _tup(g['Jd']))
    L, P = A._lib, A._plan
    km, ym = ctypes.c_double(), ctypes.c_double()
    kn, yn = ctypes.c_int(), ctypes.c_int()
    for period, pairs, timed in [(1, 1, 1), (3, 5, 2), (1, 4, 4)]:
        assert L.nufft_plan_kernel_timing(P, period) == 0
        for _ in range(pairs):
            A.forward(g['x'])
            A.adjoint(g['y'])
        assert L.nufft_plan_kernel_times(P, ctypes.byref(km), ctypes.byref(kn), ctypes.byref(ym),
                                         ctypes.byref(yn)) == 0
        assert kn.value == timed and yn.value == timed, (period, kn.value, yn.value)
        assert km.value > 0 and ym.value > 0
    assert L.nufft_plan_kernel_timing(P, -1) != 0
    L.nufft_plan_kernel_timing(P, 0)
    A.forward(g['x'])
    L.nufft_plan_kernel_times(P, ctypes.byref(km), ctypes.byref(kn), ctypes.byref(ym),
                              ctypes.byref(yn))
    assert kn.value == 0 and yn.value == 0


def test_adjoint_grid_zeroed_ahead_across_streams(NUFFT):
    """One-coil plans zero the adjoint's grid on a side stream during the
    forward: adjoints after a forward on another stream, repeated adjoints
    (zeroed inline) and a selfadjoint all match the oracle."""
    import torch
    g = load_golden('plan_3d')
    A = NUFFT(0)
    A.plan(g['om'], _tup(g['Nd']), _tup(g['Kd']), _tup(g['Jd']))
    O = OracleNUFFT()
    O.plan(g['om'], _tup(g['Nd']), _tup(g['Kd']), _tup(g['Jd']))
    ref_y, ref_x = O.forward(g['x']), O.adjoint(g['y'])
    xd = torch.from_numpy(g['x']).cuda()
    yd = torch.from_numpy(g['y']).cuda()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    for _ in range(3):
        with torch.cuda.stream(s1):
            yo = A.forward(xd)
        s2.wait_stream(s1)
        with torch.cuda.stream(s2):
            xo = A.adjoint(yd)
            xo2 = A.adjoint(yd)
        torch.cuda.synchronize()
        assert rel_l2(yo.cpu().numpy(), ref_y) < TOL
        assert rel_l2(xo.cpu().numpy(), ref_x) < TOL
        assert rel_l2(xo2.cpu().numpy(), ref_x) < TOL
    assert rel_l2(A.selfadjoint(g['x']), O.selfadjoint(g['x'])) < TOL
    A.check()

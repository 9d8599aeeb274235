"""NUFFT.run_many: operators applied to a sequence of host arrays, copies in
on an upload stream and out on a download stream around the transforms,
give the results of the methods called one at a time — bitwise on
deterministic plans, within float rounding of the gridding order on fast
plans (whose adjoint grid is zeroed on the plan's own side stream)."""
import numpy as np
import pytest

from oracle.nufft_oracle import rel_l2
from tests_util import cplx

pytestmark = pytest.mark.gpu


def _plan(B, ndim, deterministic, seed=11, M=3000):
    from pynufft_gb300 import NUFFT
    rng = np.random.default_rng(seed)
    om = rng.uniform(-np.pi, np.pi, (M, ndim))
    Nd, Kd, Jd = ((32,) * ndim, (64,) * ndim, (6,) * ndim) if ndim == 2 else \
        ((16,) * 3, (32,) * 3, (6,) * 3)
    A = NUFFT(0)
    A.plan(om, Nd, Kd, Jd, batch=B, deterministic=deterministic)
    return A, rng


def _jobs(A, rng, torch, n=3):
    sx, sy, sk = A._shape('x'), A._shape('y'), A._shape('k')
    jobs = []
    for i in range(n):
        x, y, k = cplx(rng, sx), cplx(rng, sy), cplx(rng, sk)
        jobs += [('forward', torch.from_numpy(x).pin_memory()),   # pinned
                 ('adjoint', y),                                  # numpy
                 ('selfadjoint', torch.from_numpy(x)),            # pageable tensor
                 ('xx2k', x), ('k2y', k), ('y2k', y), ('k2xx', k), ('k2y2k', k),
                 ('x2xx', x), ('xx2x', x)][: 10 if i == 0 else 3]
    return jobs


@pytest.mark.parametrize('B,ndim,depth,lanes', [(None, 2, 2, 1), (4, 2, 1, 2), (8, 3, 3, 1),
                                                (8, 3, 2, 3), (None, 3, 2, 2)])
def test_run_many_equals_single_calls_bitwise(B, ndim, depth, lanes):
    import torch
    A, rng = _plan(B, ndim, True)
    jobs = _jobs(A, rng, torch)
    outs = A.run_many(jobs, depth=depth, lanes=lanes)
    assert len(A._twins) == lanes - 1
    assert len(outs) == len(jobs)
    for (name, a), o in zip(jobs, outs):
        assert o.is_pinned() and o.dtype == torch.complex64
        ref = np.asarray(getattr(A, name)(a))
        assert np.array_equal(o.numpy(), ref), name


@pytest.mark.parametrize('lanes', [1, 2])
def test_run_many_fast_plan_and_out_buffers(lanes):
    import torch
    A, rng = _plan(None, 3, False, M=20000)
    jobs = _jobs(A, rng, torch, n=6)
    out = [torch.empty(A._shape(A._STAGES[n][1]), dtype=torch.complex64).pin_memory()
           for n, _ in jobs]
    got = A.run_many(jobs, out=out, lanes=lanes)
    assert all(g is o for g, o in zip(got, out))
    for (name, a), o in zip(jobs, out):
        ref = np.asarray(getattr(A, name)(a))
        assert rel_l2(o.numpy(), ref) < 1e-6, name


def test_run_many_rejects_bad_jobs():
    import torch
    A, rng = _plan(None, 2, False)
    x = cplx(rng, A._shape('x'))
    with pytest.raises(ValueError):
        A.run_many([('solve', x)])
    with pytest.raises(ValueError):
        A.run_many([('forward', torch.from_numpy(x).cuda())])
    with pytest.raises(ValueError):
        A.run_many([('adjoint', x)])                      # an image where samples go
    with pytest.raises(ValueError):
        A.run_many([('forward', x)], out=[torch.empty(3, dtype=torch.complex64)])
    with pytest.raises(ValueError):
        A.run_many([('forward', x)], depth=0)
    with pytest.raises(ValueError):
        A.run_many([('forward', x)], lanes=0)


def test_run_many_lanes_follow_the_plan():
    """Twin operators take the plan's points, instances, bins and transform
    choice, and are dropped when the points or the methods change."""
    import torch
    from pynufft_gb300 import NUFFT
    rng = np.random.default_rng(5)
    oms = [rng.uniform(-np.pi, np.pi, (m, 2)) for m in (700, 1300, 400)]
    A = NUFFT(0)
    A.plan_many(oms, (32, 32), (64, 64), (6, 6), batch=2, deterministic=True,
                bins=(8, 16))
    xs = [cplx(rng, A._shape('x')) for _ in range(4)]
    jobs = [('forward', x) for x in xs] + [('selfadjoint', x) for x in xs]
    outs = A.run_many(jobs, lanes=2)
    assert len(A._twins) == 1 and A._twins[0]._key == A._key
    for (name, a), o in zip(jobs, outs):
        assert np.array_equal(o.numpy(), np.asarray(getattr(A, name)(a))), name
    om2 = rng.uniform(-np.pi, np.pi, (900, 2))
    B = NUFFT(0)
    B.plan(om2, (32, 32), (64, 64), (6, 6), deterministic=True, fft='own')
    x = cplx(rng, B._shape('x'))
    got = B.run_many([('forward', x), ('forward', x), ('adjoint', np.asarray(B.forward(x)))],
                     lanes=2)
    assert B._twins[0].fft == 'own'
    assert np.array_equal(got[0].numpy(), got[1].numpy())
    assert np.array_equal(got[1].numpy(), np.asarray(B.forward(x)))
    B.plan(rng.uniform(-np.pi, np.pi, (500, 2)), (32, 32), (64, 64), (6, 6),
           deterministic=True, fft='own')
    assert B._twins == []
    got = B.run_many([('forward', x), ('forward', x)], lanes=2)
    assert got[0].shape == (500,) and np.array_equal(got[1].numpy(), np.asarray(B.forward(x)))

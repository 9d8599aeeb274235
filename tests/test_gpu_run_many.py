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


@pytest.mark.parametrize('B,ndim,depth', [(None, 2, 2), (4, 2, 1), (8, 3, 3), (None, 3, 2)])
def test_run_many_equals_single_calls_bitwise(B, ndim, depth):
    import torch
    A, rng = _plan(B, ndim, True)
    jobs = _jobs(A, rng, torch)
    outs = A.run_many(jobs, depth=depth)
    assert len(outs) == len(jobs)
    for (name, a), o in zip(jobs, outs):
        assert o.is_pinned() and o.dtype == torch.complex64
        ref = np.asarray(getattr(A, name)(a))
        assert np.array_equal(o.numpy(), ref), name


def test_run_many_fast_plan_and_out_buffers():
    import torch
    A, rng = _plan(None, 3, False, M=20000)
    jobs = _jobs(A, rng, torch, n=6)
    out = [torch.empty(A._shape(A._STAGES[n][1]), dtype=torch.complex64).pin_memory()
           for n, _ in jobs]
    got = A.run_many(jobs, out=out)
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

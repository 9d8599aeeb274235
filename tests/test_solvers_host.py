"""The Krylov recursions of pynufft_gb300.solvers (bicg, bicgstab, gmres,
lgmres) restate scipy.sparse.linalg's, which the reference calls on its
normal operator (linalg/solve_cpu.py:253-288).  On the CPU, with the oracle's
complex128 spH.sp as the operator on torch tensors, they must reproduce
scipy's iterates to rounding."""
import numpy as np
import pytest
import scipy.sparse.linalg as sla

from oracle.nufft_oracle import OracleNUFFT, rel_l2


@pytest.fixture(scope='module')
def system():
    rng = np.random.default_rng(2)
    om = rng.uniform(-np.pi, np.pi, (1500, 2))
    y = (rng.standard_normal(1500) + 1j * rng.standard_normal(1500)).astype(np.complex64)
    O = OracleNUFFT()
    O.plan(om, (24, 24), (48, 48), (6, 6))
    b = np.reshape(O._y2k1(y), (-1,))
    return O, b


@pytest.mark.parametrize('solver,kw', [('bicg', {}), ('bicgstab', {}), ('gmres', {'restart': 5}),
                                       ('gmres', {}), ('lgmres', {'inner_m': 5}),
                                       ('lgmres', {'inner_m': 4, 'outer_k': 1})])
@pytest.mark.parametrize('maxiter', [1, 4])
def test_recursions_match_scipy(system, solver, kw, maxiter):
    import torch
    from pynufft_gb300 import solvers
    O, b = system
    n = b.size

    def spHsp(v):
        return O.spH.dot(O.sp.dot(v))
    A = sla.LinearOperator((n, n), matvec=spHsp, rmatvec=spHsp, dtype=np.complex128)
    ref, info = getattr(sla, solver)(A, b, rtol=1e-5, atol=0.0, maxiter=maxiter, **kw)

    def At(v):
        return torch.from_numpy(spHsp(v.numpy()))
    bt = torch.from_numpy(b)
    got, ginfo = solvers.KRYLOV[solver](At, bt, torch.zeros_like(bt), rtol=1e-5, atol=0.0,
                                        maxiter=maxiter, **kw)
    assert ginfo == info
    assert rel_l2(got.numpy(), ref) < 1e-10, rel_l2(got.numpy(), ref)


@pytest.mark.parametrize('solver', ['bicg', 'bicgstab', 'gmres', 'lgmres'])
def test_recursions_stop_at_the_tolerance_like_scipy(system, solver):
    """A loose rtol stops early with info 0, as scipy does."""
    import torch
    from pynufft_gb300 import solvers
    O, b = system
    n = b.size

    def spHsp(v):
        return O.spH.dot(O.sp.dot(v))
    A = sla.LinearOperator((n, n), matvec=spHsp, rmatvec=spHsp, dtype=np.complex128)
    ref, info = getattr(sla, solver)(A, b, rtol=0.3, atol=0.0, maxiter=50)
    got, ginfo = solvers.KRYLOV[solver](lambda v: torch.from_numpy(spHsp(v.numpy())),
                                        torch.from_numpy(b), torch.zeros(n, dtype=torch.complex128),
                                        rtol=0.3, atol=0.0, maxiter=50)
    assert info == 0 and ginfo == 0
    assert rel_l2(got.numpy(), ref) < 1e-10

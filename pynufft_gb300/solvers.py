"""Solvers other than 'cg' for ``NUFFT.solve`` (linalg/solve_cpu.py:185-288)."""
from __future__ import annotations


def solve(nufft, y, solver, *args, maxiter=None, **kwargs):
    if solver in ('cgs', 'qmr', 'minres'):
        raise TypeError(solver + ' requires real symmetric matrix')
    raise NotImplementedError(f"solver {solver!r} is not available; use 'cg'")

"""Autotuner for the gridding/interpolation kernels.

For a planned ``NUFFT`` it times one interpolation (k2y) plus one gridding
(y2k) for each candidate setting -- bin shape, largest sub-problem, and the
lane mapping of each kernel -- with CUDA events, keeps the fastest, and
caches the choice on disk keyed by the geometry (ndim, Nd, Kd, Jd, coils,
instances) and the point density class (log2 of points per grid cell).
``NUFFT.plan(..., autotune=True)`` applies a cached choice or tunes once.
Every candidate computes the same operator; only speed differs.
"""
from __future__ import annotations

import itertools
import json
import math
import os
import time
from ctypes import c_void_p

CACHE = os.environ.get('PYNUFFT_GB300_TUNE_CACHE',
                       os.path.join(os.path.expanduser('~'), '.cache', 'pynufft_gb300', 'tune.json'))

BIN_CANDIDATES = {
    1: [(512,), (1024,), (2048,)],
    2: [(16, 16), (32, 32), (32, 64), (64, 64)],
    3: [(8, 8, 8), (8, 8, 16), (8, 16, 16), (16, 16, 16)],
}
SUB_CANDIDATES = [128, 256, 512]
K2Y = ['tile', 'tile_point', 'zteam', 'point']
Y2K = ['zteam', 'point', 'global']


def key_of(op) -> str:
    M = sum(op.counts)
    cells = op.Kdprod * op.ninst
    dens = round(math.log2(max(M, 1) / cells)) if M else -99
    return json.dumps([op.ndims, list(op.Nd), list(op.Kd), list(op.Jd), op.B, op.ninst, dens])


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(db):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + '.tmp'
    with open(tmp, 'w') as f:
        json.dump(db, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def _time_pair(op, reps=3):
    import torch
    dev = op.device
    st = torch.cuda.current_stream(dev)
    sp = c_void_p(st.cuda_stream)
    g = torch.zeros(op._shape('k'), dtype=torch.complex64, device=dev)
    y = torch.zeros(op._shape('y'), dtype=torch.complex64, device=dev)
    L, P = op._lib, op._plan

    def once():
        L.nufft_k2y(P, c_void_p(g.data_ptr()), c_void_p(y.data_ptr()), sp)
        L.nufft_y2k(P, c_void_p(y.data_ptr()), c_void_p(g.data_ptr()), sp)
    once()
    torch.cuda.synchronize(dev)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        once()
    b.record(st)
    torch.cuda.synchronize(dev)
    return a.elapsed_time(b) / reps


def tune(op, om, budget_s: float = 60.0, write_cache: bool = True):
    """Search the candidates for the planned `op` (whose points are `om`, or
    a list of per-instance arrays for a many-instance plan); re-plans `op`
    with the best setting and returns it as a dict."""
    coils_split = op.B >= 8
    k2ys = [None] if coils_split else K2Y
    y2ks = [None] if coils_split else Y2K
    oms = om if isinstance(om, (list, tuple)) else [om]
    best = None
    t0 = time.time()
    for bins, msub in itertools.product(BIN_CANDIDATES[op.ndims], SUB_CANDIDATES):
        if time.time() - t0 > budget_s:
            break
        bins = tuple(min(b, k) for b, k in zip(bins, op.Kd))
        _replan(op, oms, bins, msub)
        for k2y, y2k in itertools.product(k2ys, y2ks):
            op.set_methods(k2y, y2k)
            t = _time_pair(op)
            if best is None or t < best['ms']:
                best = {'bins': list(bins), 'max_sub_points': msub, 'k2y': k2y, 'y2k': y2k, 'ms': t}
    apply(op, oms, best)
    if write_cache:
        db = _load()
        db[key_of(op)] = best
        _save(db)
    return best


def _replan(op, oms, bins, msub):
    det = getattr(op, 'deterministic', False)
    if op.ninst > 1:
        op.plan_many(oms, op.Nd, op.Kd, op.Jd, batch=op.batch, deterministic=det,
                     bins=bins, max_sub_points=msub)
    else:
        op.plan(oms[0], op.Nd, op.Kd, op.Jd, batch=op.batch, deterministic=det,
                bins=bins, max_sub_points=msub, fft=getattr(op, 'fft', 'auto'))


def apply(op, oms, choice):
    _replan(op, oms, tuple(choice['bins']), choice['max_sub_points'])
    op.set_methods(choice.get('k2y'), choice.get('y2k'))
    op.tuned = dict(choice)


def cached(op):
    return _load().get(key_of(op))

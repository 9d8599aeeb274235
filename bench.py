"""Benchmark: NUFFT forward+adjoint pairs/s on one GB300 (per GPU, replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config c1|c2|c3|c4|c5]

Default workload (c2): 3D Nd 128^3, Kd 256^3, Jd 6^3, M = 2,000,000 points
i.i.d. uniform in [-pi, pi)^3, complex64 image of 32 random ellipsoids.  One
step = one forward + one adjoint NUFFT.  The plan's per-point tables (312 MB)
and the oversampled grid (134 MB) exceed the 129 MB L2, so no flush is needed
between steps.

Prints ONE JSON line (rank 0).  `value` times steps with inputs resident on
the device (CUDA events on the launching stream); `e2e` times the public API
(`NUFFT.forward`/`adjoint` on pinned host tensors, copies included);
`roofline` uses the dominant kernel's own average duration, from CUDA events
that the library records around every n-th of its launches (about 20 spread
over the timed steps) on the launching stream;
`cpu_baseline` times the CPU oracle (a restatement of the reference numpy
path) on a bounded sample.  With --gpus N > 1 (torchrun) every rank runs an
independent replica of the workload (no collective on the data path) and
`value` is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0
L2_BYTES = 129 * 1024 * 1024      # GB300 L2
FLUSH_BYTES = 512 * 1024 * 1024   # written between timed steps when a step's data fits in L2

CONFIGS = {
    'c1': dict(name='2D radial 256 spokes x 512 samples (M=131072), Nd 256^2, Kd 512^2, Jd 6^2, fwd+adj pair',
               Nd=(256, 256), Kd=(512, 512), Jd=(6, 6), batch=None),
    'c2': dict(name='3D uniform M=2,000,000, Nd 128^3, Kd 256^3, Jd 6^3, fwd+adj pair',
               Nd=(128, 128, 128), Kd=(256, 256, 256), Jd=(6, 6, 6), batch=None),
    'c3': dict(name='2D golden-angle radial 400x640 (M=256000), Nd 320^2, Kd 640^2, Jd 6^2, 32 coils, fwd+adj pair',
               Nd=(320, 320), Kd=(640, 640), Jd=(6, 6), batch=32),
    'c4': dict(name='2D spiral 32x2048 (M=65536), Nd 256^2, Kd 512^2, Jd 6^2, 8 coils, fwd+adj pair',
               Nd=(256, 256), Kd=(512, 512), Jd=(6, 6), batch=8),
    'c5': dict(name='3D kooshball 15625x512 (M=8,000,000), Nd 192^3, Kd 384^3, Jd 6^3, 8 coils, fwd+adj pair',
               Nd=(192, 192, 192), Kd=(384, 384, 384), Jd=(6, 6, 6), batch=8),
    'c3i': dict(name='64 independent 2D uniform instances, M ~ U{20000..200000} each, Nd 320^2, Kd 640^2, '
                     'Jd 6^2, one fwd+adj of every instance per step (a pair = one instance)',
                Nd=(320, 320), Kd=(640, 640), Jd=(6, 6), batch=None, ninst=64),
}


def workload(cfg: str):
    from pynufft_gb300 import trajectories as T
    c = CONFIGS[cfg]
    if cfg == 'c1':
        om = T.radial_2d(256, 512)
        x = T.random_image(c['Nd'], seed=0)
    elif cfg == 'c2':
        om = T.uniform(2_000_000, 3, seed=1)
        x = T.ellipsoids(c['Nd'], 32, seed=2)
    elif cfg == 'c3':
        om = T.radial_2d(400, 640, golden=True)
        x = T.random_image(c['Nd'] + (32,), seed=0)
    elif cfg == 'c4':
        om = T.spiral_2d(32, 2048, seed=6)
        x = T.random_image(c['Nd'] + (8,), seed=0)
    elif cfg == 'c3i':
        om = T.uneven_instances(c['ninst'], seed=5)
        x = T.random_image((c['ninst'],) + c['Nd'], seed=0)
    else:
        om = T.kooshball_3d(15625, 512)
        x = T.random_image(c['Nd'] + (8,), seed=0)
    return c, om, x


def alg_bytes(c, M):
    """Algorithmic bytes of one gridding (y2k) or interpolation (k2y) launch:
    per-point tables (c64 coefficients + int32 base index per axis) read once,
    plus C coils of samples and of the oversampled grid."""
    d = len(c['Nd'])
    C = c['batch'] or 1
    meta = 8 * sum(c['Jd']) + 4 * d
    return M * meta + C * (8 * M + 8 * int(np.prod(c['Kd'])) * c.get('ninst', 1))


def peaks():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return float(j['hbm_gbs']), 'measured'
    return FALLBACK_HBM_GBS, 'fallback'


def traffic_from_profiles(cfg, kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    p = os.path.join(ROOT, 'profiles', 'dram_traffic.json')
    if not os.path.exists(p):
        return None
    with open(p) as f:
        j = json.load(f)
    return j.get(cfg, {}).get(kernel)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', f'--query-gpu={self.Q}', '--format=csv,noheader,nounits',
                 '-lms', '200', '-i', str(self.index)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.6)

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        time.sleep(0.3)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, pw, reasons = [], [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in out.strip().splitlines():
            f = [t.strip() for t in line.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
                pw.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == 'active':
                    reasons.add(n)
        return {'sm_mhz': float(np.median(sm)) if sm else None,
                'sm_max_mhz': max(mx) if mx else None,
                'power_w_max': max(pw) if pw else None,
                'samples': len(sm), 'reasons': sorted(reasons)}


def cpu_baseline(cfg, c, om, x, threads=1, steps=1, warmup=0, sample_points=100_000):
    """Time the CPU oracle (numpy FFT + scipy CSR, the reference's algorithm)
    on a bounded sample: the FFT stages on the full grid, the sparse stages on
    `sample_points` points, scaled linearly to the full M."""
    from oracle.nufft_oracle import OracleNUFFT
    M = om.shape[0]
    ms = min(M, sample_points)
    rng = np.random.default_rng(123)
    sel = np.sort(rng.choice(M, ms, replace=False)) if ms < M else np.arange(M)
    O = OracleNUFFT()
    t0 = time.perf_counter()
    O.plan(om[sel], c['Nd'], c['Kd'], c['Jd'], batch=c['batch'], threads=threads)
    t_plan = time.perf_counter() - t0
    scale = M / ms
    times = []
    for it in range(warmup + steps):
        t0 = time.perf_counter()
        k = O.xx2k(O.x2xx(x))
        t1 = time.perf_counter()
        y = O.k2y(k)
        t2 = time.perf_counter()
        kk = O.y2k(y)
        t3 = time.perf_counter()
        O.xx2x(O.k2xx(kk))
        t4 = time.perf_counter()
        if it >= warmup:
            times.append((t1 - t0) + (t4 - t3) + scale * ((t2 - t1) + (t3 - t2)))
    t_pair = float(np.median(times))
    sample = (f'{ms} of {M} points ({ms / M:.1%}); FFT/scale stages on the full grid, '
              f'sparse k2y/y2k timed on the sample and scaled x{scale:.1f}; plan {t_plan:.1f} s')
    return 1.0 / t_pair, sample, t_pair


def run_reference(args, cfg, rank):
    """--impl reference: the CPU oracle (restating the reference numpy NUFFT)
    with all host threads, same metric/unit, each step a bounded sample."""
    if rank != 0:
        return
    c, om, x = workload(cfg)
    if c.get('ninst', 1) > 1:
        print(json.dumps({'impl': 'reference', 'unavailable': 'the CPU reference arm times '
                          'single-instance configurations only'}), flush=True)
        return
    threads = os.cpu_count() or 1
    v, sample, t_pair = cpu_baseline(cfg, c, om, x, threads=threads, steps=args.steps,
                                     warmup=args.warmup)
    line = {
        'impl': 'reference', 'metric': 'NUFFT fwd+adj pairs/s', 'value': v, 'unit': 'pairs/s',
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': 1e3 * t_pair, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'c64 FFT / c128 CSR', 'data': 'synthetic',
        'config': {'workload': c['name'], 'l2': 'host run'},
        'cpu_baseline': {'value': v, 'unit': 'pairs/s', 'cores': threads, 'kind': 'port',
                         'sample': sample},
        'e2e': {'value': v, 'unit': 'pairs/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=200)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--config', default='c2', choices=sorted(CONFIGS))
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline leg')
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if args.impl == 'reference':
        run_reference(args, args.config, rank)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=torch.device('cuda', local))

    from pynufft_gb300 import NUFFT, _lib
    c, om, x = workload(args.config)
    dev = torch.device('cuda', local)
    A = NUFFT(dev)
    ninst = c.get('ninst', 1)

    def make_plan():
        if ninst > 1:
            A.plan_many(om, c['Nd'], c['Kd'], c['Jd'], batch=c['batch'])
        else:
            A.plan(om, c['Nd'], c['Kd'], c['Jd'], batch=c['batch'])
    make_plan()
    torch.cuda.synchronize()
    t0 = time.perf_counter()       # second plan: host om, tables rebuilt, no first-use costs
    make_plan()
    torch.cuda.synchronize()
    plan_ms = (time.perf_counter() - t0) * 1e3
    M = sum(o.shape[0] for o in om) if ninst > 1 else om.shape[0]
    xd = torch.from_numpy(x).to(dev)
    yd = torch.empty(A._shape('y'), dtype=torch.complex64, device=dev)
    xo = torch.empty_like(xd)
    lib = A._lib
    from ctypes import c_void_p
    stream = torch.cuda.current_stream(dev)
    sp = c_void_p(stream.cuda_stream)

    def step():
        lib.nufft_forward(A._plan, c_void_p(xd.data_ptr()), c_void_p(yd.data_ptr()), sp)
        lib.nufft_adjoint(A._plan, c_void_p(yd.data_ptr()), c_void_p(xo.data_ptr()), sp)

    # working set of one step: per-point tables + samples + grid + image
    ws_bytes = M * (8 * sum(c['Jd']) + 4 * len(c['Nd'])) + 8 * (M + ninst * (np.prod(c['Kd']) + np.prod(c['Nd']))) * (c['batch'] or 1)
    flush = ws_bytes < L2_BYTES
    scratch = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device=dev) if flush else None

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # the dominant kernels' own durations, from CUDA events the library
    # records around every period-th k2y / y2k launch on the launching stream
    # during the timed steps (about 20 samples spread over the timed region;
    # an event pair around every launch costs short steps ~10%)
    t_period = max(1, args.steps // 20)
    lib.nufft_plan_kernel_timing(A._plan, t_period)
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if flush:
        # inputs fit in L2: overwrite L2 with a larger buffer between steps,
        # outside the per-step events
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        for a, b in evs:
            scratch.fill_(1)
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in evs)
    else:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
    if dist:
        dist.barrier()
    clk = clocks.stop()
    from ctypes import byref, c_double, c_int
    k_ms, y_ms, k_n, y_n = c_double(), c_double(), c_int(), c_int()
    lib.nufft_plan_kernel_times(A._plan, byref(k_ms), byref(k_n), byref(y_ms), byref(y_n))
    lib.nufft_plan_kernel_timing(A._plan, 0)
    t_k2y = k_ms.value / max(k_n.value, 1)
    t_y2k = y_ms.value / max(y_n.value, 1)
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = world * ninst * args.steps / (ms / 1e3)   # many-instance configs count instance pairs
    # own kernels per step (cuFFT kernels are the library's): with the own
    # pruned FFT passes, one pass per axis each way plus k2y and y2k; else
    # pad, k2y, y2k, crop, and with several coils the two coil transposes
    fkind = c_int(-1)
    lib.nufft_plan_transform_kind(A._plan, byref(fkind))
    if fkind.value == _lib.NUFFT_FFT_OWN_PRUNED:
        launches_per_step = 2 * len(c['Nd']) + 2
    else:
        launches_per_step = 4 if (c['batch'] or 1) == 1 else 6

    # dominant kernel alone: k2y and y2k, CUDA events on the launching stream
    def time_call(fn, reps=20):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        if flush:
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(reps)]
            for a, b in evs:
                scratch.fill_(1)
                a.record(stream)
                fn()
                b.record(stream)
            torch.cuda.synchronize()
            return sum(a.elapsed_time(b) for a, b in evs) / reps
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    nbytes = alg_bytes(c, M)
    peak, peak_kind = peaks()
    dom = 'y2k' if t_y2k >= t_k2y else 'k2y'
    t_dom = max(t_y2k, t_k2y)
    ach = nbytes / (t_dom / 1e3) / 1e9
    traffic = traffic_from_profiles(args.config, dom)

    # solve(y, 'cg', maxiter=20) on noisy samples (SNR 30 dB) of the workload
    cg = None
    if c['batch'] is None:
        from pynufft_gb300.trajectories import add_noise
        from ctypes import byref, c_int
        lib.nufft_forward(A._plan, c_void_p(xd.data_ptr()), c_void_p(yd.data_ptr()), sp)
        torch.cuda.synchronize()
        yn = torch.from_numpy(add_noise(yd.cpu().numpy(), 30.0, seed=3)).to(dev)
        xs = torch.empty_like(xd)
        it = c_int(0)

        cg_iters = 15 if ninst > 1 else 20    # c3 many-instance: 15 per instance; c2: 20

        def solve():
            lib.nufft_solve_cg(A._plan, c_void_p(yn.data_ptr()), c_void_p(xs.data_ptr()), cg_iters,
                               1e-5, 0.0, None, sp)
        t_cg = time_call(solve, reps=5)
        lib.nufft_solve_cg(A._plan, c_void_p(yn.data_ptr()), c_void_p(xs.data_ptr()), cg_iters,
                           1e-5, 0.0, byref(it), sp)
        cg = {'maxiter': cg_iters, 'iters': it.value, 'ms': t_cg, 'systems': ninst}

    # end to end through the public API, pinned host buffers, copies included
    xh = torch.from_numpy(x).pin_memory()
    for _ in range(2):
        yh = A.forward(xh)
        A.adjoint(yh)
    torch.cuda.synchronize()
    e2e_steps = max(3, min(args.steps, 50))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        yh = A.forward(xh)
        xr = A.adjoint(yh)
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / e2e_steps / ninst
    if dist:
        t = torch.tensor([t_e2e], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    h2d = (xh.numel() + yh.numel()) * 8
    d2h = (yh.numel() + xr.numel()) * 8

    cpu = None
    if rank == 0 and not args.no_cpu and ninst == 1:
        v, sample, _ = cpu_baseline(args.config, c, om, x, threads=1)
        cpu = {'value': v, 'unit': 'pairs/s', 'cores': 1, 'kind': 'port', 'sample': sample}

    if rank == 0:
        line = {
            'metric': 'NUFFT fwd+adj pairs/s', 'value': value, 'unit': 'pairs/s',
            'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': ms_per_step, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'c64', 'data': 'synthetic',
            'config': {'workload': c['name'], 'parallelism': f'replicas x{world}',
                       'l2': (('L2 flushed between timed steps (%d MB written; step data %.0f MB)'
                               % (FLUSH_BYTES >> 20, ws_bytes / 1e6)) if flush else
                              'inputs larger than L2 (per-point tables %.0f MB + grid %.0f MB)' % (
                                  M * (8 * sum(c['Jd']) + 4 * len(c['Nd'])) / 1e6,
                                  8 * np.prod(c['Kd']) * (c['batch'] or 1) * ninst / 1e6))},
            'roofline': {'bound': 'hbm', 'kernel': dom, 'achieved': ach, 'peak': peak,
                         'unit': 'GB/s', 'frac': ach / peak, 'peak_kind': peak_kind,
                         'traffic': traffic, 'alg_bytes': nbytes, 'ms': t_dom,
                         'timed_launches': y_n.value if dom == 'y2k' else k_n.value},
            'gridding': {'kernel': 'y2k', 'ms': t_y2k, 'gbs': nbytes / (t_y2k / 1e3) / 1e9,
                         'frac': nbytes / (t_y2k / 1e3) / 1e9 / peak},
            'interp': {'kernel': 'k2y', 'ms': t_k2y, 'gbs': nbytes / (t_k2y / 1e3) / 1e9,
                       'frac': nbytes / (t_k2y / 1e3) / 1e9 / peak},
            'cpu_baseline': cpu,
            'e2e': {'value': world / t_e2e, 'unit': 'pairs/s', 'h2d_bytes_per_step': h2d,
                    'd2h_bytes_per_step': d2h},
            'gpu_launches': launches_per_step * args.steps,
            'plan_ms': plan_ms,
            'cg': cg,
            'clocks': clk,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == '__main__':
    main()

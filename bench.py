"""Benchmark: NUFFT forward+adjoint pairs/s on one GB300 (per GPU, replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config c1|c2|c3|c3i|c4|c5|c5s]

Default workload (c2): 3D Nd 128^3, Kd 256^3, Jd 6^3, M = 2,000,000 points
i.i.d. uniform in [-pi, pi)^3, complex64 image of 32 random ellipsoids.  One
step = one forward + one adjoint NUFFT.  The plan's per-point tables (312 MB)
and the oversampled grid (134 MB) exceed the 129 MB L2, so no flush is needed
between steps.

Prints ONE JSON line (rank 0).  `value` times steps with inputs resident on
the device (CUDA events on the launching stream); `e2e` times the public API
on pinned host tensors, every step's copies in and out included
(`NUFFT.run_many`, which overlaps one step's copies with the neighbouring
steps' transforms and, on workloads whose step takes 0.1 ms or more on the
device, runs alternate jobs on a twin operator of the same points on a
second stream; `e2e_sync`: `NUFFT.forward`/`adjoint` one call at a time);
`roofline` uses the dominant kernel's own average duration, from CUDA events
that the library records around every n-th of its launches (about 20 spread
over the timed steps) on the launching stream;
`cpu_baseline` times the CPU oracle (a restatement of the reference numpy
path: numpy FFT + scipy CSR products, one thread as in the reference) on one
full forward+adjoint pair of the same workload after one warm-up pair;
`batched` times the multi-coil workloads (2D golden-angle radial with 32
coils; 3D kooshball with 8 coils in the deterministic gridding mode) against
the same coils run one after another as single-coil transforms of the same
points on the same GPU.  With --gpus N > 1 (torchrun) every rank runs an
independent replica of the workload (no collective on the data path) and
`value` is the sum over ranks.

`--impl reference` times the oracle on the host for the same workload: the
full plan, then --warmup untimed and --steps timed full forward+adjoint
pairs, single-threaded like the reference's numpy/scipy calls (`value`),
plus two pairs with the oracle's threaded products on every host core
(`threaded`).
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
    # a small case of the kooshball workload (same points per cell), for
    # kernel captures that must stay small
    'c5s': dict(name='3D kooshball 3906x256 (M=999,936), Nd 96^3, Kd 192^3, Jd 6^3, 8 coils, fwd+adj pair '
                     '(small case of the 8M-point kooshball)',
                Nd=(96, 96, 96), Kd=(192, 192, 192), Jd=(6, 6, 6), batch=8),
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
    elif cfg == 'c5s':
        om = T.kooshball_3d(3906, 256)
        x = T.random_image(c['Nd'] + (8,), seed=0)
    else:
        om = T.kooshball_3d(15625, 512)
        x = T.random_image(c['Nd'] + (8,), seed=0)
    return c, om, x


def n_points(om):
    return sum(o.shape[0] for o in om) if isinstance(om, list) else om.shape[0]


def step_bytes(c, M):
    """Per-point tables + samples + grid + image of one step (device working set)."""
    B = c['batch'] or 1
    ninst = c.get('ninst', 1)
    return M * (8 * sum(c['Jd']) + 4 * len(c['Nd'])) + \
        8 * (M + ninst * (int(np.prod(c['Kd'])) + int(np.prod(c['Nd'])))) * B


def bench_config(cfg, world=1):
    """The `config` object of the JSON line, identical in both arms."""
    c = CONFIGS[cfg]
    M = CONFIG_POINTS[cfg]
    if M is None:
        M = n_points(workload(cfg)[1])
    B = c['batch'] or 1
    ninst = c.get('ninst', 1)
    ws = step_bytes(c, M)
    if ws < L2_BYTES:
        l2 = 'L2 flushed between timed steps (%d MB written; step data %.0f MB)' % (
            FLUSH_BYTES >> 20, ws / 1e6)
    else:
        l2 = 'inputs larger than L2 (per-point tables %.0f MB + grid %.0f MB)' % (
            M * (8 * sum(c['Jd']) + 4 * len(c['Nd'])) / 1e6,
            8 * np.prod(c['Kd']) * B * ninst / 1e6)
    return {'workload': c['name'], 'parallelism': f'replicas x{world}', 'l2': l2}


CONFIG_POINTS = {'c1': 256 * 512, 'c2': 2_000_000, 'c3': 400 * 640, 'c4': 32 * 2048,
                 'c5': 15625 * 512, 'c3i': None, 'c5s': 3906 * 256}


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


def cpu_pairs(c, om, x, steps, warmup, threads=1, build_threads=None):
    """Time the CPU oracle (numpy FFT + scipy CSR, the reference's algorithm)
    on the full workload: plan once (CSR built with `build_threads`), then
    `warmup` untimed and `steps` timed forward+adjoint pairs with `threads`
    host threads.  Returns (seconds of each timed pair, plan seconds, oracle)."""
    from oracle.nufft_oracle import OracleNUFFT
    O = OracleNUFFT()
    t0 = time.perf_counter()
    O.plan(om, c['Nd'], c['Kd'], c['Jd'], batch=c['batch'], threads=threads,
           build_threads=build_threads or threads)
    t_plan = time.perf_counter() - t0
    times = []
    for it in range(warmup + steps):
        t0 = time.perf_counter()
        O.adjoint(O.forward(x))
        if it >= warmup:
            times.append(time.perf_counter() - t0)
    return times, t_plan, O


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(cfg, c, om, x):
    """One full pair of the workload on one host thread after one warm-up pair
    (the reference's numpy FFT and scipy CSR products are single-threaded);
    the CSR is built with every host core to keep the plan short."""
    cores = host_cores()
    times, t_plan, _ = cpu_pairs(c, om, x, steps=1, warmup=1, threads=1, build_threads=cores)
    M = n_points(om)
    sample = (f'1 full forward+adjoint pair (M={M}, all points) after 1 warm-up pair, 1 thread; '
              f'plan {t_plan:.1f} s (CSR built on {cores} threads)')
    return {'value': 1.0 / times[0], 'unit': 'pairs/s', 'cores': 1, 'kind': 'port',
            'sample': sample}


def run_reference(args, cfg, rank):
    """--impl reference: the CPU oracle (restating the reference numpy NUFFT)
    on the same workload, every step a full forward+adjoint pair."""
    if rank != 0:
        return
    c, om, x = workload(cfg)
    if c.get('ninst', 1) > 1:
        print(json.dumps({'impl': 'reference', 'unavailable': 'the CPU reference arm times '
                          'single-instance configurations only'}), flush=True)
        return
    cores = host_cores()
    t_start = time.perf_counter()
    times, t_plan, O = cpu_pairs(c, om, x, steps=args.steps, warmup=args.warmup, threads=1,
                                 build_threads=cores)
    total = float(np.sum(times))
    value = args.steps / total
    # the same oracle with its row-chunked sparse products and FFTs on every core
    O.threads = cores
    O._row_chunks = None
    tt = []
    for it in range(3):
        t0 = time.perf_counter()
        O.adjoint(O.forward(x))
        if it > 0:
            tt.append(time.perf_counter() - t0)
    M = n_points(om)
    sample = (f'full workload (M={M}): plan {t_plan:.1f} s (CSR built on {cores} threads), '
              f'{args.warmup} warm-up + {args.steps} timed forward+adjoint pairs on 1 thread '
              f'(numpy FFT and scipy CSR products, single-threaded as in the reference)')
    line = {
        'impl': 'reference', 'metric': 'NUFFT fwd+adj pairs/s', 'value': value, 'unit': 'pairs/s',
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': 1e3 * total / args.steps, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'c64 FFT / c128 CSR', 'data': 'synthetic',
        'config': bench_config(cfg, args.gpus),
        'cpu_baseline': {'value': value, 'unit': 'pairs/s', 'cores': 1, 'kind': 'port',
                         'sample': sample},
        'threaded': {'value': len(tt) / float(np.sum(tt)), 'unit': 'pairs/s', 'cores': cores,
                     'sample': f'{len(tt)} pairs after 1 warm-up, the oracle\'s row-chunked CSR '
                               f'products and scipy.fft on {cores} threads'},
        'e2e': {'value': value, 'unit': 'pairs/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
        'wall_s': time.perf_counter() - t_start,
    }
    print(json.dumps(line), flush=True)


def time_pairs(torch, stream, fn, steps, warmup=3):
    """Milliseconds per call of fn over `steps` calls after `warmup`, CUDA
    events on the launching stream."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def batched_leg(torch, dev, peak, steps):
    """Multi-coil workloads: coil-pairs/s of one batched plan against the
    same coils run one after another through a single-coil plan of the same
    points (the plain single-instance path) on the same GPU, and the batched
    gridding / interpolation kernels against the HBM roofline."""
    from ctypes import byref, c_double, c_int, c_void_p
    from pynufft_gb300 import NUFFT
    out = {}
    stream = torch.cuda.current_stream(dev)
    sp = c_void_p(stream.cuda_stream)
    for cfg, det in (('c3', False), ('c5', True)):
        c, om, x = workload(cfg)
        B, M = c['batch'], om.shape[0]
        A = NUFFT(dev)
        A.plan(om, c['Nd'], c['Kd'], c['Jd'], batch=B, deterministic=det)
        lib = A._lib
        xd = torch.from_numpy(x).to(dev)
        yd = torch.empty((M, B), dtype=torch.complex64, device=dev)
        xo = torch.empty_like(xd)

        def pair():
            lib.nufft_forward(A._plan, c_void_p(xd.data_ptr()), c_void_p(yd.data_ptr()), sp)
            lib.nufft_adjoint(A._plan, c_void_p(yd.data_ptr()), c_void_p(xo.data_ptr()), sp)
        ms_b = time_pairs(torch, stream, pair, steps)
        lib.nufft_plan_kernel_timing(A._plan, 1)
        time_pairs(torch, stream, pair, max(3, steps // 2), warmup=0)
        k_ms, y_ms, k_n, y_n = c_double(), c_double(), c_int(), c_int()
        lib.nufft_plan_kernel_times(A._plan, byref(k_ms), byref(k_n), byref(y_ms), byref(y_n))
        lib.nufft_plan_kernel_timing(A._plan, 0)
        t_k2y = k_ms.value / max(k_n.value, 1)
        t_y2k = y_ms.value / max(y_n.value, 1)
        # solve(y, 'cg') on every coil (one system each): 15 iterations for
        # the 2D radial workload, 10 for the kooshball; and the kooshball's
        # trajectory derivative (d forward / d om, every axis and coil)
        cg_iters = 15 if cfg == 'c3' else 10
        xcg = torch.empty_like(xd)
        it = c_int(0)

        def solve():
            lib.nufft_solve_cg(A._plan, c_void_p(yd.data_ptr()), c_void_p(xcg.data_ptr()), cg_iters,
                               1e-5, 0.0, None, sp)
        ms_cg = time_pairs(torch, stream, solve, 3, warmup=1)
        lib.nufft_solve_cg(A._plan, c_void_p(yd.data_ptr()), c_void_p(xcg.data_ptr()), cg_iters,
                           1e-5, 0.0, byref(it), sp)
        cg = {'maxiter': cg_iters, 'iters': it.value, 'ms': ms_cg, 'systems': B}
        del xcg
        dom = None
        if cfg == 'c5':
            dy = torch.empty((len(c['Nd']), M, B), dtype=torch.complex64, device=dev)

            def fdom():
                lib.nufft_forward_dom(A._plan, c_void_p(xd.data_ptr()), c_void_p(dy.data_ptr()), sp)
            dom = {'ms': time_pairs(torch, stream, fdom, 3, warmup=1),
                   'what': 'd forward / d om for every axis and coil (nufft_forward_dom)'}
            del dy
        A.release()
        del yd, xo
        # the plain path: one single-coil plan, the coils' pairs one after another
        P = NUFFT(dev)
        P.plan(om, c['Nd'], c['Kd'], c['Jd'], deterministic=det)
        xs = [xd[..., b].contiguous() for b in range(B)]
        ys = [torch.empty((M,), dtype=torch.complex64, device=dev) for _ in range(B)]
        xos = [torch.empty_like(xs[0]) for _ in range(B)]
        del xd

        def plain():
            for b in range(B):
                P._lib.nufft_forward(P._plan, c_void_p(xs[b].data_ptr()), c_void_p(ys[b].data_ptr()), sp)
                P._lib.nufft_adjoint(P._plan, c_void_p(ys[b].data_ptr()), c_void_p(xos[b].data_ptr()), sp)
        ms_p = time_pairs(torch, stream, plain, steps)
        P.release()
        del xs, ys, xos
        torch.cuda.empty_cache()
        nbytes = alg_bytes(c, M)
        out[cfg] = {
            'workload': c['name'] + (', deterministic gridding' if det else ''),
            'coil_pairs_per_s': B * 1e3 / ms_b, 'ms_per_pair': ms_b,
            'gridding': {'kernel': 'y2k', 'ms': t_y2k, 'gbs': nbytes / (t_y2k / 1e3) / 1e9,
                         'frac': nbytes / (t_y2k / 1e3) / 1e9 / peak},
            'interp': {'kernel': 'k2y', 'ms': t_k2y, 'gbs': nbytes / (t_k2y / 1e3) / 1e9,
                       'frac': nbytes / (t_k2y / 1e3) / 1e9 / peak},
            'alg_bytes': nbytes,
            'plain': {'coil_pairs_per_s': B * 1e3 / ms_p, 'ms_per_coil_pair': ms_p / B,
                      'how': f'{B} single-coil forward+adjoint pairs in turn through one '
                             'single-coil plan of the same points'},
            'speedup_vs_plain': ms_p / ms_b,
            'cg': cg,
            'forward_dom': dom,
            'steps': steps,
        }
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=None,
                    help='timed steps (default 200 on the GPU, 5 full pairs for the CPU reference)')
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--config', default='c2', choices=sorted(CONFIGS))
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline leg')
    ap.add_argument('--no-batched', action='store_true', help='skip the multi-coil leg')
    ap.add_argument('--batched-steps', type=int, default=10,
                    help='timed pairs per measurement of the multi-coil leg')
    ap.add_argument('--batched-only', action='store_true',
                    help='print only the multi-coil leg (a development aid; not a bench line)')
    ap.add_argument('--deterministic', action='store_true',
                    help='plan the workload in the deterministic gridding mode')
    ap.add_argument('--lanes', type=int, default=0,
                    help='concurrent lanes of the end-to-end leg (NUFFT.run_many); '
                         '0: two when a step takes 0.1 ms or more on the device, else one '
                         '(shorter steps are bound by the host issuing them)')
    ap.add_argument('--fft', default='auto', choices=['auto', 'cufft', 'own'],
                    help="the plan's image <-> spectrum transform (auto: the library's choice; "
                         "own: its pruned passes, one-coil power-of-two plans; cufft)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 5 if args.impl == 'reference' else 200
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

    dev = torch.device('cuda', local)
    if args.batched_only:
        print(json.dumps({'batched': batched_leg(torch, dev, peaks()[0], args.batched_steps)}),
              flush=True)
        return
    from pynufft_gb300 import NUFFT, _lib
    c, om, x = workload(args.config)
    A = NUFFT(dev)
    ninst = c.get('ninst', 1)

    def make_plan():
        if ninst > 1:
            A.plan_many(om, c['Nd'], c['Kd'], c['Jd'], batch=c['batch'],
                        deterministic=args.deterministic)
        else:
            A.plan(om, c['Nd'], c['Kd'], c['Jd'], batch=c['batch'],
                   deterministic=args.deterministic, fft=args.fft)
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
    ws_bytes = step_bytes(c, M)
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
    elif fkind.value == _lib.NUFFT_FFT_OWN_COILS:
        # the coil-batched passes (2 or 3 each way), k2y, y2k (deterministic:
        # + the scale's two kernels; the first inverse pass rounds the sums)
        launches_per_step = 2 * len(c['Nd']) + 2 + (2 if args.deterministic else 0)
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

    # end to end through the public API, pinned host buffers, copies included:
    # every step copies its image and its samples in and both results out.
    # `run_many` keeps the host link busy while the GPU transforms (the
    # copies of one step overlap the neighbouring steps' transforms) and
    # runs consecutive steps on `--lanes` operators of the same points, one
    # stream each, so that independent steps' kernels overlap on the GPU;
    # `e2e_sync` calls forward() and adjoint() one at a time, each returning
    # its host result before the next starts.
    xh = torch.from_numpy(x).pin_memory()
    yh = A.forward(xh)                   # the steps' sample input (host)
    for _ in range(2):
        A.adjoint(A.forward(xh))
    torch.cuda.synchronize()
    e2e_steps = max(3, min(args.steps, 50))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        yr = A.forward(xh)
        xr = A.adjoint(yh)
    torch.cuda.synchronize()
    t_sync = (time.perf_counter() - t0) / e2e_steps / ninst
    jobs = [j for _ in range(e2e_steps) for j in (('forward', xh), ('adjoint', yh))]
    outs = [torch.empty_like(xh if name == 'adjoint' else yh).pin_memory() for name, _ in jobs]
    lanes = args.lanes if args.lanes > 0 else (2 if ms_per_step >= 0.1 else 1)
    A.run_many(jobs, out=outs, lanes=lanes)   # warm-up (twins, streams, device buffers)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    A.run_many(jobs, out=outs, lanes=lanes)
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / e2e_steps / ninst
    if dist:
        t = torch.tensor([t_e2e, t_sync], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e, t_sync = float(t[0].item()), float(t[1].item())
    h2d = (xh.numel() + yh.numel()) * 8
    d2h = (yr.numel() + xr.numel()) * 8
    del outs

    batched = None
    if not args.no_batched and args.config == 'c2':
        A.release()
        del xd, yd, xo, xh, yh, xr, yr
        if scratch is not None:
            del scratch
        torch.cuda.empty_cache()
        batched = batched_leg(torch, dev, peak, args.batched_steps)

    cpu = None
    if rank == 0 and not args.no_cpu and ninst == 1:
        cpu = cpu_baseline(args.config, c, om, x)

    if rank == 0:
        line = {
            'metric': 'NUFFT fwd+adj pairs/s', 'value': value, 'unit': 'pairs/s',
            'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': ms_per_step, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'c64', 'data': 'synthetic',
            'config': dict(bench_config(args.config, world),
                           **({'fft': args.fft} if args.fft != 'auto' else {})),
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
                    'd2h_bytes_per_step': d2h, 'api': 'NUFFT.run_many', 'steps': e2e_steps,
                    'lanes': lanes},
            'e2e_sync': {'value': world / t_sync, 'unit': 'pairs/s',
                         'api': 'NUFFT.forward + NUFFT.adjoint, one call at a time'},
            'gpu_launches': launches_per_step * args.steps,
            'plan_ms': plan_ms,
            'cg': cg,
            'batched': batched,
            'clocks': clk,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == '__main__':
    main()

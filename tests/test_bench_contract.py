"""bench.py's reference arm on the CPU: one JSON line with the benchmark's
keys (the oracle port, timed on full forward+adjoint pairs of the 2D radial
workload, with the same config object as the GPU arm), and the line that
says why the many-instance workload has no CPU arm."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), *args],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def test_reference_arm_prints_one_contract_line():
    d = _run('--impl', 'reference', '--config', 'c1', '--steps', '1', '--warmup', '3')
    assert d['impl'] == 'reference'
    assert d['metric'] == 'NUFFT fwd+adj pairs/s' and d['unit'] == 'pairs/s'
    assert d['value'] > 0 and d['ms_per_step'] > 0
    assert d['n_gpus'] == 1 and d['steps'] == 1 and d['warmup'] >= 3
    assert d['higher_is_better'] is True and d['scaling'] == 'weak'
    assert d['vs_baseline'] is None and d['data'] == 'synthetic'
    assert d['config']['workload'].startswith('2D radial')
    sys.path.insert(0, ROOT)
    import bench
    assert d['config'] == bench.bench_config('c1', 1)
    cb = d['cpu_baseline']
    assert cb['kind'] == 'port' and cb['cores'] == 1 and cb['value'] == d['value']
    assert 'M=131072' in cb['sample'] and '3 warm-up + 1 timed' in cb['sample']
    assert d['threaded']['value'] > 0 and d['threaded']['cores'] >= 1
    # every step is a full pair, so the timed pairs fit in the run's own clock
    assert d['ms_per_step'] * d['steps'] / 1e3 <= d['wall_s']
    assert d['e2e'] == {'value': d['value'], 'unit': 'pairs/s', 'h2d_bytes_per_step': 0,
                        'd2h_bytes_per_step': 0}


def test_reference_arm_names_why_many_instances_have_no_cpu_arm():
    d = _run('--impl', 'reference', '--config', 'c3i', '--steps', '1', '--warmup', '3')
    assert d['impl'] == 'reference' and d['unavailable']

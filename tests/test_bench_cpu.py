"""bench.py's CPU legs, which need no GPU: the fresh-process oracle timing used by the
GPU arm's cpu_baseline, and the reference arm's JSON line, on a two-frame stack."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BENCH = os.path.join(ROOT, 'bench.py')


def _run(*args):
    out = subprocess.run([sys.executable, BENCH, *args], capture_output=True, text=True,
                         timeout=600, cwd=ROOT, env={**os.environ, 'WORLD_SIZE': '1',
                                                     'RANK': '0', 'LOCAL_RANK': '0'})
    assert out.returncode == 0, out.stderr[-2000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_cpu_child_times_the_oracle():
    r = _run('--cpu-child', '--frames', '2', '--cpu-frames', '1', '--cpu-threads', '2',
             '--repeats', '1', '--seed', '1000')
    assert r['frames'] == 1 and r['lines'] > 1000 and r['seconds'] > 0


def test_reference_arm_line():
    r = _run('--impl', 'reference', '--frames', '2', '--steps', '2', '--warmup', '1',
             '--cpu-frames', '1')
    assert r['impl'] == 'reference' and r['unit'] == 'Mlines/s' and r['value'] > 0
    assert r['cpu_baseline']['kind'] == 'port' and r['cpu_baseline']['cores'] >= 1
    assert r['e2e']['h2d_bytes_per_step'] == 0 and r['e2e']['value'] == r['value']
    assert r['config']['workload'].startswith('detector_stack_2x2167x2070')

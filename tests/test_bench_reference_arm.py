"""The bench's reference arm runs on the host cores only: its JSON line carries
the fields the bench contract asks of it, and under a multi-rank launch only
rank 0 prints."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CMD = [sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--config', 'C1', '--steps', '1',
       '--warmup', '3', '--ref-sample', '2']


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    r = subprocess.run(CMD, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [json.loads(l) for l in r.stdout.splitlines() if l.startswith('{')]


def test_reference_arm_line():
    lines = _run({'WORLD_SIZE': '1', 'RANK': '0', 'LOCAL_RANK': '0'})
    assert len(lines) == 1
    d = lines[0]
    assert d['impl'] == 'reference'
    assert d['unit'] == 'particle-substeps/s' and d['higher_is_better'] is True
    assert d['value'] > 0 and d['steps'] == 1 and d['warmup'] == 3
    cb = d['cpu_baseline']
    assert cb['kind'] in ('port', 'reference') and cb['cores'] >= 1 and cb['sample'] and cb['value'] == d['value']
    e2e = d['e2e']
    assert e2e['value'] == d['value'] and e2e['h2d_bytes_per_step'] == 0 and e2e['d2h_bytes_per_step'] == 0
    assert d['config']['workload'].startswith('C1')


def test_reference_arm_other_ranks_print_nothing():
    assert _run({'WORLD_SIZE': '2', 'RANK': '1', 'LOCAL_RANK': '1'}) == []

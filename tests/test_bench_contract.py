"""The reference arm of bench.py on the host cores (no GPU needed): the JSON line it prints
for a tiny workload carries the keys and meanings of the bench contract, and ranks other
than 0 exit without work."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TINY = ['--impl', 'reference', '--views', '2', '--image', '256', '--cells', '100', '--steps', '1', '--warmup', '0']


def _run(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py')] + TINY, cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_line():
    p = _run()
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line['impl'] == 'reference'
    for key in ('metric', 'unit', 'ms_per_step', 'dtype', 'data', 'config', 'scaling', 'wall_s'):
        assert key in line, key
    assert line['value'] > 0 and line['ms_per_step'] > 0
    assert line['n_gpus'] == 1 and line['steps'] == 1 and line['warmup'] == 0
    assert line['higher_is_better'] is True and line['vs_baseline'] is None
    assert line['config']['workload'].startswith('aoi2') and line['config']['views'] == 2
    # the step is a measured sample of the workload and says which fraction
    assert 0 < line['step_is_sample_fraction'] <= 1
    cb = line['cpu_baseline']
    assert cb['kind'] == 'port' and cb['cores'] >= 1 and cb['value'] == line['value'] and cb['sample']
    e2e = line['e2e']
    assert e2e['value'] == line['value'] and e2e['unit'] == line['unit']
    assert e2e['h2d_bytes_per_step'] == 0 and e2e['d2h_bytes_per_step'] == 0


def test_reference_arm_other_ranks_exit_quietly():
    p = _run({'RANK': '1', 'WORLD_SIZE': '2'})
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ''

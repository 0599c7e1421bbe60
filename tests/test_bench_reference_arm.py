"""The reference arm of the bench (``bench.py --impl reference``), on CPU:
the JSON line keeps the contract of the GPU arm's line (same metric, unit,
direction and workload naming, a cpu_baseline block, an e2e block with no
host-device traffic), it maps none of the product's native code, and under
a rank other than 0 it prints nothing.  The small workload (8 waters) and
a 16-point sample keep it to about a second."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ['--impl', 'reference', '--small', '--steps', '1', '--warmup', '3',
        '--ref-points', '16']

# runs the bench's main() in this interpreter, then reports whether the
# product library is mapped into the process
_PROBE = r'''
import runpy, sys
sys.argv = ['bench.py'] + sys.argv[1:]
runpy.run_path('bench.py', run_name='__main__')
with open('/proc/self/maps') as fh:
    mapped = [l.split()[-1] for l in fh if 'libwb97mv_gb300' in l]
print('PRODUCT_LIB_MAPPED=%d' % bool(mapped))
'''


def _run(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    res = subprocess.run([sys.executable, '-c', _PROBE] + ARGS, cwd=ROOT,
                         env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-3000:]
    return res.stdout.strip().splitlines()


def test_reference_arm_line_keeps_the_bench_contract():
    out = _run()
    assert out[-1] == 'PRODUCT_LIB_MAPPED=0'
    lines = [l for l in out if l.startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench
    assert d['impl'] == 'reference'
    assert d['metric'] == bench.METRIC and d['unit'] == bench.UNIT
    assert d['higher_is_better'] is True and d['scaling'] == 'weak'
    assert d['steps'] == 1 and d['warmup'] == 3 and d['n_gpus'] == 1
    assert d['value'] > 0 and d['ms_per_step'] > 0
    assert d['vs_baseline'] is None
    assert d['config']['workload'] == 'cosx_g_water8_svp'
    assert d['config']['nao'] == 192
    cb = d['cpu_baseline']
    assert cb['kind'] in ('port', 'reference')
    assert cb['cores'] >= 1 and cb['value'] == d['value'] and cb['unit'] == d['unit']
    assert cb['sample'].startswith('16 of ')
    e2e = d['e2e']
    assert e2e['value'] == d['value'] and e2e['unit'] == d['unit']
    assert e2e['h2d_bytes_per_step'] == 0 and e2e['d2h_bytes_per_step'] == 0


def test_reference_arm_prints_nothing_off_rank_zero():
    out = _run({'RANK': '1', 'WORLD_SIZE': '2'})
    assert out == ['PRODUCT_LIB_MAPPED=0']

"""The class-kernel generator (csrc/gen_cosx.py) is deterministic: its
output is regenerated by every build and is not tracked, so two runs must
give the same text, and the files build() wrote must equal a fresh run."""
import importlib
import os
import sys

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    'pyscf_wb97mv_fast_gb300', 'csrc')


def _gen():
    sys.path.insert(0, CSRC)
    try:
        return importlib.import_module('gen_cosx')
    finally:
        sys.path.pop(0)


def test_generator_output_is_deterministic():
    g = _gen()
    a, b = g.source(), g.source()
    assert a == b and len(a) > 100_000
    assert g.layout_source() == g.layout_source()


def test_written_files_match_a_fresh_run(tmp_path):
    g = _gen()
    path = g.write(str(tmp_path / 'cosx_classes.cuh'))
    with open(path) as fh:
        assert fh.read() == g.source()
    with open(tmp_path / 'cosx_layout.h') as fh:
        assert fh.read() == g.layout_source()

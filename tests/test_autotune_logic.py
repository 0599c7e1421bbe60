"""The autotuner's variant space on the CPU (the timing itself needs the
GPU: tests/test_gpu_autotune.py)."""
from pyscf_wb97mv_fast_gb300.autotune import candidates, variant_name


def test_variant_names_follow_what_runs():
    assert variant_name((1, 0), 2) == variant_name((1, 1), 2) == 'two-omega (staged)'
    assert variant_name((1, 1), 1) == 'single-omega staged'
    assert variant_name((1, 0), 1) == 'single-omega register prefetch'
    assert variant_name((0, 0), 2) == 'single-omega register prefetch'


def test_candidates_cover_the_kernels_that_can_run():
    two = candidates((1, 0), 2)
    assert {variant_name(v, 2) for v in two} == {
        'two-omega (staged)', 'single-omega staged', 'single-omega register prefetch'}
    assert (1, 0) in two                  # the current staging choice is kept
    one = candidates((1, 1), 1)
    assert len(one) == 2 and all(v[0] == 1 for v in one)
    assert {variant_name(v, 1) for v in one} == {
        'single-omega staged', 'single-omega register prefetch'}

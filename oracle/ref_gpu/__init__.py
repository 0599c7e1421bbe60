"""The reference's own CUDA kernels on this GPU: the GPU-side baseline.

TEST INFRASTRUCTURE ONLY (a measurement arm of bench.py, never the product).

The reference compiles its kernels at run time from CUDA C strings
(gpu/sgx_k.py:72-400 sgx_k_tile / sgx_k_cls<LA,LB>, :417-456
sgx_screen_mask; gpu/vv10.py:47-98 vv10_kernel_sum) through CuPy, which is
absent here.  ``extract.py`` (run where a reference checkout exists) writes
those strings, unmodified, to oracle/_ref/ref_kernels.cuh together with the
reference's own ShellPairsDevice arrays of the bench molecule
(gpu/shellpairs.py:184-446, packed by the reference's code); ``harness.cu``
(this directory) adds extern "C" launchers with the reference's launch
shapes (gpu/sgx_k.py:754-781: one warp per 32-point sub-block, warps per
block = min(4, max threads / 32)), and ``runner.py`` drives them from
PyTorch: the reference's screen, the per-class CSR task lists
(gpu/sgx_k.py:905-924), the class launches, and the VV10 sum.
oracle/_ref/ is build output (git-ignored); without it the arm reports
itself unavailable.
"""

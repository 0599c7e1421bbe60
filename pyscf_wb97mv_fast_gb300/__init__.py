"""GB300-native (sm_103a) COSX exchange hot path of the wB97M-V / COSX(pjs)
SCF, behind the removable PySCF-hook API of pyscf-wb97mv-fast.

    core.hooks      HookSet, reset_diis, track_residual
    core.sgx_patch  the RSH-branch fix of PySCF's SGX.get_jk
    gpu.install     install_gpu(mf, k=True) -> HookSet
    gpu.sgx_k       GpuKBuilder, get_k_only_gpu
    gpu.vv10        VV10 kernel sum and the nr_nlc_vxc flow
    gpu.xc          the semilocal nr_rks flow
    staging         StagedSCF, run_staged
    cosx            CosxEngine: the native handle driven from PyTorch
    basis, systems, grids   synthetic inputs (no PySCF needed)

Importing the package imports neither PySCF nor torch; the native library
(libwb97mv_gb300.so, built by pyscf_wb97mv_fast_gb300.build) is loaded on
first use.
"""
__version__ = '0.1.0'

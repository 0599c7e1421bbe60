"""Builds libwb97mv_gb300.so in-tree (nvcc, sm_103a) from csrc/.

    python -m pyscf_wb97mv_fast_gb300.build

Translation units compile in parallel; the class kernels are regenerated
first (csrc/gen_cosx.py).  Objects go to _build/ at the repository root, the
library to pyscf_wb97mv_fast_gb300/_lib/.  Nothing is rebuilt when the
sources are older than the library and the compile flags (WB_NVCC_EXTRA
included) are those it was built with, recorded beside it in
libwb97mv_gb300.so.flags.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
INCLUDE = os.path.join(ROOT, 'include')
BUILD = os.path.join(ROOT, '_build', 'lib')
LIBDIR = os.path.join(PKG, '_lib')
LIBNAME = 'libwb97mv_gb300.so'
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']

SOURCES = ['cosx_kernels_spd.cu', 'cosx_kernels_f.cu', 'cosx_batch_spd.cu',
           'cosx_batch_f.cu', 'cosx_fp64.cu', 'cosx_fp64_f.cu', 'cosx_grad64.cu',
           'aux_kernels.cu', 'scf_kernels.cu',
           'vv10.cu', 'ozaki.cu', 'ozaki_tc.cu', 'capi.cu', 'host_pairs.cpp']


def cuda_home():
    for cand in (os.environ.get('CUDA_HOME'), '/usr/local/cuda'):
        if cand and os.path.exists(os.path.join(cand, 'bin', 'nvcc')):
            return cand
    nvcc = shutil.which('nvcc')
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError('nvcc not found (set CUDA_HOME)')


def library_path():
    return os.path.join(LIBDIR, LIBNAME)


def _deps():
    out = []
    for dirpath, _, files in os.walk(CSRC):
        for f in files:
            if f.endswith(('.cu', '.cuh', '.cpp', '.hpp', '.h', '.py')):
                out.append(os.path.join(dirpath, f))
    out.append(os.path.join(INCLUDE, 'wb97mv_gb300.h'))
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _flags():
    """The flags that change the code: architecture and WB_NVCC_EXTRA
    (e.g. WB_NVCC_EXTRA=-DWB_COSX_SPLIT=0)."""
    return ARCH + os.environ.get('WB_NVCC_EXTRA', '').split()


def _flags_changed(lib):
    try:
        with open(lib + '.flags') as fh:
            return fh.read() != ' '.join(_flags())
    except OSError:
        return True


def build(verbose=False, force=False, jobs=None):
    """Compile and link; returns the library path."""
    sys.path.insert(0, CSRC)
    try:
        import gen_cosx
    finally:
        sys.path.pop(0)
    gen_cosx.write()
    lib = library_path()
    deps = _deps()
    if not force and not _stale(lib, deps) and not _flags_changed(lib):
        return lib
    home = cuda_home()
    nvcc = os.path.join(home, 'bin', 'nvcc')
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    common = ['-std=c++17', '-O3', '-lineinfo', '-I', INCLUDE, '-I', CSRC,
              '-Xcompiler', '-fPIC,-fopenmp,-O2', '-Xptxas', '-v' if verbose else '-O3']
    # extra nvcc flags, e.g. WB_NVCC_EXTRA=-DWB_COSX_MIN_BLOCKS=9766431111LL
    common += os.environ.get('WB_NVCC_EXTRA', '').split()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + '.o')
        cmd = [nvcc] + ARCH + common + ['-c', os.path.join(CSRC, src), '-o', obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError('nvcc failed on %s:\n%s\n%s' % (src, res.stdout,
                                                            res.stderr))
        return obj, res.stderr

    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = lib + '.tmp'
    cmd = [nvcc] + ARCH + ['-shared', '-o', tmp] + objs + [
        '-L', os.path.join(home, 'lib64'), '-lcublas', '-Xcompiler', '-fopenmp',
        '-Xlinker', '-rpath,' + os.path.join(home, 'lib64')]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (res.stdout, res.stderr))
    os.replace(tmp, lib)
    with open(lib + '.flags', 'w') as fh:
        fh.write(' '.join(_flags()))
    return lib


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv, force='-f' in sys.argv))

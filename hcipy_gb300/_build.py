"""Build recipe of the CUDA library: nvcc for sm_103a, one object per .cu, one shared library.

Compiles every ``csrc/*.cu`` in parallel into ``_build/`` and links
``lib/libhcipy_gb300.so``.  Objects are rebuilt when their source or any
header under ``csrc/`` or ``include/`` is newer.
"""
import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(ROOT, '_build')
LIBDIR = os.path.join(PKG, 'lib')
LIBNAME = 'libhcipy_gb300.so'
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '--expt-relaxed-constexpr', '-Xcompiler', '-fPIC',
              '-Xcompiler', '-fvisibility=hidden', '-I' + os.path.join(ROOT, 'include')]


def nvcc_path():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build hcipy_gb300')


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(ROOT, 'include', '*.h'))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(nvcc, src, obj, extra):
    cmd = [nvcc] + ARCH + NVCC_FLAGS + extra + ['-c', src, '-o', obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (os.path.basename(src), res.stdout, res.stderr))
    return res.stderr


def build(verbose=False, extra_flags=()):
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    newest_h = _newest_header()
    jobs = []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + '.o')
        if (not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), newest_h)
                or extra_flags):
            jobs.append((src, obj))
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        futs = [ex.submit(_compile, nvcc, s, o, list(extra_flags)) for s, o in jobs]
        for f in futs:
            msg = f.result()
            if verbose and msg:
                sys.stderr.write(msg)
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + '.o') for s in sources]
    lib = os.path.join(LIBDIR, LIBNAME)
    if jobs or not os.path.exists(lib):
        tmp = lib + '.tmp'
        cmd = [nvcc] + ARCH + ['-shared', '-cudart', 'shared', '-o', tmp] + objs
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError('link failed:\n%s\n%s' % (res.stdout, res.stderr))
        os.replace(tmp, lib)
    return lib


if __name__ == '__main__':
    print(build(verbose=True))

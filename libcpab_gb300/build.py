"""Build the sm_103a shared library libcpab_gb300/libcpab_gb300.so.

Each translation unit in csrc/ is compiled by nvcc in parallel
(-gencode arch=compute_103a,code=sm_103a) and linked into one shared library
whose exported symbols are the C ABI of include/cpab_gb300.h.  Objects go to
libcpab_gb300/_build/; both stay out of version control.

    python -m libcpab_gb300.build [-f] [-v]
"""
import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libcpab_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc_path():
    cand = [os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc']
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError('nvcc not found')


def _compile(nvcc, src, obj, verbose):
    cmd = [nvcc, *ARCH, '-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
           '-Xcompiler', '-fvisibility=hidden', '-c', src, '-o', obj]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s' % (src, r.stderr))
    return r.stderr


def build(force=False, verbose=False):
    """Compile if any source is newer than the library; returns the .so path."""
    srcs = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    deps = srcs + glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(CSRC, '*.h')) + \
        [os.path.join(os.path.dirname(HERE), 'include', 'cpab_gb300.h'), __file__]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d)):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = nvcc_path()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + '.o') for s in srcs]
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        logs = list(ex.map(lambda so: _compile(nvcc, so[0], so[1], verbose), zip(srcs, objs)))
    if verbose:
        for s, lg in zip(srcs, logs):
            print('==', os.path.basename(s))
            print(lg)
    tmp = LIB + '.tmp%d' % os.getpid()
    cmd = [nvcc, *ARCH, '-shared', '-o', tmp, *objs, '-lcudart']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n' + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='-f' in sys.argv, verbose='-v' in sys.argv))

"""Build recipe for the CPU oracle (TEST INFRASTRUCTURE ONLY).

* oracle/libcpab_oracle.so -- the C restatement in oracle/cpab_oracle.c,
  built wherever gcc exists (here and on the GPU host).
* oracle/_ref/libcpab_ref.so -- the reference's own CPU ops
  (libcpab/core/cpab_ops.cpp) compiled with oracle/ref_shim.cpp from the
  read-only reference checkout or, where the checkout is absent (a machine
  the working tree was copied to), from the unmodified copy of the reference
  package in baseline/_ref/libcpab (baseline/plain_gpu.py makes it).  Built
  only when one of the two exists; the output stays out of version control.

Both are built without FMA contraction so x86-64 and aarch64 round alike.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_ROOT = os.environ.get('CPAB_REFERENCE_ROOT', '/root/reference')
REF_CORE = os.path.join(REFERENCE_ROOT, 'libcpab', 'core')
REF_CORE_COPY = os.path.join(os.path.dirname(HERE), 'baseline', '_ref', 'libcpab', 'core')
ORACLE_SO = os.path.join(HERE, 'libcpab_oracle.so')
REF_SO = os.path.join(HERE, '_ref', 'libcpab_ref.so')

_FLAGS = ['-O2', '-fPIC', '-shared', '-ffp-contract=off', '-fno-fast-math']


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, 'cpab_oracle.c')
    if force or _stale(ORACLE_SO, [src]):
        tmp = ORACLE_SO + '.tmp%d' % os.getpid()
        subprocess.check_call(['gcc', '-std=c11', *_FLAGS, '-fopenmp', src, '-o', tmp, '-lm'])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(force=False):
    """Compile the reference's CPU ops; returns the .so path or None."""
    core = REF_CORE if os.path.exists(os.path.join(REF_CORE, 'cpab_ops.cpp')) else REF_CORE_COPY
    cpp = os.path.join(core, 'cpab_ops.cpp')
    shim = os.path.join(HERE, 'ref_shim.cpp')
    if not os.path.exists(cpp):
        return REF_SO if os.path.exists(REF_SO) else None
    if force or _stale(REF_SO, [cpp, shim]):
        os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
        tmp = REF_SO + '.tmp%d' % os.getpid()
        subprocess.check_call(['g++', *_FLAGS, '-I', core, shim, cpp, '-o', tmp])
        os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == '__main__':
    print(build_oracle(force='-f' in sys.argv))
    print(build_ref(force='-f' in sys.argv))

"""The reference's own pytorch GPU path: the "plain" comparator of the headline
metric (fused transform_data forward + dtheta backward vs the one-kernel-per-op
GPU path).

The reference is run unmodified through its public API:
``libcpab.Cpab(..., backend='pytorch', device='gpu').transform_data`` and
autograd, i.e. its basis upload and Pade expm (libcpab/pytorch/expm.py), its
CUDA integrator and analytic-gradient kernels (libcpab/core/cpab_ops.cu:268-697,
launched from libcpab/pytorch/transformer_cuda.cu) with the contraction of the
[d, n_theta, ndim, nP] sensitivity tensor (libcpab/pytorch/transformer.py:186-202),
and its gather-based interpolation with autograd (libcpab/pytorch/interpolation.py).

install()  copies the reference package (libcpab/: its Python sources and its
           C++/CUDA op sources, nothing compiled) from the reference checkout
           into baseline/_ref/libcpab, which version control ignores and which
           travels with the working tree.  ``pip install --target`` of the
           checkout is not enough: its setup.py lists only the top-level
           package, so libcpab/core, libcpab/pytorch and the op sources are
           left out.
load()     imports it with process-local shims (a matplotlib stub: the
           reference imports it for plotting only; scipy.transpose /
           scipy.compress aliased to numpy's; torch.solve mapped to
           torch.linalg.solve; a pass-through tqdm where that progress-bar
           package is not installed) and lets the reference JIT-build its own
           extensions (torch.utils.cpp_extension.load at import,
           libcpab/pytorch/transformer.py:27-69) for sm_103a into
           baseline/_ref/torch_extensions.  It raises if the CUDA op did not
           build: the reference would otherwise fall back to its slow path
           without a word.

    python baseline/plain_gpu.py     # install (where the checkout exists) and build
"""
import os
import shutil
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, '_ref')
REF_PKG = os.path.join(REF_DIR, 'libcpab')
EXT_DIR = os.path.join(REF_DIR, 'torch_extensions')
REFERENCE_ROOT = os.environ.get('CPAB_REFERENCE_ROOT', '/root/reference')


def install(force=False):
    """Copy the reference package into baseline/_ref; returns its path or None
    when neither the checkout nor an earlier copy exists."""
    src = os.path.join(REFERENCE_ROOT, 'libcpab')
    if not os.path.isdir(src):
        return REF_PKG if os.path.isdir(REF_PKG) else None
    if os.path.isdir(REF_PKG) and not force:
        return REF_PKG
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = REF_PKG + '.tmp%d' % os.getpid()
    # the TensorFlow backend ships a prebuilt object file: not copied
    shutil.copytree(src, tmp, ignore=shutil.ignore_patterns('*.o', '__pycache__'))
    if os.path.isdir(REF_PKG):
        shutil.rmtree(REF_PKG)
    os.replace(tmp, REF_PKG)
    return REF_PKG


def _shims():
    import numpy as np
    import scipy
    import torch
    if 'matplotlib' not in sys.modules:
        mpl = types.ModuleType('matplotlib')
        plt = types.ModuleType('matplotlib.pyplot')
        plt.figure = lambda *a, **k: None
        mpl.pyplot = plt
        sys.modules['matplotlib'] = mpl
        sys.modules['matplotlib.pyplot'] = plt
    if not hasattr(scipy, 'transpose'):
        scipy.transpose = np.transpose
    if not hasattr(scipy, 'compress'):
        scipy.compress = np.compress
    # torch keeps a torch.solve that only raises (removed in 1.9): always replace it
    torch.solve = lambda P, Q: (torch.linalg.solve(Q, P), None)
    try:
        import tqdm  # noqa: F401  (the reference's alignment loop's progress bar)
    except ImportError:
        tq = types.ModuleType('tqdm')
        tq.tqdm = lambda it=None, *a, **k: it
        sys.modules['tqdm'] = tq


def load():
    """Import the reference (building its extensions on first use); returns
    the libcpab module."""
    if not os.path.isdir(REF_PKG):
        raise RuntimeError('the reference package is not installed in %s (run '
                           'baseline/plain_gpu.py where the reference checkout exists)' % REF_DIR)
    os.makedirs(EXT_DIR, exist_ok=True)
    os.environ['TORCH_EXTENSIONS_DIR'] = EXT_DIR
    os.environ.setdefault('TORCH_CUDA_ARCH_LIST', '10.3a')
    _shims()
    if REF_DIR not in sys.path:
        sys.path.insert(0, REF_DIR)
    import libcpab
    from libcpab.pytorch import transformer
    if not getattr(transformer, '_gpu_succes', False):
        raise RuntimeError('the reference CUDA op (cpab_gpu) did not build')
    return libcpab


if __name__ == '__main__':
    print(install(force='-f' in sys.argv))
    load()
    print('reference CUDA op built in', EXT_DIR)

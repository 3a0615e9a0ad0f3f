"""ctypes binding of the C ABI in include/cpab_gb300.h.

The shared library libcpab_gb300/libcpab_gb300.so is built by
libcpab_gb300/build.py.  There is no fallback: if the library is missing or
fails to load, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libcpab_gb300.so')

GRAD_REFERENCE = 0
GRAD_EXACT = 1
GRAD_REFERENCE_MAP = 2

_c_int_p = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_i = ctypes.c_int
_ll = ctypes.c_longlong
_sz = ctypes.c_size_t
_fp = ctypes.POINTER(ctypes.c_float)

_SIGS = {
    'cpab_last_error': ([], ctypes.c_char_p),
    'cpab_version': ([], _i),
    'cpab_num_cells': ([_i, _c_int_p], _i),
    'cpab_cell_tables': ([_i, _c_int_p, _i, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp], _i),
    'cpab_forward': ([_i, _c_int_p, _i, _vp, _i, _ll, _vp, _i, _vp, _vp], _i),
    'cpab_integrate': ([_i, _c_int_p, _i, _vp, _i, _ll, _vp, _i, _vp, _vp, _vp], _i),
    'cpab_integrate_trace': ([_i, _c_int_p, _i, _vp, _i, _ll, _vp, _i, _vp, _vp, _vp], _i),
    'cpab_integrate_exact': ([_i, _c_int_p, _vp, _i, _ll, _vp, _i, _vp, _vp, _vp, _vp], _i),
    'cpab_backward_exact_workspace': ([_i, _c_int_p, _ll, _i], _sz),
    'cpab_backward_exact': ([_i, _c_int_p, _vp, _ll, _vp, _i, _vp, _i, _vp, _vp, _vp, _vp, _sz,
                             _vp, _vp], _i),
    'cpab_backward_workspace': ([_i, _c_int_p, _i, _ll, _i], _sz),
    'cpab_backward': ([_i, _c_int_p, _i, _i, _vp, _i, _ll, _vp, _vp, _i, _vp, _i, _vp, _vp, _vp,
                       _vp, _sz, _vp, _vp], _i),
    'cpab_backward_noalloc': ([_i, _c_int_p, _i, _i, _vp, _i, _ll, _vp, _vp, _i, _vp, _i, _vp,
                               _vp, _vp, _vp, _vp], _i),
    'cpab_interpolate': ([_i, _vp, _i, _i, _c_int_p, _vp, _c_int_p, _vp, _vp], _i),
    'cpab_interpolate_backward': ([_i, _vp, _i, _i, _c_int_p, _vp, _c_int_p, _vp, _vp, _vp, _vp],
                                  _i),
    'cpab_transform_data': ([_i, _c_int_p, _i, _vp, _c_int_p, _vp, _i, _vp, _i, _c_int_p, _vp,
                             _vp, _vp, _vp], _i),
    'cpab_transform_grid_image': ([_i, _c_int_p, _i, _vp, _c_int_p, _vp, _i, _vp, _vp, _vp], _i),
    'cpab_sample_grid': ([_i, _vp, _i, _i, _c_int_p, _vp, _c_int_p, _vp, _vp], _i),
    'cpab_transform_data_backward_workspace': ([_i, _c_int_p, _i, _i, _c_int_p, _i], _sz),
    'cpab_transform_data_backward': ([_i, _c_int_p, _i, _i, _vp, _c_int_p, _vp, _vp, _vp, _i, _vp,
                                      _i, _c_int_p, _vp, _i, _vp, _vp, _vp, _vp, _sz, _vp, _vp],
                                     _i),
    'cpab_findcellidx': ([_i, _c_int_p, _vp, _ll, _vp, _vp, _vp], _i),
    'cpab_device_status': ([ctypes.POINTER(ctypes.c_uint), _i], _i),
    'cpab_sequential_transform_data': ([_i, _i, _c_int_p, _c_int_p, _vp, _c_int_p, _vp, _i, _vp,
                                        _i, _c_int_p, _vp, _vp, _vp, _vp], _i),
    'cpab_sequential_transform_data_backward': ([_i, _i, _c_int_p, _c_int_p, _i, _vp, _c_int_p,
                                                 _vp, _vp, _vp, _i, _vp, _i, _c_int_p, _vp, _i,
                                                 _vp, _vp, _vp, _vp, _sz, _vp, _vp], _i),
    'cpab_ragged1d_workspace': ([_i, _i, _i], _sz),
    'cpab_ragged1d_forward': ([_i, _i, _vp, _i, _vp, _ll, _vp, _vp, _vp, _sz, _vp, _vp], _i),
    'cpab_ragged1d_backward': ([_i, _i, _i, _vp, _vp, _i, _vp, _ll, _vp, _i, _vp, _vp, _vp, _vp,
                                _vp, _sz, _vp, _vp], _i),
    'cpab_ragged1d_mse': ([_i, _i, _i, _vp, _vp, _i, _vp, _ll, _vp, _i, _vp, _vp, ctypes.c_float,
                           _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp], _i),
    'cpab_ragged1d_tune': ([_i, _i, _i, _i, _vp, _vp, _i, _vp, _ll, _vp, _i, _vp, _vp,
                            ctypes.c_float, _vp, _vp, _vp, _vp, _vp, _sz, _c_int_p, _c_int_p,
                            ctypes.POINTER(ctypes.c_float), _vp], _i),
    'cpab_ragged_points_workspace': ([_i, _c_int_p, _i], _sz),
    'cpab_ragged_points_forward': ([_i, _c_int_p, _i, _vp, _i, _vp, _ll, _vp, _vp, _vp, _sz, _vp,
                                    _vp], _i),
    'cpab_ragged_points_backward': ([_i, _c_int_p, _i, _i, _vp, _vp, _i, _vp, _ll, _vp, _i, _vp,
                                     _vp, _vp, _vp, _vp, _sz, _vp, _vp], _i),
    'cpab_ragged_images_plan': ([_i, _i, _c_int_p, _c_int_p, _vp, _vp], _i),
    'cpab_interpolate_ragged': ([_i, _i, _i, _vp, _ll, _ll, _ll, _vp, _vp, _vp, _vp], _i),
    'cpab_interpolate_ragged_backward': ([_i, _i, _i, _vp, _ll, _ll, _ll, _vp, _vp, _vp, _vp, _vp,
                                          _vp], _i),
    'cpab_integrate_tune': ([_i, _c_int_p, _i, _vp, _i, _ll, _vp, _i, _vp, _c_int_p, _c_int_p,
                             _fp, _vp], _i),
    'cpab_backward_tune': ([_i, _c_int_p, _i, _i, _vp, _i, _ll, _vp, _vp, _i, _vp, _i, _vp, _vp,
                            _vp, _c_int_p, _c_int_p, _fp, _vp], _i),
    'cpab_transform_data_tune': ([_i, _c_int_p, _i, _vp, _c_int_p, _vp, _i, _vp, _i, _c_int_p,
                                  _vp, _vp, _c_int_p, _c_int_p, _fp, _vp], _i),
    'cpab_transform_data_backward_tune': ([_i, _c_int_p, _i, _i, _vp, _c_int_p, _vp, _vp, _vp,
                                           _i, _vp, _i, _c_int_p, _vp, _i, _vp, _vp, _vp,
                                           _c_int_p, _c_int_p, _fp, _vp], _i),
    'cpab_ragged_points_tune': ([_i, _i, _c_int_p, _i, _i, _vp, _vp, _i, _vp, _ll, _vp, _i, _vp,
                                 _vp, _vp, _vp, _vp, _c_int_p, _c_int_p, _fp, _vp], _i),
    'cpab_tune_reset': ([], None),
}

EXPORTED = tuple(_SIGS)

_lib = None
_lock = threading.Lock()


class CpabError(RuntimeError):
    """Raised when a C-ABI call returns an error status."""


def load(path: str | None = None):
    """Load (once) and return the shared library.  Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise ImportError(
                'libcpab_gb300 native library not found at %s; build it with '
                '"python -m libcpab_gb300.build" (there is no CPU fallback)' % p)
        lib = ctypes.CDLL(p)
        for name, (args, res) in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        if path is None:
            _lib = lib
        return lib


def _check(rc: int):
    if rc != 0:
        msg = load().cpab_last_error().decode(errors='replace')
        raise CpabError('libcpab_gb300 error %d: %s' % (rc, msg))


_ints_cache = {}


def _ints(v):
    # the C side only reads these arrays, so one per distinct tuple is reused
    # (the per-call host overhead sits on the critical path of eager steps)
    key = tuple(int(x) for x in v)
    a = _ints_cache.get(key)
    if a is None:
        if len(_ints_cache) > 256:
            _ints_cache.clear()
        a = _ints_cache[key] = (ctypes.c_int * len(key))(*key)
    return a


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


# The current stream's cudaStream_t: torch's raw-handle query where present
# (torch.cuda.current_stream(device) normalises the device and builds a Stream
# object on every call, a measurable share of an eager step's host time).
_raw_stream = getattr(torch._C, '_cuda_getCurrentRawStream', None)


def _stream(device) -> ctypes.c_void_p:
    if _raw_stream is not None and isinstance(device, torch.device) and device.type == 'cuda':
        idx = device.index if device.index is not None else torch.cuda.current_device()
        return ctypes.c_void_p(_raw_stream(idx))
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _require(t, name, dtype=torch.float32):
    if not isinstance(t, torch.Tensor):
        raise TypeError('%s must be a torch.Tensor' % name)
    if not t.is_cuda:
        raise ValueError('%s must be a CUDA tensor (no CPU fallback)' % name)
    if t.dtype != dtype:
        raise TypeError('%s must be %s (got %s)' % (name, dtype, t.dtype))
    if not t.is_contiguous():
        raise ValueError('%s must be contiguous' % name)


# ----------------------------------------------------------------------------- #
_cells_cache = {}


def num_cells(nc) -> int:
    key = tuple(int(x) for x in nc)
    n = _cells_cache.get(key)
    if n is None:
        n = load().cpab_num_cells(len(key), _ints(key))
        if n < 0:
            _check(1)
        _cells_cache[key] = n
    return n


def cell_tables(nc, nsteps, theta, basis, want_A=True, want_T=False, want_E=True):
    """theta [n_theta, d], basis [D, d] (device fp32) -> (A, T, E) tables."""
    _require(theta, 'theta')
    _require(basis, 'basis')
    ndim = len(nc)
    n_theta, d = theta.shape
    nC = num_cells(nc)
    shape = (n_theta, nC, ndim, ndim + 1)
    mk = lambda w: torch.empty(shape, device=theta.device, dtype=torch.float32) if w else None
    A, T, E = mk(want_A), mk(want_T), mk(want_E)
    _check(load().cpab_cell_tables(ndim, _ints(nc), int(nsteps), _ptr(theta), n_theta, d,
                                   _ptr(basis), _ptr(A), _ptr(T), _ptr(E), _stream(theta.device)))
    return A, T, E


def forward_trels(nc, nsteps, points, trels):
    """Reference-layout step maps T: drop-in for cpab_gpu.forward."""
    _require(points, 'points')
    _require(trels, 'trels')
    ndim = len(nc)
    n_theta = trels.shape[0]
    broadcast = int(points.dim() == 3 and points.shape[0] == n_theta)
    nP = points.shape[-1]
    out = torch.empty((n_theta, ndim, nP), device=points.device, dtype=torch.float32)
    _check(load().cpab_forward(ndim, _ints(nc), int(nsteps), _ptr(points), broadcast, nP,
                               _ptr(trels), n_theta, _ptr(out), _stream(points.device)))
    return out


def integrate(nc, nsteps, points, E, ties=None):
    _require(points, 'points')
    _require(E, 'E')
    ndim = len(nc)
    n_theta = E.shape[0]
    broadcast = int(points.dim() == 3 and points.shape[0] == n_theta)
    nP = points.shape[-1]
    out = torch.empty((n_theta, ndim, nP), device=points.device, dtype=torch.float32)
    _check(load().cpab_integrate(ndim, _ints(nc), int(nsteps), _ptr(points), broadcast, nP,
                                 _ptr(E), n_theta, _ptr(out), _ptr(ties), _stream(points.device)))
    return out


def integrate_exact(nc, points, A, ties=None, steps=None):
    """Exact flow of the field A for time 1 (opt-in scheme, forward only)."""
    _require(points, 'points')
    _require(A, 'A')
    ndim = len(nc)
    n_theta = A.shape[0]
    broadcast = int(points.dim() == 3 and points.shape[0] == n_theta)
    nP = points.shape[-1]
    out = torch.empty((n_theta, ndim, nP), device=points.device, dtype=torch.float32)
    _check(load().cpab_integrate_exact(ndim, _ints(nc), _ptr(points), broadcast, nP, _ptr(A),
                                       n_theta, _ptr(out), _ptr(ties), _ptr(steps),
                                       _stream(points.device)))
    return out


def backward_exact(nc, out, A, basis, grad_out, want_dpoints=False, ties=None, workspace=None):
    """Gradient of integrate_exact: dtheta [n_theta, d] and dL/dpoints per theta
    [n_theta, ndim, nP] (or None) from out = integrate_exact(...) [n_theta, ndim,
    nP] and dL/d(out)."""
    _require(out, 'out')
    _require(A, 'A')
    _require(basis, 'basis')
    _require(grad_out, 'grad_out')
    ndim = len(nc)
    n_theta, nP = out.shape[0], out.shape[-1]
    d = basis.shape[1]
    dev = out.device
    dtheta = torch.empty((n_theta, d), device=dev, dtype=torch.float32)
    dpoints = torch.empty_like(out) if want_dpoints else None
    lib = load()
    need = lib.cpab_backward_exact_workspace(ndim, _ints(nc), nP, n_theta)
    if need == 0 and nP > 0 and n_theta > 0:
        _check(3)
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(max(need, 1), device=dev, dtype=torch.uint8)
    _check(lib.cpab_backward_exact(ndim, _ints(nc), _ptr(out), nP, _ptr(A), n_theta,
                                   _ptr(basis), d, _ptr(grad_out), _ptr(dtheta), _ptr(dpoints),
                                   _ptr(workspace), workspace.numel(), _ptr(ties), _stream(dev)))
    return dtheta, dpoints


def integrate_trace(nc, nsteps, points, E):
    """integrate() plus the cell of every step, [n_theta, nP, nsteps] int32."""
    _require(points, 'points')
    _require(E, 'E')
    ndim = len(nc)
    n_theta = E.shape[0]
    broadcast = int(points.dim() == 3 and points.shape[0] == n_theta)
    nP = points.shape[-1]
    out = torch.empty((n_theta, ndim, nP), device=points.device, dtype=torch.float32)
    cells = torch.empty((n_theta, nP, int(nsteps)), device=points.device, dtype=torch.int32)
    _check(load().cpab_integrate_trace(ndim, _ints(nc), int(nsteps), _ptr(points), broadcast, nP,
                                       _ptr(E), n_theta, _ptr(out), _ptr(cells),
                                       _stream(points.device)))
    return out, cells


def backward(nc, nsteps, mode, points, A, E, basis, grad_out, want_dpoints=False, ties=None,
             workspace=None):
    """dtheta [n_theta, d] (and dL/dpoints per theta) from dL/d(out)."""
    _require(points, 'points')
    _require(A, 'A')
    _require(basis, 'basis')
    _require(grad_out, 'grad_out')
    if mode == GRAD_EXACT:
        _require(E, 'E')
    ndim = len(nc)
    n_theta = A.shape[0]
    d = basis.shape[1]
    broadcast = int(points.dim() == 3 and points.shape[0] == n_theta)
    nP = points.shape[-1]
    dev = points.device
    dtheta = torch.empty((n_theta, d), device=dev, dtype=torch.float32)
    dpoints = torch.empty((n_theta, ndim, nP), device=dev, dtype=torch.float32) \
        if want_dpoints else None
    lib = load()
    need = lib.cpab_backward_workspace(ndim, _ints(nc), int(nsteps), nP, n_theta)
    if need == 0 and nP > 0 and n_theta > 0:
        _check(3)
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(max(need, 1), device=dev, dtype=torch.uint8)
    _check(lib.cpab_backward(ndim, _ints(nc), int(nsteps), int(mode), _ptr(points), broadcast, nP,
                             _ptr(A), _ptr(E), n_theta, _ptr(basis), d, _ptr(grad_out),
                             _ptr(dtheta), _ptr(dpoints), _ptr(workspace), workspace.numel(),
                             _ptr(ties), _stream(dev)))
    return dtheta, dpoints


def interpolate(data, grid, outsize):
    _require(data, 'data')
    _require(grid, 'grid')
    ndim = grid.shape[1]
    nb, C = data.shape[0], data.shape[1]
    out = torch.empty((nb, C, *[int(o) for o in outsize]), device=data.device,
                      dtype=torch.float32)
    _check(load().cpab_interpolate(ndim, _ptr(data), nb, C, _ints(data.shape[2:]), _ptr(grid),
                                   _ints(outsize), _ptr(out), _stream(data.device)))
    return out


def interpolate_backward(data, grid, outsize, grad_out, want_ddata=True, want_dgrid=True):
    _require(data, 'data')
    _require(grid, 'grid')
    _require(grad_out, 'grad_out')
    ndim = grid.shape[1]
    nb, C = data.shape[0], data.shape[1]
    ddata = torch.empty_like(data) if want_ddata else None
    dgrid = torch.empty_like(grid) if want_dgrid else None
    _check(load().cpab_interpolate_backward(ndim, _ptr(data), nb, C, _ints(data.shape[2:]),
                                            _ptr(grid), _ints(outsize), _ptr(grad_out),
                                            _ptr(ddata), _ptr(dgrid), _stream(data.device)))
    return ddata, dgrid


def transform_data(nc, nsteps, lin, outsize, E, data, save_grid=False, ties=None, out=None,
                   grid=None):
    """Fused forward; out ([nb, C, *outsize]) and grid ([nb, ndim, prod(outsize)], only with
    save_grid) may be given (contiguous, e.g. batch slices of larger buffers)."""
    _require(lin, 'lin')
    _require(E, 'E')
    _require(data, 'data')
    ndim = len(nc)
    nb, C = data.shape[0], data.shape[1]
    nP = 1
    for o in outsize:
        nP *= int(o)
    oshape = (nb, C, *[int(o) for o in outsize])
    if out is None:
        out = torch.empty(oshape, device=data.device, dtype=torch.float32)
    else:
        _require(out, 'out')
        if tuple(out.shape) != oshape:
            raise ValueError('out must be %s' % (oshape,))
    if not save_grid:
        grid = None
    elif grid is None:
        grid = torch.empty((nb, ndim, nP), device=data.device, dtype=torch.float32)
    else:
        _require(grid, 'grid')
        if tuple(grid.shape) != (nb, ndim, nP):
            raise ValueError('grid must be %s' % ((nb, ndim, nP),))
    _check(load().cpab_transform_data(ndim, _ints(nc), int(nsteps), _ptr(lin), _ints(outsize),
                                      _ptr(E), nb, _ptr(data), C, _ints(data.shape[2:]),
                                      _ptr(out), _ptr(grid), _ptr(ties), _stream(data.device)))
    return out, grid


def transform_grid_image(nc, nsteps, lin, outsize, E, ties=None):
    """The integration half of transform_data: the transformed meshgrid of lin
    for every table, [nb, ndim, prod(outsize)] in image order."""
    _require(lin, 'lin')
    _require(E, 'E')
    ndim = len(nc)
    nb = E.shape[0]
    nP = 1
    for o in outsize:
        nP *= int(o)
    grid = torch.empty((nb, ndim, nP), device=E.device, dtype=torch.float32)
    _check(load().cpab_transform_grid_image(ndim, _ints(nc), int(nsteps), _ptr(lin),
                                            _ints(outsize), _ptr(E), nb, _ptr(grid), _ptr(ties),
                                            _stream(E.device)))
    return grid


def sample_grid(data, grid, outsize):
    """The sampling half of transform_data: data [nb, C, *size] at an
    image-order grid from transform_grid_image."""
    _require(data, 'data')
    _require(grid, 'grid')
    ndim = grid.shape[1]
    nb, C = data.shape[0], data.shape[1]
    out = torch.empty((nb, C, *[int(o) for o in outsize]), device=data.device,
                      dtype=torch.float32)
    _check(load().cpab_sample_grid(ndim, _ptr(data), nb, C, _ints(data.shape[2:]), _ptr(grid),
                                   _ints(outsize), _ptr(out), _stream(data.device)))
    return out


def transform_data_backward(nc, nsteps, mode, lin, outsize, A, E, grid_saved, data, basis,
                            grad_out, want_ddata=True, ties=None, workspace=None):
    _require(lin, 'lin')
    _require(A, 'A')
    _require(data, 'data')
    _require(basis, 'basis')
    _require(grad_out, 'grad_out')
    if mode == GRAD_EXACT:
        _require(E, 'E')
    else:
        _require(grid_saved, 'grid_saved')
    ndim = len(nc)
    nb, C = data.shape[0], data.shape[1]
    d = basis.shape[1]
    dev = data.device
    dtheta = torch.empty((nb, d), device=dev, dtype=torch.float32)
    ddata = torch.empty_like(data) if want_ddata else None
    lib = load()
    need = lib.cpab_transform_data_backward_workspace(ndim, _ints(nc), int(nsteps), int(mode),
                                                      _ints(outsize), nb)
    if need == 0 and nb > 0:
        _check(3)
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(max(need, 1), device=dev, dtype=torch.uint8)
    _check(lib.cpab_transform_data_backward(
        ndim, _ints(nc), int(nsteps), int(mode), _ptr(lin), _ints(outsize), _ptr(A), _ptr(E),
        _ptr(grid_saved), nb, _ptr(data), C, _ints(data.shape[2:]), _ptr(basis), d,
        _ptr(grad_out), _ptr(ddata), _ptr(dtheta), _ptr(workspace), workspace.numel(),
        _ptr(ties), _stream(dev)))
    return ddata, dtheta


def findcellidx(nc, points, ties=None):
    _require(points, 'points')
    ndim = len(nc)
    nP = points.shape[-1]
    out = torch.empty((nP,), device=points.device, dtype=torch.int32)
    _check(load().cpab_findcellidx(ndim, _ints(nc), _ptr(points), nP, _ptr(out), _ptr(ties),
                                   _stream(points.device)))
    return out


def device_status(clear=True) -> int:
    flags = ctypes.c_uint(0)
    _check(load().cpab_device_status(ctypes.byref(flags), int(bool(clear))))
    return flags.value


# ------------------------- ragged batched 1D series ------------------------- #
def _ragged_common(nc, offsets, values):
    if len(nc) != 1:
        raise ValueError('ragged series are 1D (nc has %d entries)' % len(nc))
    _require(offsets, 'offsets', torch.int64)
    _require(values, 'values')
    if offsets.dim() != 1 or offsets.numel() < 1:
        raise ValueError('offsets must be a 1D tensor of S + 1 entries')
    return int(nc[0]), offsets.numel() - 1, values.numel()


def ragged_workspace(nc, nsteps, S, device, workspace=None):
    need = load().cpab_ragged1d_workspace(int(nc), int(nsteps), int(S))
    if need == 0 and S > 0:
        _check(1)
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(max(need, 1), device=device, dtype=torch.uint8)
    return workspace


def ragged_forward(nc, nsteps, E, offsets, values, ties=None, workspace=None):
    """Warped values of every series, [total] (same offsets as values)."""
    n, S, total = _ragged_common(nc, offsets, values)
    _require(E, 'E')
    dev = values.device
    out = torch.empty_like(values)
    ws = ragged_workspace(n, nsteps, S, dev, workspace)
    _check(load().cpab_ragged1d_forward(n, int(nsteps), _ptr(E), S, _ptr(offsets), total,
                                        _ptr(values), _ptr(out), _ptr(ws), ws.numel(), _ptr(ties),
                                        _stream(dev)))
    return out


def ragged_backward(nc, nsteps, mode, A, E, offsets, values, basis, grad_out, want_dvalues=True,
                    ties=None, workspace=None):
    """(dtheta [S, d], dvalues [total] or None) from dL/d(out)."""
    n, S, total = _ragged_common(nc, offsets, values)
    for t, name in ((A, 'A'), (E, 'E'), (basis, 'basis'), (grad_out, 'grad_out')):
        _require(t, name)
    dev = values.device
    d = basis.shape[1]
    dtheta = torch.empty((S, d), device=dev, dtype=torch.float32)
    dvalues = torch.empty_like(values) if want_dvalues else None
    ws = ragged_workspace(n, nsteps, S, dev, workspace)
    _check(load().cpab_ragged1d_backward(n, int(nsteps), int(mode), _ptr(A), _ptr(E), S,
                                         _ptr(offsets), total, _ptr(basis), d, _ptr(values),
                                         _ptr(grad_out), _ptr(dtheta), _ptr(dvalues), _ptr(ws),
                                         ws.numel(), _ptr(ties), _stream(dev)))
    return dtheta, dvalues


def _mse_args(nc, nsteps, mode, A, E, offsets, values, target, basis, loss_scale, want_out,
              want_dvalues, workspace):
    n, S, total = _ragged_common(nc, offsets, values)
    for t, name in ((A, 'A'), (E, 'E'), (basis, 'basis'), (target, 'target')):
        _require(t, name)
    dev = values.device
    d = basis.shape[1]
    if loss_scale is None:
        loss_scale = 2.0 / max(total, 1)
    res = {
        'out': torch.empty_like(values) if want_out else None,
        'sse': torch.empty((S,), device=dev, dtype=torch.float32),
        'dtheta': torch.empty((S, d), device=dev, dtype=torch.float32),
        'dvalues': torch.empty_like(values) if want_dvalues else None,
    }
    ws = ragged_workspace(n, nsteps, S, dev, workspace)
    args = (n, int(nsteps), int(mode), _ptr(A), _ptr(E), S, _ptr(offsets), total, _ptr(basis), d,
            _ptr(values), _ptr(target), float(loss_scale), _ptr(res['out']), _ptr(res['sse']),
            _ptr(res['dtheta']), _ptr(res['dvalues']), _ptr(ws), ws.numel())
    return args, res, dev


def ragged_mse(nc, nsteps, mode, A, E, offsets, values, target, basis, loss_scale=None,
               want_out=False, want_dvalues=True, ties=None, workspace=None):
    """Fused forward + squared-error loss + backward.  Returns a dict with
    out (or None), sse [S], dtheta [S, d] and dvalues (or None); the loss is
    loss_scale/2 * sse.sum() (loss_scale defaults to 2/total: the MSE)."""
    args, res, dev = _mse_args(nc, nsteps, mode, A, E, offsets, values, target, basis,
                               loss_scale, want_out, want_dvalues, workspace)
    _check(load().cpab_ragged1d_mse(*args, _ptr(ties), _stream(dev)))
    return res


def ragged_tune(kind, nc, nsteps, mode, A, E, offsets, values, target, basis, loss_scale=None,
                workspace=None, force=None):
    """Autotune (or, with force = (threads, points per lane), pin) the ragged
    forward (kind 0) or adjoint (kind 1) launch shape on these inputs.
    Returns ((threads, points per lane), best ms, outputs)."""
    args, res, dev = _mse_args(nc, nsteps, mode, A, E, offsets, values, target, basis,
                               loss_scale, True, True, workspace)
    f = None if force is None else (ctypes.c_int * 2)(int(force[0]), int(force[1]))
    shape = (ctypes.c_int * 2)(0, 0)
    ms = ctypes.c_float(0.0)
    _check(load().cpab_ragged1d_tune(int(kind), *args, f, shape, ctypes.byref(ms),
                                     _stream(dev)))
    return (shape[0], shape[1]), ms.value, res


# ------------------------------- composition ------------------------------- #
def _stage_args(ncs, nsteps, Es):
    K = len(ncs)
    ndim = len(ncs[0])
    if any(len(n) != ndim for n in ncs):
        raise ValueError('all transformations of a composition have the same dimension')
    if len(nsteps) != K or len(Es) != K:
        raise ValueError('one nsteps and one table per transformation')
    for k, E in enumerate(Es):
        _require(E, 'E[%d]' % k)
    nc_flat = _ints([x for n in ncs for x in n])
    ptrs = (ctypes.c_void_p * K)(*[E.data_ptr() for E in Es])
    return K, ndim, nc_flat, _ints(nsteps), ptrs


def sequential_transform_data(ncs, nsteps, lin, outsize, Es, data, save_grid=False, ties=None):
    """Fused transform_data through T_K o ... o T_1 (ncs: K tessellations,
    nsteps: K step counts, Es: K compensated tables)."""
    K, ndim, ncf, nsf, ptrs = _stage_args(ncs, nsteps, Es)
    _require(lin, 'lin')
    _require(data, 'data')
    nb, C = data.shape[0], data.shape[1]
    nP = 1
    for o in outsize:
        nP *= int(o)
    out = torch.empty((nb, C, *[int(o) for o in outsize]), device=data.device,
                      dtype=torch.float32)
    grid = torch.empty((nb, ndim, nP), device=data.device, dtype=torch.float32) \
        if save_grid else None
    _check(load().cpab_sequential_transform_data(ndim, K, ncf, nsf, _ptr(lin), _ints(outsize),
                                                 ptrs, nb, _ptr(data), C, _ints(data.shape[2:]),
                                                 _ptr(out), _ptr(grid), _ptr(ties),
                                                 _stream(data.device)))
    return out, grid


def sequential_transform_data_backward(ncs, nsteps, mode, lin, outsize, Es, A_last, grid_saved,
                                       data, basis_last, grad_out, want_ddata=True, ties=None,
                                       workspace=None):
    """(d(data), dtheta of the last transformation) of the fused composition."""
    K, ndim, ncf, nsf, ptrs = _stage_args(ncs, nsteps, Es)
    for t, name in ((lin, 'lin'), (A_last, 'A_last'), (data, 'data'), (basis_last, 'basis_last'),
                    (grad_out, 'grad_out')):
        _require(t, name)
    if mode != GRAD_EXACT:
        _require(grid_saved, 'grid_saved')
    nb, C = data.shape[0], data.shape[1]
    d = basis_last.shape[1]
    dev = data.device
    dtheta = torch.empty((nb, d), device=dev, dtype=torch.float32)
    ddata = torch.empty_like(data) if want_ddata else None
    lib = load()
    need = lib.cpab_transform_data_backward_workspace(ndim, _ints(ncs[-1]), int(nsteps[-1]),
                                                      int(mode), _ints(outsize), nb)
    if need == 0 and nb > 0:
        _check(3)
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(max(need, 1), device=dev, dtype=torch.uint8)
    _check(lib.cpab_sequential_transform_data_backward(
        ndim, K, ncf, nsf, int(mode), _ptr(lin), _ints(outsize), ptrs, _ptr(A_last),
        _ptr(grid_saved), nb, _ptr(data), C, _ints(data.shape[2:]), _ptr(basis_last), d,
        _ptr(grad_out), _ptr(ddata), _ptr(dtheta), _ptr(workspace), workspace.numel(),
        _ptr(ties), _stream(dev)))
    return ddata, dtheta


# --------------------------- ragged point sets ------------------------------ #
def _points_common(nc, offsets, points):
    _require(offsets, 'offsets', torch.int64)
    _require(points, 'points')
    if offsets.dim() != 1 or offsets.numel() < 1:
        raise ValueError('offsets must be a 1D tensor of S + 1 entries')
    if points.dim() != 2 or points.shape[0] != len(nc):
        raise ValueError('points must be [ndim, total] with ndim = %d' % len(nc))
    return len(nc), offsets.numel() - 1, points.shape[1]


def ragged_points_workspace(nc, S, device, workspace=None):
    need = load().cpab_ragged_points_workspace(len(nc), _ints(nc), int(S))
    if need == 0 and S > 0:
        _check(1)
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(max(need, 1), device=device, dtype=torch.uint8)
    return workspace


def ragged_points_forward(nc, nsteps, E, offsets, points, ties=None, workspace=None):
    """Each set's points integrated with its own table: out [ndim, total]."""
    ndim, S, total = _points_common(nc, offsets, points)
    _require(E, 'E')
    dev = points.device
    out = torch.empty_like(points)
    ws = ragged_points_workspace(nc, S, dev, workspace)
    _check(load().cpab_ragged_points_forward(ndim, _ints(nc), int(nsteps), _ptr(E), S,
                                             _ptr(offsets), total, _ptr(points), _ptr(out),
                                             _ptr(ws), ws.numel(), _ptr(ties), _stream(dev)))
    return out


def ragged_points_backward(nc, nsteps, mode, A, E, offsets, points, basis, grad_out,
                           want_dpoints=False, ties=None, workspace=None):
    """(dtheta [S, d], dpoints [ndim, total] or None) from dL/d(out)."""
    ndim, S, total = _points_common(nc, offsets, points)
    _require(A, 'A')
    _require(basis, 'basis')
    _require(grad_out, 'grad_out')
    if E is not None:
        _require(E, 'E')
    dev = points.device
    d = basis.shape[1]
    dtheta = torch.empty((S, d), device=dev, dtype=torch.float32)
    dpoints = torch.empty_like(points) if want_dpoints else None
    ws = ragged_points_workspace(nc, S, dev, workspace)
    _check(load().cpab_ragged_points_backward(ndim, _ints(nc), int(nsteps), int(mode), _ptr(A),
                                              _ptr(E), S, _ptr(offsets), total, _ptr(basis), d,
                                              _ptr(points), _ptr(grad_out), _ptr(dtheta),
                                              _ptr(dpoints), _ptr(ws), ws.numel(), _ptr(ties),
                                              _stream(dev)))
    return dtheta, dpoints


# ------------------------ ragged images (mixed sizes) ----------------------- #
IMAGE_PLAN_FIELDS = 10
RAGGED_MAX_LEN = 1 << 22   # points per set of the ragged point-set kernels


def ragged_images_plan(ndim, sizes, outsizes=None):
    """Host plan of S images of mixed sizes (no CUDA call): (plan int64
    [S + 1, IMAGE_PLAN_FIELDS], (data_points, total, tiles))."""
    import numpy as np
    S = len(sizes)
    flat = [int(x) for sz in sizes for x in sz]
    if len(flat) != S * ndim or (outsizes is not None and len(outsizes) != S):
        raise ValueError('sizes and outsizes must be S tuples of %d extents' % ndim)
    oflat = None if outsizes is None else [int(x) for sz in outsizes for x in sz]
    if oflat is not None and len(oflat) != S * ndim:
        raise ValueError('outsizes must be S tuples of %d extents' % ndim)
    plan = np.zeros((S + 1) * IMAGE_PLAN_FIELDS, dtype=np.int64)
    totals = np.zeros(3, dtype=np.int64)
    sz_c = (ctypes.c_int * max(len(flat), 1))(*flat)
    osz_c = None if oflat is None else (ctypes.c_int * max(len(oflat), 1))(*oflat)
    _check(load().cpab_ragged_images_plan(int(ndim), S, sz_c, osz_c,
                                          ctypes.c_void_p(plan.ctypes.data),
                                          ctypes.c_void_p(totals.ctypes.data)))
    return plan.reshape(S + 1, IMAGE_PLAN_FIELDS), tuple(int(x) for x in totals)


def interpolate_ragged(ndim, plan, totals, data, grid, C):
    """Sample the packed images `data` at `grid` [ndim, total] with the
    device plan [S + 1, IMAGE_PLAN_FIELDS]; returns the packed output
    [C * total]."""
    _require(plan, 'plan', torch.int64)
    _require(data, 'data')
    _require(grid, 'grid')
    data_points, total, tiles = totals
    if data.numel() != C * data_points or grid.shape != (ndim, total):
        raise ValueError('data must hold C * %d values and grid be [%d, %d]'
                         % (data_points, ndim, total))
    out = torch.empty(C * total, device=data.device, dtype=torch.float32)
    _check(load().cpab_interpolate_ragged(int(ndim), plan.shape[0] - 1, int(C), _ptr(plan),
                                          data_points, total, tiles, _ptr(data), _ptr(grid),
                                          _ptr(out), _stream(data.device)))
    return out


def interpolate_ragged_backward(ndim, plan, totals, data, grid, C, grad_out, want_ddata=True,
                                want_dgrid=True):
    """(ddata like data or None, dgrid [ndim, total] or None)."""
    _require(plan, 'plan', torch.int64)
    _require(data, 'data')
    _require(grid, 'grid')
    _require(grad_out, 'grad_out')
    data_points, total, tiles = totals
    if grad_out.numel() != C * total:
        raise ValueError('grad_out must hold C * %d values' % total)
    ddata = torch.empty_like(data) if want_ddata else None
    dgrid = torch.empty_like(grid) if want_dgrid else None
    _check(load().cpab_interpolate_ragged_backward(
        int(ndim), plan.shape[0] - 1, int(C), _ptr(plan), data_points, total, tiles, _ptr(data),
        _ptr(grid), _ptr(grad_out), _ptr(ddata), _ptr(dgrid), _stream(data.device)))
    return ddata, dgrid


# -------------------------------- autotuner --------------------------------- #
SHAPE_FIELDS = 4   # (threads per CTA, points per thread, CTAs per theta/image, table staging)


def _shape_io(force):
    """(force array or None, shape array, best-ms float) for a *_tune call."""
    f = None
    if force is not None:
        force = tuple(int(v) for v in force)
        if len(force) != SHAPE_FIELDS:
            raise ValueError('a launch shape has %d fields' % SHAPE_FIELDS)
        f = (ctypes.c_int * SHAPE_FIELDS)(*force)
    return f, (ctypes.c_int * SHAPE_FIELDS)(), ctypes.c_float(0.0)


def integrate_tune(nc, nsteps, points, E, force=None):
    """Autotune (or, with force, pin) the launch shape of integrate() on these
    inputs.  Returns (shape tuple, best ms, out)."""
    _require(points, 'points')
    _require(E, 'E')
    ndim = len(nc)
    n_theta = E.shape[0]
    broadcast = int(points.dim() == 3 and points.shape[0] == n_theta)
    nP = points.shape[-1]
    out = torch.empty((n_theta, ndim, nP), device=points.device, dtype=torch.float32)
    f, sh, ms = _shape_io(force)
    _check(load().cpab_integrate_tune(ndim, _ints(nc), int(nsteps), _ptr(points), broadcast, nP,
                                      _ptr(E), n_theta, _ptr(out), f, sh, ctypes.byref(ms),
                                      _stream(points.device)))
    return tuple(sh), ms.value, out


def backward_tune(nc, nsteps, mode, points, A, E, basis, grad_out, want_dpoints=False,
                  force=None):
    """Autotune (or pin) the launch shape of backward().  Returns (shape tuple,
    best ms, dtheta, dpoints or None)."""
    _require(points, 'points')
    _require(A, 'A')
    _require(basis, 'basis')
    _require(grad_out, 'grad_out')
    if mode == GRAD_EXACT:
        _require(E, 'E')
    ndim = len(nc)
    n_theta = A.shape[0]
    d = basis.shape[1]
    broadcast = int(points.dim() == 3 and points.shape[0] == n_theta)
    nP = points.shape[-1]
    dev = points.device
    dtheta = torch.empty((n_theta, d), device=dev, dtype=torch.float32)
    dpoints = torch.empty((n_theta, ndim, nP), device=dev, dtype=torch.float32) \
        if want_dpoints else None
    f, sh, ms = _shape_io(force)
    _check(load().cpab_backward_tune(ndim, _ints(nc), int(nsteps), int(mode), _ptr(points),
                                     broadcast, nP, _ptr(A), _ptr(E), n_theta, _ptr(basis), d,
                                     _ptr(grad_out), _ptr(dtheta), _ptr(dpoints), f, sh,
                                     ctypes.byref(ms), _stream(dev)))
    return tuple(sh), ms.value, dtheta, dpoints


def transform_data_tune(nc, nsteps, lin, outsize, E, data, save_grid=False, force=None):
    """Autotune (or pin) the fused forward's launch shape.  Returns (shape
    tuple, best ms, out, grid or None)."""
    _require(lin, 'lin')
    _require(E, 'E')
    _require(data, 'data')
    ndim = len(nc)
    nb, C = data.shape[0], data.shape[1]
    nP = 1
    for o in outsize:
        nP *= int(o)
    out = torch.empty((nb, C, *[int(o) for o in outsize]), device=data.device,
                      dtype=torch.float32)
    grid = torch.empty((nb, ndim, nP), device=data.device, dtype=torch.float32) \
        if save_grid else None
    f, sh, ms = _shape_io(force)
    _check(load().cpab_transform_data_tune(ndim, _ints(nc), int(nsteps), _ptr(lin),
                                           _ints(outsize), _ptr(E), nb, _ptr(data), C,
                                           _ints(data.shape[2:]), _ptr(out), _ptr(grid), f, sh,
                                           ctypes.byref(ms), _stream(data.device)))
    return tuple(sh), ms.value, out, grid


def transform_data_backward_tune(nc, nsteps, mode, lin, outsize, A, E, grid_saved, data, basis,
                                 grad_out, want_ddata=True, force=None):
    """Autotune (or pin) the fused backward's launch shape.  Returns (shape
    tuple, best ms, ddata or None, dtheta)."""
    _require(lin, 'lin')
    _require(A, 'A')
    _require(data, 'data')
    _require(basis, 'basis')
    _require(grad_out, 'grad_out')
    if mode == GRAD_EXACT:
        _require(E, 'E')
    else:
        _require(grid_saved, 'grid_saved')
    ndim = len(nc)
    nb, C = data.shape[0], data.shape[1]
    d = basis.shape[1]
    dev = data.device
    dtheta = torch.empty((nb, d), device=dev, dtype=torch.float32)
    ddata = torch.empty_like(data) if want_ddata else None
    f, sh, ms = _shape_io(force)
    _check(load().cpab_transform_data_backward_tune(
        ndim, _ints(nc), int(nsteps), int(mode), _ptr(lin), _ints(outsize), _ptr(A), _ptr(E),
        _ptr(grid_saved), nb, _ptr(data), C, _ints(data.shape[2:]), _ptr(basis), d,
        _ptr(grad_out), _ptr(ddata), _ptr(dtheta), f, sh, ctypes.byref(ms), _stream(dev)))
    return tuple(sh), ms.value, ddata, dtheta


def ragged_points_tune(kind, nc, nsteps, mode, A, E, offsets, points, basis=None, grad_out=None,
                       want_dpoints=False, force=None):
    """Autotune (or pin) the ragged point-set forward (kind 0) or backward
    (kind 1) launch shape.  Returns (shape tuple, best ms, out or None,
    dtheta or None, dpoints or None)."""
    ndim, S, total = _points_common(nc, offsets, points)
    dev = points.device
    out = dtheta = dpoints = None
    d = 0
    if kind == 0:
        _require(E, 'E')
        out = torch.empty_like(points)
    else:
        _require(A, 'A')
        _require(basis, 'basis')
        _require(grad_out, 'grad_out')
        if E is not None:
            _require(E, 'E')
        d = basis.shape[1]
        dtheta = torch.empty((S, d), device=dev, dtype=torch.float32)
        dpoints = torch.empty_like(points) if want_dpoints else None
    f, sh, ms = _shape_io(force)
    _check(load().cpab_ragged_points_tune(int(kind), ndim, _ints(nc), int(nsteps), int(mode),
                                          _ptr(A), _ptr(E), S, _ptr(offsets), total,
                                          _ptr(basis), d, _ptr(points), _ptr(grad_out),
                                          _ptr(out), _ptr(dtheta), _ptr(dpoints), f, sh,
                                          ctypes.byref(ms), _stream(dev)))
    return tuple(sh), ms.value, out, dtheta, dpoints


def tune_reset():
    """Forget every kept launch shape (the ragged 1D series' excepted)."""
    load().cpab_tune_reset()

"""Launch-shape autotuning of the hot kernels, per problem shape.

Each function runs the C-ABI tuner of one operation's kernels (forward and,
optionally, backward) on the caller's own inputs: the candidate launch shapes
(threads per CTA, points per thread, CTAs per theta or image, per-warp table
staging) are timed on the GPU and the fastest is kept by the library for
every later call on the same problem (device, tessellation, nsteps, gradient
mode, sizes).  A launch shape changes only how points are spread over threads
and CTAs: outputs per point are identical under every shape; sums over points
(dtheta, d(data)) change only in their float summation order.

The backward is tuned with a fixed pseudo-random cotangent (the kernel's time
does not depend on its values).  Tuning synchronises the device and cannot run
inside CUDA-graph capture; tune first, then capture.

Results are dicts {'forward': (shape, ms), 'backward': (shape, ms)}; shape is
the C ABI's (threads, points per thread, CTAs per theta/image, staging)
tuple, which `force=` accepts back to restore a saved shape without timing.
"""
from __future__ import annotations

import torch

from . import _native as N
from ._autograd import _mode
from .functions import _check_ragged_points, _require_cuda, basis_on, grid_axes


def _cotangent(shape, device):
    g = torch.Generator(device='cpu').manual_seed(12345)
    return torch.randn(shape, generator=g).to(device)


def _tables(theta, params):
    theta_c = theta.detach().to(torch.float32).contiguous()
    basis = basis_on(params, theta.device)
    A, _, E = N.cell_tables(params.nc, params.nstepsolver, theta_c, basis)
    return A, E, basis


def _fixed_step(params):
    if params.numeric_grad or getattr(params, 'integration', 'fixed_step') != 'fixed_step':
        raise ValueError('tuning covers the fixed-step kernels (integration="fixed_step", '
                         'numeric_grad=False)')


def tune_transform_grid(points, theta, params, backward=True, force=None):
    """Tune the kernels of transformer(points, theta, params).  force: an
    optional {'forward': shape, 'backward': shape} to pin instead of time."""
    _require_cuda(points, theta)
    _fixed_step(params)
    force = force or {}
    pts = points.detach().to(torch.float32).contiguous()
    A, E, basis = _tables(theta, params)
    res = {}
    sh, ms, out = N.integrate_tune(params.nc, params.nstepsolver, pts, E,
                                   force=force.get('forward'))
    res['forward'] = (sh, ms)
    if backward:
        sh, ms, _, _ = N.backward_tune(params.nc, params.nstepsolver, _mode(params), pts, A, E,
                                       basis, _cotangent(out.shape, out.device),
                                       want_dpoints=getattr(params, 'point_gradient', False),
                                       force=force.get('backward'))
        res['backward'] = (sh, ms)
    return res


def tune_transform_data(data, theta, params, outsize, backward=True, force=None):
    """Tune the fused kernels of transform_data(data, theta, params, outsize)."""
    _require_cuda(data, theta)
    _fixed_step(params)
    force = force or {}
    outsize = tuple(int(o) for o in outsize[:params.ndim])
    data_c = data.detach().to(torch.float32).contiguous()
    A, E, basis = _tables(theta, params)
    lin = grid_axes(params, outsize, data.device)
    mode = _mode(params)
    res = {}
    # the backward of the reference modes reads the forward's saved grid
    want_grid = backward and mode != N.GRAD_EXACT
    sh, ms, out, grid = N.transform_data_tune(params.nc, params.nstepsolver, lin, outsize, E,
                                              data_c, save_grid=want_grid,
                                              force=force.get('forward'))
    res['forward'] = (sh, ms)
    if backward:
        sh, ms, _, _ = N.transform_data_backward_tune(
            params.nc, params.nstepsolver, mode, lin, outsize, A, E, grid, data_c, basis,
            _cotangent(out.shape, out.device), want_ddata=True, force=force.get('backward'))
        res['backward'] = (sh, ms)
    return res


def tune_transform_grid_ragged(points, offsets, theta, params, backward=True, force=None):
    """Tune the kernels of transform_grid_ragged(points, offsets, theta, params)
    on the points in the order given (tune on sorted points when the calls use
    sort_by_cell=True)."""
    _require_cuda(points, offsets, theta)
    _check_ragged_points(points, offsets, theta, params)
    _fixed_step(params)
    force = force or {}
    pts = points.detach().to(torch.float32).contiguous()
    offsets = offsets.contiguous()
    A, E, basis = _tables(theta, params)
    mode = _mode(params)
    res = {}
    sh, ms, _, _, _ = N.ragged_points_tune(0, params.nc, params.nstepsolver, mode, A, E, offsets,
                                           pts, force=force.get('forward'))
    res['forward'] = (sh, ms)
    if backward:
        sh, ms, _, _, _ = N.ragged_points_tune(
            1, params.nc, params.nstepsolver, mode, A, E if mode == N.GRAD_EXACT else None,
            offsets, pts, basis=basis, grad_out=_cotangent(pts.shape, pts.device),
            want_dpoints=getattr(params, 'point_gradient', False), force=force.get('backward'))
        res['backward'] = (sh, ms)
    return res


def reset():
    """Forget all kept shapes; later calls use the built-in launch heuristics."""
    N.tune_reset()

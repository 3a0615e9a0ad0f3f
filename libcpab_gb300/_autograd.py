"""torch.autograd.Function wrappers around the C ABI.

TransformGrid  -- forward/backward of transformer (libcpab/pytorch/transformer.py:136-202)
TransformGridNumeric -- forward differences in theta, the scheme the reference's
                  numeric_grad option intends (libcpab/pytorch/transformer.py:205-295)
Interpolate    -- interpolation with its backward (libcpab/pytorch/interpolation.py)
TransformData  -- fused meshgrid -> integrate -> sample (libcpab/cpab.py:304-331)
TransformDataRagged -- the same for many 1D series of uneven lengths in one
                  persistent launch (one theta per series)
TransformGridRagged -- transformer for many point sets of uneven sizes, one
                  theta per set, in one persistent launch

Gradient modes (params.gradient):
  'reference'     -- the reference's analytic gradient: the midpoint-rule
                     sensitivity of libcpab/core/cpab_ops.cu:390-697, evaluated
                     in reverse mode along the reference's own midpoint
                     trajectory (default, for drop-in parity);
  'reference_map' -- the same gradient along the trajectory of the collapsed
                     per-cell midpoint map (fewer instructions per step; its
                     cells can differ from the reference's at boundary ties);
  'exact'         -- the exact derivative of the forward map that was evaluated.
"""
from __future__ import annotations

import torch
from torch.autograd.function import once_differentiable

from . import _native as N


_MODES = {'reference': N.GRAD_REFERENCE, 'exact': N.GRAD_EXACT,
          'reference_map': N.GRAD_REFERENCE_MAP}


def _mode(params):
    g = getattr(params, 'gradient', 'reference')
    if g not in _MODES:
        raise ValueError("params.gradient must be one of %s (got %r)" % (sorted(_MODES), g))
    return _MODES[g]


def _ties(params):
    return getattr(params, 'tie_counter', None)


def _basis(params, device):
    from .functions import basis_on
    return basis_on(params, device)


class TransformGrid(torch.autograd.Function):
    @staticmethod
    def forward(ctx, points, theta, params):
        points = points.detach().to(torch.float32).contiguous()
        theta_c = theta.detach().to(torch.float32).contiguous()
        basis = _basis(params, theta.device)
        ctx.exact = getattr(params, 'integration', 'fixed_step') == 'exact'
        if ctx.exact:
            A, _, E = N.cell_tables(params.nc, params.nstepsolver, theta_c, basis, want_E=False)
            out = N.integrate_exact(params.nc, points, A, ties=_ties(params))
        else:
            A, _, E = N.cell_tables(params.nc, params.nstepsolver, theta_c, basis)
            out = N.integrate(params.nc, params.nstepsolver, points, E, ties=_ties(params))
        # the exact scheme's backward integrates back from its result
        ctx.save_for_backward(points, A, out if ctx.exact else E)
        ctx.params = params
        ctx.points_dim = points.dim()
        ctx.theta_like = (theta_c.shape, theta_c.dtype, theta_c.device)
        # no upstream gradient (e.g. the output only feeds the points of a
        # later transformation) arrives as None instead of zeros
        ctx.set_materialize_grads(False)
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, grad):
        points, A, E = ctx.saved_tensors
        params = ctx.params
        if grad is None:
            # the reference computes this gradient from a zero cotangent: zeros
            shape, dtype, dev = ctx.theta_like
            zeros = torch.zeros(shape, dtype=dtype, device=dev) if ctx.needs_input_grad[1] else None
            return None, zeros, None
        # the reference returns no gradient for the points
        # (libcpab/pytorch/transformer.py:202); params.point_gradient opts in
        want_p = ctx.needs_input_grad[0] and getattr(params, 'point_gradient', False)
        if not (want_p or ctx.needs_input_grad[1]):
            return None, None, None
        if ctx.exact:
            # E holds the forward result here
            dtheta, dpoints = N.backward_exact(params.nc, E, A, _basis(params, points.device),
                                               grad.to(torch.float32).contiguous(),
                                               want_dpoints=want_p, ties=_ties(params))
        else:
            dtheta, dpoints = N.backward(params.nc, params.nstepsolver, _mode(params), points, A,
                                         E, _basis(params, points.device),
                                         grad.to(torch.float32).contiguous(),
                                         want_dpoints=want_p, ties=_ties(params))
        if dpoints is not None and ctx.points_dim == 2:
            dpoints = dpoints.sum(dim=0)
        return dpoints, (dtheta if ctx.needs_input_grad[1] else None), None


class TransformGridNumeric(torch.autograd.Function):
    STEP = 0.01

    @staticmethod
    def forward(ctx, points, theta, params):
        points = points.detach().to(torch.float32).contiguous()
        theta_c = theta.detach().to(torch.float32).contiguous()
        basis = _basis(params, theta.device)
        _, _, E = N.cell_tables(params.nc, params.nstepsolver, theta_c, basis, want_A=False)
        out = N.integrate(params.nc, params.nstepsolver, points, E)
        ctx.save_for_backward(points, theta_c, out)
        ctx.params = params
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, grad):
        points, theta, out = ctx.saved_tensors
        params = ctx.params
        basis = _basis(params, theta.device)
        h = TransformGridNumeric.STEP
        cols = []
        for k in range(theta.shape[1]):
            t = theta.clone()
            t[:, k] += h
            _, _, E = N.cell_tables(params.nc, params.nstepsolver, t, basis, want_A=False)
            o = N.integrate(params.nc, params.nstepsolver, points, E)
            cols.append((grad * (o - out) / h).sum(dim=(1, 2)))
        return None, torch.stack(cols, dim=1), None


class Interpolate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, grid, outsize):
        data_c = data.detach().to(torch.float32).contiguous()
        grid_c = grid.detach().to(torch.float32).contiguous()
        out = N.interpolate(data_c, grid_c, outsize)
        ctx.save_for_backward(data_c, grid_c)
        ctx.outsize = outsize
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, grad):
        data, grid = ctx.saved_tensors
        want_d, want_g = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if not (want_d or want_g):
            return None, None, None
        ddata, dgrid = N.interpolate_backward(data, grid, ctx.outsize,
                                              grad.to(torch.float32).contiguous(),
                                              want_ddata=want_d, want_dgrid=want_g)
        return ddata, dgrid, None


class TransformData(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, theta, params, outsize, staged=None):
        # staged (functions.transform_data_from_host): `data` is still being
        # copied (staged['upload']); the tables and the trajectories
        # (staged['A'], ['E'], ['lin'], ['grid']: integrated before the copy
        # was queued, they need no image) are ready, so the stream waits for
        # the copy and samples (split forward, same bits as the fused one)
        data_c = data.detach().to(torch.float32).contiguous()
        mode = _mode(params)
        needs_grad = ctx.needs_input_grad[0] or ctx.needs_input_grad[1]
        save_grid = needs_grad and mode != N.GRAD_EXACT
        if staged is None:
            theta_c = theta.detach().to(torch.float32).contiguous()
            dev = data.device
            from .functions import grid_axes
            lin = grid_axes(params, outsize, dev)
            A, _, E = N.cell_tables(params.nc, params.nstepsolver, theta_c, _basis(params, dev))
            out, grid = N.transform_data(params.nc, params.nstepsolver, lin, outsize, E, data_c,
                                         save_grid=save_grid, ties=_ties(params))
        else:
            upload = staged['upload']
            if data_c.data_ptr() != upload.tensor.data_ptr():
                raise ValueError('data must be the uploaded tensor')
            A, E, lin, grid = staged['A'], staged['E'], staged['lin'], staged['grid']
            upload.wait()
            out = N.sample_grid(data_c, grid, outsize)
            if not save_grid:
                grid = None
        ctx.save_for_backward(data_c, lin, A, E, grid)
        ctx.params = params
        ctx.outsize = outsize
        ctx.mode = mode
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, grad):
        data, lin, A, E, grid = ctx.saved_tensors
        params = ctx.params
        want_d, want_t = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if not (want_d or want_t):
            return None, None, None, None, None
        ddata, dtheta = N.transform_data_backward(
            params.nc, params.nstepsolver, ctx.mode, lin, ctx.outsize, A, E, grid, data,
            _basis(params, data.device), grad.to(torch.float32).contiguous(), want_ddata=want_d,
            ties=_ties(params))
        return ddata, (dtheta if want_t else None), None, None, None


class TransformDataRagged(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, theta, offsets, params):
        values_c = values.detach().to(torch.float32).contiguous()
        theta_c = theta.detach().to(torch.float32).contiguous()
        basis = _basis(params, values.device)
        A, _, E = N.cell_tables(params.nc, params.nstepsolver, theta_c, basis)
        out = N.ragged_forward(params.nc, params.nstepsolver, E, offsets, values_c,
                               ties=_ties(params))
        ctx.save_for_backward(values_c, offsets, A, E)
        ctx.params = params
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, grad):
        values, offsets, A, E = ctx.saved_tensors
        params = ctx.params
        want_v, want_t = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if not (want_v or want_t):
            return None, None, None, None
        dtheta, dvalues = N.ragged_backward(
            params.nc, params.nstepsolver, _mode(params), A, E, offsets, values,
            _basis(params, values.device), grad.to(torch.float32).contiguous(),
            want_dvalues=want_v, ties=_ties(params))
        return dvalues, (dtheta if want_t else None), None, None


class TransformGridRagged(torch.autograd.Function):
    @staticmethod
    def forward(ctx, points, theta, offsets, params):
        points_c = points.detach().to(torch.float32).contiguous()
        theta_c = theta.detach().to(torch.float32).contiguous()
        basis = _basis(params, points.device)
        mode = _mode(params)
        A, _, E = N.cell_tables(params.nc, params.nstepsolver, theta_c, basis)
        out = N.ragged_points_forward(params.nc, params.nstepsolver, E, offsets, points_c,
                                      ties=_ties(params))
        ctx.save_for_backward(points_c, offsets, A, E if mode == N.GRAD_EXACT else None)
        ctx.params = params
        ctx.mode = mode
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, grad):
        points, offsets, A, E = ctx.saved_tensors
        params = ctx.params
        # as in TransformGrid: no point gradient unless params.point_gradient
        want_p = ctx.needs_input_grad[0] and getattr(params, 'point_gradient', False)
        want_t = ctx.needs_input_grad[1]
        if not (want_p or want_t):
            return None, None, None, None
        dtheta, dpoints = N.ragged_points_backward(
            params.nc, params.nstepsolver, ctx.mode, A, E, offsets, points,
            _basis(params, points.device), grad.to(torch.float32).contiguous(),
            want_dpoints=want_p, ties=_ties(params))
        return dpoints, (dtheta if want_t else None), None, None


class InterpolateRagged(torch.autograd.Function):
    """Packed images of mixed sizes sampled at a ragged grid (one launch each
    way); `layout` is a functions.ImageLayout."""

    @staticmethod
    def forward(ctx, data, grid, layout, C):
        data_c = data.detach().to(torch.float32).contiguous()
        grid_c = grid.detach().to(torch.float32).contiguous()
        out = N.interpolate_ragged(layout.ndim, layout.plan, layout.totals, data_c, grid_c, C)
        ctx.save_for_backward(data_c, grid_c)
        ctx.layout = layout
        ctx.C = C
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, grad):
        data, grid = ctx.saved_tensors
        want_d, want_g = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if not (want_d or want_g):
            return None, None, None, None
        lay = ctx.layout
        ddata, dgrid = N.interpolate_ragged_backward(lay.ndim, lay.plan, lay.totals, data, grid,
                                                     ctx.C, grad.to(torch.float32).contiguous(),
                                                     want_ddata=want_d, want_dgrid=want_g)
        return ddata, dgrid, None, None

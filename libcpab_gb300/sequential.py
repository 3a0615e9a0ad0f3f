"""CpabSequential: a composition of CPAB transformations (libcpab/sequential.py).

Same methods and checks as the reference class.  transform_data (with
output_all=False) runs the whole composition in one fused kernel: every grid
point passes through all transformations in registers and the data is sampled
once at the end (the reference calls transform_grid once per transformation,
with the grid in global memory in between, then interpolates).

Gradients follow the reference: its transform_grid gives the points no
gradient (libcpab/pytorch/transformer.py:202), so only the last theta receives
a non-zero gradient through transform_data (the earlier ones receive zeros,
as autograd hands them a zero cotangent there), and the data receives its
gradient.  A transformation whose solver parameters set point_gradient=True
makes the composition run unfused, so that every theta gets its gradient.
"""
from __future__ import annotations

import torch
from torch.autograd.function import once_differentiable

from . import _native as N
from .cpab import Cpab


def _basis(params, device):
    from .functions import basis_on
    return basis_on(params, device)


class SequentialTransformData(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, params_list, outsize, *thetas):
        from ._autograd import _mode, _ties
        dev = data.device
        data_c = data.detach().to(torch.float32).contiguous()
        last = params_list[-1]
        from .functions import grid_axes
        lin = grid_axes(last, outsize, dev)
        As, Es = [], []
        for p, th in zip(params_list, thetas):
            A, _, E = N.cell_tables(p.nc, p.nstepsolver, th.detach().to(torch.float32).contiguous(),
                                    _basis(p, dev))
            As.append(A)
            Es.append(E)
        mode = _mode(last)
        needs = ctx.needs_input_grad[0] or ctx.needs_input_grad[-1]
        out, grid = N.sequential_transform_data(
            [p.nc for p in params_list], [p.nstepsolver for p in params_list], lin, outsize, Es,
            data_c, save_grid=needs and mode != N.GRAD_EXACT, ties=_ties(last))
        ctx.save_for_backward(data_c, lin, As[-1], grid, *Es)
        ctx.params_list = params_list
        ctx.outsize = outsize
        ctx.mode = mode
        ctx.theta_shapes = [th.shape for th in thetas]
        return out

    @staticmethod
    @once_differentiable
    def backward(ctx, grad):
        from ._autograd import _ties
        data, lin, A_last, grid, *Es = ctx.saved_tensors
        plist = ctx.params_list
        K = len(plist)
        want_d, want_t = ctx.needs_input_grad[0], ctx.needs_input_grad[-1]
        # the earlier thetas: the reference's chain backpropagates a zero
        # cotangent to them (its transform_grid gives the points no gradient)
        none = [torch.zeros(shape, dtype=torch.float32, device=grad.device)
                if ctx.needs_input_grad[3 + k] else None
                for k, shape in enumerate(ctx.theta_shapes[:-1])]
        if not (want_d or want_t):
            return (None, None, None, *none, None)
        last = plist[-1]
        ddata, dtheta = N.sequential_transform_data_backward(
            [p.nc for p in plist], [p.nstepsolver for p in plist], ctx.mode, lin, ctx.outsize,
            list(Es), A_last, grid, data, _basis(last, data.device),
            grad.to(torch.float32).contiguous(), want_ddata=want_d, ties=_ties(last))
        return (ddata, None, None, *none, dtheta if want_t else None)


class CpabSequential(object):
    """Sequence of CPAB transformations (libcpab/sequential.py:15-141)."""

    def __init__(self, *cpab):
        self.n_cpab = len(cpab)
        self.cpab = cpab
        for i in range(self.n_cpab):
            assert isinstance(self.cpab[i], Cpab), \
                ''' Class {0} is not a member of the cpab core class '''.format(i)
        self.ndim = self.cpab[0].params.ndim
        for i in range(1, self.n_cpab):
            assert self.ndim == self.cpab[i].params.ndim, \
                ''' Mismatching dimensionality of transformers. Transformer 1
                have dimensionality {0} but transformer {1} have dimensionality
                {2}'''.format(self.ndim, i + 1, self.cpab[i].params.ndim)
        self.backend = self.cpab[0].backend
        self.backend_name = self.cpab[0].backend_name
        for i in range(1, self.n_cpab):
            assert self.backend_name == self.cpab[i].backend_name, \
                ''' Mismatch in backend. Transformer 1 have backend {0} but
                transformer {1} have backend {2}'''.format(
                    self.backend_name, i + 1, self.cpab[i].backend_name)

    def get_theta_dim(self):
        # the reference returns the bound methods (sequential.py:58); the
        # dimensions are returned here
        return [c.get_theta_dim() for c in self.cpab]

    def get_params(self):
        return [c.get_params() for c in self.cpab]

    def get_basis(self):
        return [c.get_basis() for c in self.cpab]

    def uniform_meshgrid(self, n_points):
        return self.cpab[0].uniform_meshgrid(n_points)

    def sample_transformation(self, n_sample, means=None, covs=None):
        if means is None:
            means = self.n_cpab * [None]
        else:
            assert len(means) == self.n_cpab, ''' The number of supplied means
                should be equal to the number of transformations '''
        if covs is None:
            covs = self.n_cpab * [None]
        else:
            assert len(covs) == self.n_cpab, ''' The number of supplied covariances
                should be equal to the number of transformations '''
        return [c.sample_transformation(n_sample, mean, cov)
                for c, mean, cov in zip(self.cpab, means, covs)]

    def identity(self, n_sample, epsilon=0):
        return [c.identity(n_sample, epsilon) for c in self.cpab]

    def transform_grid(self, grid, thetas, output_all=False):
        self._assert_theta_shape(thetas)
        if not output_all:
            for i in range(self.n_cpab):
                grid = self.cpab[i].transform_grid(grid, thetas[i])
            return grid
        grid = [self.cpab[0].transform_grid(grid, thetas[0])]
        for i in range(1, self.n_cpab):
            grid.append(self.cpab[i].transform_grid(grid[-1], thetas[i]))
        return grid

    def transform_data(self, data, thetas, outsize, output_all=False):
        self._assert_theta_shape(thetas)
        if output_all:
            grid = self.uniform_meshgrid(outsize)
            grid_t = self.transform_grid(grid, thetas, output_all=True)
            return [self.cpab[i].interpolate(data, grid_t[i], outsize)
                    for i in range(self.n_cpab)]
        plist = [c.params for c in self.cpab]
        fused = (1 <= self.n_cpab <= 4
                 and not any(getattr(p, 'point_gradient', False) for p in plist)
                 and not any(p.numeric_grad for p in plist)
                 and all(getattr(p, 'integration', 'fixed_step') == 'fixed_step'
                         for p in plist))
        if not fused:
            grid = self.uniform_meshgrid(outsize)
            grid_t = self.transform_grid(grid, thetas)
            return self.cpab[-1].interpolate(data, grid_t, outsize)
        for c, th in zip(self.cpab, thetas):
            c._check_type(data); c._check_device(data)
            c._check_type(th); c._check_device(th)
        osz = tuple(int(o) for o in outsize[:self.ndim])
        return SequentialTransformData.apply(data, plist, osz, *thetas)

    def _assert_theta_shape(self, thetas):
        n_theta = len(thetas)
        assert n_theta == self.n_cpab, \
            ''' Number of parametrizations needed are {0}'''.format(self.n_cpab)
        batch_size = thetas[0].shape[0]
        for i in range(1, n_theta):
            assert batch_size == thetas[i].shape[0], ''' Batch size should be the
                same for all theta's '''

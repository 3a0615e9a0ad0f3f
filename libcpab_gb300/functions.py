"""Backend module for the Cpab class: the function set of
libcpab/pytorch/functions.py:15-129, computed by the sm_103a kernels.

``transformer``, ``interpolate`` and ``findcellidx`` run on CUDA tensors only;
there is no CPU path.  The small tensor utilities keep the reference's
semantics so that ``Cpab`` code written against libcpab's pytorch backend
binds to this module unchanged (libcpab/cpab.py:112-118 selects a backend
module by name).
"""
from __future__ import annotations

import torch

from . import _native as N
from ._autograd import (TransformGrid, TransformGridNumeric, Interpolate, TransformData,
                        TransformDataRagged)


# ---------------------------------------------------------------- utilities --
def assert_version():
    major, minor = (int(x) for x in torch.__version__.split('+')[0].split('.')[:2])
    assert (major, minor) >= (1, 0), 'PyTorch 1.0 or newer is required'


def _device(device):
    if isinstance(device, str):
        return torch.device('cuda') if device == 'gpu' else torch.device(device)
    return device


def to(x, dtype=torch.float32, device=None):
    return torch.tensor(x, dtype=dtype, device=_device(device))


def tonumpy(x):
    return x.detach().cpu().numpy()


def check_device(x, device_name):
    return x.is_cuda == (device_name == 'gpu')


def backend_type():
    return torch.Tensor


def pdist(mat):
    norm = torch.sum(mat * mat, 1).reshape(-1, 1)
    return norm - 2 * mat.mm(mat.t()) + norm.t()


def norm(x):
    return torch.norm(x)


def matmul(x, y):
    return torch.matmul(x, y)


def transpose(x):
    return x.t()


def exp(x):
    return torch.exp(x)


def zeros(*s, device=None):
    return torch.zeros(*s, device=_device(device))


def ones(*s, device=None):
    return torch.ones(*s, device=_device(device))


def arange(x):
    return torch.arange(x)


def repeat(x, reps):
    return x.repeat(reps)


def batch_repeat(x, reps):
    return x.repeat(reps, *(x.dim() * [1]))


def maximum(x):
    return x.max()


def sample_transformation(d, n_sample=1, mean=None, cov=None, device='cpu'):
    dev = _device(device)
    mean = torch.zeros(d, dtype=torch.float32, device=dev) if mean is None else mean
    cov = torch.eye(d, dtype=torch.float32, device=dev) if cov is None else cov
    dist = torch.distributions.MultivariateNormal(mean, cov)
    return dist.sample((n_sample,)).to(dev)


def identity(d, n_sample=1, epsilon=0, device='cpu'):
    assert epsilon >= 0, 'epsilon need to be larger than 0'
    return torch.zeros(n_sample, d, dtype=torch.float32, device=_device(device)) + epsilon


def linspaces(domain_min, domain_max, n_points, device):
    """Per-axis meshgrid coordinates, exactly as uniform_meshgrid builds them."""
    return [torch.linspace(domain_min[i], domain_max[i], n_points[i], device=_device(device))
            for i in range(len(n_points))]


def uniform_meshgrid(ndim, domain_min, domain_max, n_points, device='cpu'):
    """[ndim, prod(n_points)] grid with the first axis varying fastest
    (libcpab/pytorch/functions.py:102-108)."""
    lin = linspaces(domain_min, domain_max, n_points[:ndim], device)
    mesh = torch.meshgrid(*lin[::-1], indexing='ij')
    return torch.cat([g.reshape(1, -1) for g in mesh[::-1]], dim=0)


# ---------------------------------------------------------------- hot path ---
def basis_on(params, device):
    """fp32 copy of params.basis on `device`, uploaded once and cached."""
    cache = params.__dict__.setdefault('_basis_cache', {})
    key = (str(device), id(params.basis))
    t = cache.get(key)
    if t is None:
        t = torch.as_tensor(params.basis, dtype=torch.float32).to(device).contiguous()
        cache.clear()
        cache[key] = t
    return t


def grid_axes(params, outsize, device):
    """The meshgrid's per-axis coordinates (torch.linspace per axis, as
    uniform_meshgrid builds them) concatenated, for the fused kernels; cached
    per (device, outsize, domain) outside CUDA-graph capture (a tensor made
    during capture only receives its values when the graph replays)."""
    key = (str(device), tuple(int(o) for o in outsize), tuple(params.domain_min[:params.ndim]),
           tuple(params.domain_max[:params.ndim]))
    cache = params.__dict__.setdefault('_axes_cache', {})
    t = cache.get(key)
    if t is not None:
        return t
    t = torch.cat([torch.linspace(params.domain_min[i], params.domain_max[i], outsize[i],
                                  device=device) for i in range(params.ndim)]).contiguous()
    capturing = torch.device(device).type == 'cuda' and torch.cuda.is_current_stream_capturing()
    if not capturing:
        if len(cache) >= 16:
            cache.clear()
        cache[key] = t
    return t


def _require_cuda(*tensors):
    for t in tensors:
        if not t.is_cuda:
            raise ValueError('libcpab_gb300 computes on CUDA tensors only (no CPU fallback); '
                             'got a tensor on %s' % t.device)


def transformer(points, theta, params):
    """Integrate points [ndim, nP] or [n_theta, ndim, nP] through the field of
    every theta [n_theta, d]; returns [n_theta, ndim, nP]
    (libcpab/pytorch/transformer.py:72-87, 131-202)."""
    _require_cuda(points, theta)
    if points.dim() == 3 and points.shape[0] != theta.shape[0]:
        raise ValueError('a batched grid needs one grid per theta (%d vs %d)'
                         % (points.shape[0], theta.shape[0]))
    if points.shape[-2] != params.ndim:
        raise ValueError('points must have %d coordinates (got %d)' % (params.ndim, points.shape[-2]))
    if params.numeric_grad:
        return TransformGridNumeric.apply(points, theta, params)
    return TransformGrid.apply(points, theta, params)


def interpolate(ndim, data, grid, outsize):
    """Sample data [n_b, C, *size] at grid [n_b, ndim, prod(outsize)]
    (libcpab/pytorch/interpolation.py:12-172)."""
    _require_cuda(data, grid)
    outsize = [int(o) for o in outsize]
    if data.dim() != ndim + 2:
        raise ValueError('data must be [n_batch, n_channels, *%dD size]' % ndim)
    if grid.dim() != 3 or grid.shape[1] != ndim or grid.shape[0] != data.shape[0]:
        raise ValueError('grid must be [n_batch=%d, %d, n_points]' % (data.shape[0], ndim))
    n = 1
    for o in outsize[:ndim]:
        n *= o
    if grid.shape[2] != n:
        raise ValueError('grid has %d points but outsize %s needs %d' % (grid.shape[2], outsize, n))
    return Interpolate.apply(data, grid, tuple(outsize[:ndim]))


def transform_data(data, theta, params, outsize):
    """Fused uniform_meshgrid -> transformer -> interpolate (libcpab/cpab.py:304-331)."""
    _require_cuda(data, theta)
    outsize = tuple(int(o) for o in outsize[:params.ndim])
    if data.dim() != params.ndim + 2:
        raise ValueError('data must be [n_batch, n_channels, *%dD size]' % params.ndim)
    if data.shape[0] != theta.shape[0]:
        raise ValueError('data and theta must have the same batch size (%d vs %d)'
                         % (data.shape[0], theta.shape[0]))
    if params.numeric_grad or getattr(params, 'integration', 'fixed_step') == 'exact':
        grid = uniform_meshgrid(params.ndim, params.domain_min, params.domain_max, outsize,
                                data.device)
        return interpolate(params.ndim, data, transformer(grid, theta, params), outsize)
    return TransformData.apply(data, theta, params, outsize)


def transform_data_from_host(data, theta, params, outsize, requires_grad=False):
    """transform_data for a batch held in host memory: the batch is copied to
    the GPU on a side stream (host_io.HostUpload) while the trajectories are
    integrated, and sampled once it has arrived.  Same result as
    transform_data(data.cuda(), theta, params, outsize), bit for bit.
    Returns (out, data on the device); with requires_grad the device copy is
    a leaf whose .grad receives d(data)."""
    from .host_io import HostUpload
    _require_cuda(theta)
    if data.is_cuda:
        raise ValueError('transform_data_from_host takes a host tensor (got %s)' % data.device)
    outsize = tuple(int(o) for o in outsize[:params.ndim])
    if data.dim() != params.ndim + 2:
        raise ValueError('data must be [n_batch, n_channels, *%dD size]' % params.ndim)
    if data.shape[0] != theta.shape[0]:
        raise ValueError('data and theta must have the same batch size (%d vs %d)'
                         % (data.shape[0], theta.shape[0]))
    if params.numeric_grad or getattr(params, 'integration', 'fixed_step') == 'exact':
        dev = HostUpload(data, theta.device).wait().requires_grad_(requires_grad)
        return transform_data(dev, theta, params, outsize), dev
    # queue the tables and the integration first (no image needed), then the
    # copy of the images on the side stream, then the sampling (in the
    # autograd Function, which also saves what the backward needs)
    from ._autograd import _ties
    device = theta.device
    lin = grid_axes(params, outsize, device)
    A, _, E = N.cell_tables(params.nc, params.nstepsolver,
                            theta.detach().to(torch.float32).contiguous(),
                            basis_on(params, device))
    grid = N.transform_grid_image(params.nc, params.nstepsolver, lin, outsize, E,
                                  ties=_ties(params))
    up = HostUpload(data, device)
    dev = up.tensor.requires_grad_(requires_grad)
    staged = {'upload': up, 'A': A, 'E': E, 'lin': lin, 'grid': grid}
    return TransformData.apply(dev, theta, params, outsize, staged), dev


def _check_ragged(values, offsets, theta, params):
    _require_cuda(values, offsets, theta)
    if params.ndim != 1:
        raise ValueError('ragged series need a 1D tessellation')
    if values.dim() != 1:
        raise ValueError('values must be 1D: all series concatenated')
    if offsets.dim() != 1 or offsets.dtype != torch.int64:
        raise ValueError('offsets must be a 1D int64 tensor of n_series + 1 entries')
    if theta.dim() != 2 or theta.shape[0] != offsets.numel() - 1:
        raise ValueError('theta must be [n_series=%d, d]' % (offsets.numel() - 1))


def transform_data_ragged(values, offsets, theta, params):
    """Ragged batch of 1D series: series s is values[offsets[s]:offsets[s+1]]
    and is warped by theta[s] exactly as transform_data(values_s[None, None],
    theta[s:s+1], params, [L_s]) would (libcpab/cpab.py:304-331), all series
    in one launch.  Returns the warped values, concatenated like values."""
    _check_ragged(values, offsets, theta, params)
    return TransformDataRagged.apply(values, theta, offsets.contiguous(), params)


def ragged_mse(values, target, offsets, theta, params, loss_scale=None, want_out=False,
               want_dvalues=True, workspace=None):
    """Fused forward + squared-error loss + backward for ragged 1D series.
    Returns a dict: loss (scalar tensor, loss_scale/2 * sum of squared
    residuals; the mean squared error by default), sse [n_series], dtheta
    [n_series, d], dvalues (or None) and out (or None)."""
    _check_ragged(values, offsets, theta, params)
    from ._autograd import _mode, _ties
    basis = basis_on(params, values.device)
    A, _, E = N.cell_tables(params.nc, params.nstepsolver,
                            theta.detach().to(torch.float32).contiguous(), basis)
    if loss_scale is None:
        loss_scale = 2.0 / max(values.numel(), 1)
    res = N.ragged_mse(params.nc, params.nstepsolver, _mode(params), A, E, offsets.contiguous(),
                       values.detach().contiguous(), target.detach().contiguous(), basis,
                       loss_scale=loss_scale, want_out=want_out, want_dvalues=want_dvalues,
                       ties=_ties(params), workspace=workspace)
    res['loss'] = res['sse'].sum() * (0.5 * loss_scale)
    return res


def _check_ragged_points(points, offsets, theta, params):
    if points.dim() != 2 or points.shape[0] != params.ndim:
        raise ValueError('points must be [ndim=%d, total]' % params.ndim)
    if offsets.dim() != 1 or offsets.dtype != torch.int64:
        raise ValueError('offsets must be a 1D int64 tensor of n_sets + 1 entries')
    if theta.dim() != 2 or theta.shape[0] != offsets.numel() - 1:
        raise ValueError('theta must be [n_sets=%d, d]' % (offsets.numel() - 1))


def transform_grid_ragged(points, offsets, theta, params, sort_by_cell=False):
    """Ragged batch of point sets: set s is points[:, offsets[s]:offsets[s+1]]
    and is moved by theta[s] exactly as transformer(points_s, theta[s:s+1],
    params) would (libcpab/pytorch/transformer.py:72-87), all sets in one
    launch.  points [ndim, total] float32, offsets [S+1] int64, theta [S, d];
    returns [ndim, total].

    sort_by_cell=True runs each set's points in the order of their starting
    cell (a stable sort, undone on the output): the same result, faster when
    a set's points are scattered over many cells."""
    _require_cuda(points, offsets, theta)
    _check_ragged_points(points, offsets, theta, params)
    from ._autograd import TransformGridRagged
    offsets = offsets.contiguous()
    if not sort_by_cell or points.shape[1] == 0:
        return TransformGridRagged.apply(points, theta, offsets, params)
    total = points.shape[1]
    nC = N.num_cells(params.nc)
    pos = torch.arange(total, device=points.device)
    set_id = torch.searchsorted(offsets, pos, right=True) - 1
    cell = findcellidx(params.ndim, points, params.nc)
    perm = torch.sort(set_id * nC + cell, stable=True).indices
    inv = torch.empty_like(perm)
    inv[perm] = pos
    out = TransformGridRagged.apply(points[:, perm], theta, offsets, params)
    return out[:, inv]


class ImageLayout:
    """Where S images of mixed sizes sit in the packed buffers of
    transform_data_mixed: the device plan of cpab_ragged_images_plan, the
    point-set offsets (its pts_off column) and the concatenated meshgrids
    [ndim, total] of the outsizes."""

    def __init__(self, params, sizes, outsizes, device):
        self.ndim = params.ndim
        self.sizes = [tuple(s) for s in sizes]
        self.outsizes = [tuple(o) for o in outsizes]
        plan, self.totals = N.ragged_images_plan(self.ndim, self.sizes, self.outsizes)
        self.plan = torch.from_numpy(plan).to(device)
        self.offsets = self.plan[:, 1].contiguous()
        self.npoints = [int(plan[s + 1, 1] - plan[s, 1]) for s in range(len(self.sizes))]
        grids = {}
        for o in set(self.outsizes):
            grids[o] = uniform_meshgrid(self.ndim, params.domain_min, params.domain_max, list(o),
                                        device)
        if self.outsizes:
            self.points = torch.cat([grids[o] for o in self.outsizes], dim=1).contiguous()
        else:
            self.points = torch.empty((self.ndim, 0), device=device)


def image_layout(params, sizes, outsizes, device):
    """ImageLayout for these sizes, cached per (device, sizes, outsizes,
    domain) outside CUDA-graph capture (like grid_axes)."""
    key = (str(device), tuple(sizes), tuple(outsizes), tuple(params.domain_min[:params.ndim]),
           tuple(params.domain_max[:params.ndim]))
    cache = params.__dict__.setdefault('_layout_cache', {})
    lay = cache.get(key)
    if lay is not None:
        return lay
    lay = ImageLayout(params, sizes, outsizes, device)
    capturing = torch.device(device).type == 'cuda' and torch.cuda.is_current_stream_capturing()
    if not capturing:
        if len(cache) >= 16:
            cache.clear()
        cache[key] = lay
    return lay


def _count(extents):
    n = 1
    for e in extents:
        n *= e
    return n


def _mixed_outsizes(ndim, sizes, outsize):
    if outsize is None:
        return list(sizes)
    outsize = list(outsize)
    if len(outsize) == ndim and all(not isinstance(o, (list, tuple)) for o in outsize):
        return [tuple(int(o) for o in outsize)] * len(sizes)
    if len(outsize) != len(sizes):
        raise ValueError('outsize must be None, one size of %d extents, or one per image' % ndim)
    res = [tuple(int(x) for x in o) for o in outsize]
    if any(len(o) != ndim for o in res):
        raise ValueError('every outsize must have %d extents' % ndim)
    return res


def _check_mixed_mode(params):
    if params.numeric_grad or getattr(params, 'integration', 'fixed_step') == 'exact':
        raise ValueError('transform_data_mixed runs the fixed-step scheme with the analytic '
                         'gradient (numeric_grad=False, integration="fixed_step")')


def _mixed_layout(params, sizes, outsize, theta, tensors):
    outsizes = _mixed_outsizes(params.ndim, sizes, outsize)
    if any(_count(o) >= N.RAGGED_MAX_LEN for o in outsizes):
        raise ValueError('transform_data_mixed: every output must have fewer than %d points '
                         '(the ragged integrator\'s per-set limit)' % N.RAGGED_MAX_LEN)
    _require_cuda(theta, *tensors)
    if any(t.device != theta.device for t in tensors):
        raise ValueError('the images and theta must be on the same device (%s)' % theta.device)
    return image_layout(params, sizes, outsizes, theta.device)


def _mixed_apply(packed, theta, params, lay, C):
    from ._autograd import InterpolateRagged, TransformGridRagged
    grid = TransformGridRagged.apply(lay.points, theta, lay.offsets, params)
    return InterpolateRagged.apply(packed, grid, lay, C)


def transform_data_mixed(data, theta, params, outsize=None):
    """Images of mixed sizes, each warped by its own theta, in one
    integration launch and one sampling launch: image s ([C, *size_s], all
    with the same C) comes out exactly as transform_data(data[s][None],
    theta[s:s+1], params, outsize_s)[0] would (libcpab/cpab.py:304-331).
    outsize: None (each image keeps its size), one size for all images, or a
    list of S sizes.  Returns the list of S outputs [C, *outsize_s];
    gradients reach theta and the images."""
    _check_mixed_mode(params)
    data = list(data)
    S = len(data)
    if theta.dim() != 2 or theta.shape[0] != S:
        raise ValueError('theta must be [n_images=%d, d]' % S)
    if S == 0:
        return []
    ndim = params.ndim
    C = data[0].shape[0] if data[0].dim() == ndim + 1 else -1
    for im in data:
        if im.dim() != ndim + 1 or im.shape[0] != C:
            raise ValueError('every image must be [C, *%dD size] with the same C' % ndim)
    sizes = [tuple(int(x) for x in im.shape[1:]) for im in data]
    lay = _mixed_layout(params, sizes, outsize, theta, data)
    packed = torch.cat([im.reshape(-1).to(torch.float32) for im in data])
    out = _mixed_apply(packed, theta, params, lay, C)
    return [o.view(C, *osz) for o, osz in zip(out.split([C * n for n in lay.npoints]),
                                              lay.outsizes)]


def transform_data_packed(data, sizes, theta, params, outsize=None):
    """transform_data_mixed on images already packed in one buffer: data is
    1D, the [C, *size_s] blocks of the S images back to back; returns the
    [C, *outsize_s] blocks of the outputs back to back (1D), and
    back-propagates to data and theta.  Same values as transform_data_mixed,
    without its per-image views (less host work per call)."""
    _check_mixed_mode(params)
    sizes = [tuple(int(x) for x in sz) for sz in sizes]
    S = len(sizes)
    if theta.dim() != 2 or theta.shape[0] != S:
        raise ValueError('theta must be [n_images=%d, d]' % S)
    if any(len(sz) != params.ndim for sz in sizes):
        raise ValueError('every size must have %d extents' % params.ndim)
    if data.dim() != 1:
        raise ValueError('data must be 1D: the images\' [C, *size] blocks back to back')
    if S == 0:
        return data.new_zeros(0, dtype=torch.float32)
    pix = sum(_count(sz) for sz in sizes)
    if pix == 0 or data.numel() % pix:
        raise ValueError('data holds %d values, not C x %d pixels' % (data.numel(), pix))
    lay = _mixed_layout(params, sizes, outsize, theta, [data])
    return _mixed_apply(data.to(torch.float32).contiguous(), theta, params, lay,
                        data.numel() // pix)


def findcellidx(ndim, p, nc):
    """Cell index of each column of p [ndim, nP] (int64), with the reference's
    C++/CUDA lookup rules (libcpab/core/cpab_ops.cpp:26-190)."""
    _require_cuda(p)
    pts = p.detach().to(torch.float32).contiguous()
    return N.findcellidx(list(nc)[:ndim], pts).to(torch.int64)


def calc_vectorfield(grid, theta, params):
    """Velocity at each point of grid [ndim, nP] for one theta
    (libcpab/pytorch/functions.py:111-129)."""
    _require_cuda(grid, theta)
    B = basis_on(params, theta.device)
    As = torch.matmul(B, theta.flatten().to(torch.float32)).reshape(params.nC, *params.Ashape)
    idx = findcellidx(params.ndim, grid, params.nc)
    gh = torch.cat((grid, torch.ones(1, grid.shape[1], device=grid.device, dtype=grid.dtype)), 0)
    v = torch.matmul(As[idx], gh.t()[:, :, None])
    return v[:, :, 0].t()

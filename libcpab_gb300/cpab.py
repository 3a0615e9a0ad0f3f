"""The Cpab class: libcpab's public API (libcpab/cpab.py:16-539) on GB300.

Same constructor arguments, methods, argument checks, tensor layouts and
``params`` fields as the reference.  Only the pytorch backend on the GPU is
provided -- that is the path this library replaces; asking for the numpy or
tensorflow backend or for device='cpu' raises.  The plotting helpers
(visualize_*) need matplotlib and are not provided.
"""
from __future__ import annotations

import os

import numpy as np
import torch

from .tessellation import make_tessellation


class params:
    """Plain attribute container, like libcpab.core.utility.params."""

    def __repr__(self):
        return str({k: v for k, v in self.__dict__.items() if not k.startswith('_')})


def default_basis_dir() -> str:
    d = os.environ.get('CPAB_GB300_BASIS_DIR')
    if d:
        return d
    return os.path.join(os.path.expanduser('~'), '.cache', 'libcpab_gb300', 'basis_files')


class Cpab(object):
    """CPA transformations on a tessellation of [0,1]^ndim (ndim = 1, 2, 3).

    Arguments (libcpab/cpab.py:54-60):
        tess_size: list of cells per dimension
        backend: 'pytorch' (the only backend of this library)
        device: 'gpu' (computation is on the current CUDA device)
        zero_boundary: velocity normal to the domain boundary is zero
        volume_perservation: zero-trace (volume preserving) velocity fields
        override: rebuild the basis even if a cached one exists
        basis_dir: where bases are cached (libcpab's basis_files naming and
            pickle format; a libcpab basis_files directory can be used)
    """

    def __init__(self, tess_size, backend='pytorch', device='gpu', zero_boundary=True,
                 volume_perservation=False, override=False, basis_dir=None):
        self._check_input(tess_size, backend, device, zero_boundary, volume_perservation,
                          override)
        if backend != 'pytorch':
            raise NotImplementedError(
                "libcpab_gb300 provides the pytorch backend only (got backend=%r)" % backend)
        if device != 'gpu':
            raise NotImplementedError(
                "libcpab_gb300 computes on the GPU only (got device=%r); there is no CPU path"
                % device)
        p = params()
        p.nc = list(tess_size)
        p.ndim = len(tess_size)
        p.Ashape = [p.ndim, p.ndim + 1]
        p.valid_outside = not zero_boundary
        p.zero_boundary = zero_boundary
        p.volume_perservation = volume_perservation
        p.domain_max = [1 for _ in p.nc]
        p.domain_min = [0 for _ in p.nc]
        p.inc = [(p.domain_max[i] - p.domain_min[i]) / p.nc[i] for i in range(p.ndim)]
        p.nstepsolver = 50
        p.numeric_grad = False
        p.use_slow = False
        p.gradient = 'reference'
        p.point_gradient = False
        p.integration = 'fixed_step'
        if p.ndim == 1:
            p.nC = p.nc[0]
            p.params_pr_cell = 2
        elif p.ndim == 2:
            p.nC = 4 * int(np.prod(p.nc))
            p.params_pr_cell = 6
        else:
            p.nC = 5 * int(np.prod(p.nc))
            p.params_pr_cell = 12
        self._dir = basis_dir if basis_dir is not None else default_basis_dir()
        self.tesselation = make_tessellation(p.nc, zero_boundary, volume_perservation,
                                             self._dir, override)
        p.constrain_mat = self.tesselation.L
        p.basis = self.tesselation.B
        p.D, p.d = p.basis.shape
        self.params = p
        from . import functions as backend
        self.backend_name = 'pytorch'
        self.backend = backend
        self.device = device.lower()
        self.backend.assert_version()

    # ------------------------------------------------------------- getters --
    def get_theta_dim(self):
        return self.params.d

    def get_params(self):
        return self.params

    def get_basis(self):
        return self.params.basis

    def set_solver_params(self, nstepsolver=50, numeric_grad=False, use_slow=False,
                          gradient=None, point_gradient=None, integration=None):
        """Integration settings (libcpab/cpab.py:140-157).

        use_slow selected the reference's pure-PyTorch loop; the same
        fixed-step scheme always runs in the CUDA kernels here, so it only
        records the flag.  gradient selects the backward: 'reference' (the
        reference's analytic midpoint-rule sensitivity gradient along its own
        midpoint trajectory), 'reference_map' (the same gradient along the
        trajectory of the collapsed per-cell midpoint map: faster, with cells
        that can differ from the reference's at boundary ties) or 'exact' (the
        exact derivative of the forward map).
        point_gradient (default False, as the reference, whose
        transform_grid returns no gradient for the points:
        libcpab/pytorch/transformer.py:202) makes transform_grid also
        return dL/dpoints, e.g. to train every stage of a composition.
        integration: 'fixed_step' (default, the reference's scheme: nstepsolver
        steps of the cell's step map, the cell chosen at the start of each
        step) or 'exact' (opt-in: the true flow of the continuous field for
        time 1, with cell crossings; forward only, nstepsolver unused).
        """
        assert nstepsolver > 0, 'nstepsolver must be a positive number'
        assert type(nstepsolver) == int, 'nstepsolver must be integer'
        assert type(numeric_grad) == bool, 'numeric_grad must be bool'
        assert type(use_slow) == bool, 'use_slow must be bool'
        if gradient is not None:
            assert gradient in ('reference', 'reference_map', 'exact'), \
                "gradient must be 'reference', 'reference_map' or 'exact'"
            self.params.gradient = gradient
        if integration is not None:
            assert integration in ('fixed_step', 'exact'), \
                "integration must be 'fixed_step' or 'exact'"
            self.params.integration = integration
        if point_gradient is not None:
            assert type(point_gradient) == bool, 'point_gradient must be bool'
            self.params.point_gradient = point_gradient
        self.params.nstepsolver = nstepsolver
        self.params.numeric_grad = numeric_grad
        self.params.use_slow = use_slow

    def enable_tie_counter(self, enable=True):
        """Count cell lookups resolved by the FP64 path (boundary ties)."""
        if enable:
            self.params.tie_counter = torch.zeros(1, dtype=torch.int64,
                                                  device=torch.device('cuda'))
        else:
            self.params.tie_counter = None

    def tie_count(self) -> int:
        t = getattr(self.params, 'tie_counter', None)
        return 0 if t is None else int(t.item())

    # ------------------------------------------------------------ sampling --
    def uniform_meshgrid(self, n_points):
        return self.backend.uniform_meshgrid(self.params.ndim, self.params.domain_min,
                                             self.params.domain_max, n_points, self.device)

    def sample_transformation(self, n_sample=1, mean=None, cov=None):
        if mean is not None:
            self._check_type(mean); self._check_device(mean)
        if cov is not None:
            self._check_type(cov); self._check_device(cov)
        samples = self.backend.sample_transformation(self.params.d, n_sample, mean, cov,
                                                     self.device)
        return samples.to(self.backend._device(self.device))

    def sample_transformation_with_prior(self, n_sample=1, mean=None, length_scale=0.1,
                                         output_variance=1):
        """Smooth prior: squared-exponential covariance between cell centres,
        mapped to theta space (libcpab/cpab.py:191-241)."""
        dev = self.backend._device(self.device)
        centers = torch.as_tensor(self.tesselation.get_cell_centers(), dtype=torch.float32,
                                  device=dev)
        dist = self.backend.pdist(centers)
        ppc = self.params.params_pr_cell
        nC = self.params.nC
        big = 100 * dist.max()
        # block (i, j) is big everywhere except its diagonal, which holds dist[i, j]
        cov_init = big.expand(nC * ppc, nC * ppc).clone()
        eye = torch.eye(ppc, dtype=torch.bool, device=dev)
        mask = eye.repeat(nC, nC)
        cov_init[mask] = dist.repeat_interleave(ppc, 0).repeat_interleave(ppc, 1)[mask]
        cov_avees = output_variance ** 2 * torch.exp(-(cov_init / (2 * length_scale ** 2)))
        B = torch.as_tensor(self.params.basis, dtype=torch.float32, device=dev)
        cov_theta = B.t() @ cov_avees @ B
        return self.sample_transformation(n_sample, mean=mean, cov=cov_theta)

    def identity(self, n_sample=1, epsilon=0):
        return self.backend.identity(self.params.d, n_sample, epsilon, self.device)

    # ------------------------------------------------------------- hot path --
    def transform_grid(self, grid, theta):
        """grid [ndim, nP] or [n_batch, ndim, nP], theta [n_batch, d]
        -> [n_batch, ndim, nP] (libcpab/cpab.py:257-277)."""
        self._check_type(grid); self._check_device(grid)
        self._check_type(theta); self._check_device(theta)
        if len(grid.shape) == 3:
            assert grid.shape[0] == theta.shape[0], \
                'When passing a 3D grid, expects the first dimension to be of same length ' \
                'as the first dimension of theta'
        return self.backend.transformer(grid, theta, self.params)

    def interpolate(self, data, grid, outsize):
        """data [n_batch, C, *size], grid [n_batch, ndim, prod(outsize)]
        -> [n_batch, C, *outsize] (libcpab/cpab.py:280-301)."""
        self._check_type(data); self._check_device(data)
        self._check_type(grid); self._check_device(grid)
        return self.backend.interpolate(self.params.ndim, data, grid, outsize)

    def transform_data(self, data, theta, outsize):
        """uniform_meshgrid(outsize) -> transform_grid -> interpolate, fused
        into one kernel (libcpab/cpab.py:304-331)."""
        self._check_type(data); self._check_device(data)
        self._check_type(theta); self._check_device(theta)
        return self.backend.transform_data(data, theta, self.params, outsize)

    def transform_data_from_host(self, data, theta, outsize, requires_grad=False):
        """transform_data with the batch in (pinned) host memory (extension):
        the copy to the GPU runs under the integration of the trajectories.
        Returns (output, the device copy of data); with requires_grad the
        device copy receives d(data) in .grad."""
        self._check_type(theta); self._check_device(theta)
        return self.backend.transform_data_from_host(data, theta, self.params, outsize,
                                                     requires_grad=requires_grad)

    def transform_data_ragged(self, values, offsets, theta):
        """Ragged batch of 1D series (extension; no reference counterpart):
        series s = values[offsets[s]:offsets[s+1]] warped by theta[s] as
        transform_data(values_s[None, None], theta[s:s+1], [L_s]) would, all
        in one launch.  values [total] float32, offsets [S+1] int64 (CUDA)."""
        self._check_type(values); self._check_device(values)
        self._check_type(theta); self._check_device(theta)
        return self.backend.transform_data_ragged(values, offsets, theta, self.params)

    def transform_grid_ragged(self, points, offsets, theta, sort_by_cell=False):
        """Ragged batch of point sets (extension; no reference counterpart):
        set s = points[:, offsets[s]:offsets[s+1]] moved by theta[s] as
        transform_grid(points_s, theta[s:s+1]) would, all in one launch.
        points [ndim, total] float32, offsets [S+1] int64 (CUDA)."""
        self._check_type(points); self._check_device(points)
        self._check_type(theta); self._check_device(theta)
        return self.backend.transform_grid_ragged(points, offsets, theta, self.params,
                                                  sort_by_cell=sort_by_cell)

    def transform_data_mixed(self, data, theta, outsize=None):
        """Images of mixed sizes (extension; no reference counterpart): a list
        of S images [C, *size_s] with theta [S, d]; image s comes out as
        transform_data(data[s][None], theta[s:s+1], outsize_s)[0] would, with
        one integration launch and one sampling launch for all images.
        outsize: None (keep each size), one size, or a list of S sizes."""
        self._check_type(theta); self._check_device(theta)
        for im in data:
            self._check_type(im); self._check_device(im)
        return self.backend.transform_data_mixed(data, theta, self.params, outsize)

    def transform_data_packed(self, data, sizes, theta, outsize=None):
        """transform_data_mixed on images packed in one 1D buffer (their
        [C, *size_s] blocks back to back, sizes: the S sizes); returns the
        outputs' [C, *outsize_s] blocks back to back (extension)."""
        self._check_type(data); self._check_device(data)
        self._check_type(theta); self._check_device(theta)
        return self.backend.transform_data_packed(data, sizes, theta, self.params, outsize)

    def ragged_mse(self, values, target, offsets, theta, **kwargs):
        """Fused forward + mean-squared-error loss + backward for ragged 1D
        series (extension).  Returns a dict with loss, sse, dtheta, dvalues."""
        self._check_type(values); self._check_device(values)
        self._check_type(theta); self._check_device(theta)
        return self.backend.ragged_mse(values, target, offsets, theta, self.params, **kwargs)

    # ------------------------------------------------------------- tuning --
    def tune_transform_grid(self, grid, theta, backward=True, force=None):
        """Autotune the launch shapes of transform_grid (and its backward) for
        these shapes (extension); later calls on the same problem use them.
        Returns {'forward': (shape, ms), 'backward': (shape, ms)}."""
        self._check_type(grid); self._check_device(grid)
        self._check_type(theta); self._check_device(theta)
        from .tuning import tune_transform_grid
        return tune_transform_grid(grid, theta, self.params, backward=backward, force=force)

    def tune_transform_data(self, data, theta, outsize, backward=True, force=None):
        """Autotune the fused transform_data kernels for these shapes (extension)."""
        self._check_type(data); self._check_device(data)
        self._check_type(theta); self._check_device(theta)
        from .tuning import tune_transform_data
        return tune_transform_data(data, theta, self.params, outsize, backward=backward,
                                   force=force)

    def tune_transform_grid_ragged(self, points, offsets, theta, backward=True, force=None):
        """Autotune the ragged point-set kernels for these sets (extension)."""
        self._check_type(points); self._check_device(points)
        self._check_type(theta); self._check_device(theta)
        from .tuning import tune_transform_grid_ragged
        return tune_transform_grid_ragged(points, offsets, theta, self.params,
                                          backward=backward, force=force)

    def calc_vectorfield(self, grid, theta):
        self._check_type(grid); self._check_device(grid)
        self._check_type(theta); self._check_device(theta)
        return self.backend.calc_vectorfield(grid, theta, self.params)

    def visualize_vectorfield(self, *args, **kwargs):
        raise NotImplementedError('plotting (matplotlib) is not part of libcpab_gb300')

    visualize_deformgrid = visualize_vectorfield
    visualize_tesselation = visualize_vectorfield

    # --------------------------------------------------------------- checks --
    def _check_input(self, tess_size, backend, device, zero_boundary, volume_perservation,
                     override):
        assert 0 < len(tess_size) <= 3, 'Transformer only supports 1D, 2D or 3D'
        assert type(tess_size) == list or type(tess_size) == tuple, \
            'Argument tess_size must be a list or tuple'
        assert all(type(e) == int for e in tess_size), \
            'All elements of tess_size must be integers'
        assert all(e > 0 for e in tess_size), 'All elements of tess_size must be positive'
        assert backend in ['numpy', 'tensorflow', 'pytorch'], \
            "Unknown backend, choose between 'numpy', 'tensorflow' or 'pytorch'"
        assert device in ['cpu', 'gpu'], "Unknown device, choose between 'cpu' or 'gpu'"
        if backend == 'numpy':
            assert device == 'cpu', 'Cannot use gpu with numpy backend'
        assert type(zero_boundary) == bool, 'Argument zero_boundary must be True or False'
        assert type(volume_perservation) == bool, \
            'Argument volume_perservation must be True or False'
        assert type(override) == bool, 'Argument override must be True or False'

    def _check_type(self, x):
        assert isinstance(x, self.backend.backend_type()), \
            'Input has type {0} but expected type {1}'.format(type(x), self.backend.backend_type())

    def _check_device(self, x):
        assert self.backend.check_device(x, self.device), \
            'Input is placed on device {0} but the class expects it to be on device {1}'.format(
                str(x.device), self.device)

    def __repr__(self):
        p = self.params
        return ('\n        CPAB transformer class (libcpab_gb300).\n'
                '            Tesselation size:           {0}\n'
                '            Total number of cells:      {1}\n'
                '            Theta size:                 {2}\n'
                '            Domain lower bound:         {3}\n'
                '            Domain upper bound:         {4}\n'
                '            Zero Boundary:              {5}\n'
                '            Volume perservation:        {6}\n'
                '            Backend:                    {7}\n').format(
            p.nc, p.nC, p.d, p.domain_min, p.domain_max, p.zero_boundary,
            p.volume_perservation, self.backend_name)

"""The timed workloads at their full size, through the public API, against the
oracle on sampled rows.

* 1D [50] zero boundary, 16 theta ~ N(0, I), the 1,000-point meshgrid,
  transform_grid (the reference's CPU-runnable configuration): every
  trajectory against the FP64 oracle of the same scheme (C++ cell rules) with
  boundary ties classified; dtheta (reference mode) against the reference's
  analytic gradient (C oracle) for a random cotangent.
* 2D [3,3] zero boundary, 64 theta ~ N(0, 0.25 I), data [64, 3, 224, 224]
  uniform[0,1] smoothed by a 5x5 box filter, transform_data on the 224 x 224
  grid, MSE against the images warped by a second theta ~ N(0, 0.25 I),
  forward and backward through Cpab.transform_data + F.mse_loss + autograd
  (the headline step).  Checked: the fused output equals interpolate of
  transform_grid (bit for bit); 2,048 sampled grid points of every theta and
  the full grid of two theta against the FP64 oracle with ties classified;
  dtheta and d(data) of 16 of the 64 images against the reference's
  algorithm (interpolation adjoint, then its analytic gradient) on the GPU's
  warped grid.

Gates: point error <= 1e-5 of the domain width on trajectories with the
oracle's cells, every other trajectory first diverging within 1e-6 of a
decision boundary; dtheta <= 1e-4 and d(data) <= 1e-5 relative
(max |diff| / max |ref|).  Seeds as in bench.py: theta 0, data 1, second
theta 2.
"""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

from test_gpu_parity import classify_vs_fp64, rel_err

pytestmark = pytest.mark.gpu

NSTEPS = 50


def test_cfg1_transform_grid_full(cuda, oracle):
    from libcpab_gb300 import Cpab, _native as N
    from libcpab_gb300.functions import basis_on
    T = Cpab([50], backend='pytorch', device='gpu', zero_boundary=True,
             volume_perservation=False)
    d = T.get_theta_dim()
    theta = torch.randn(16, d, generator=torch.Generator().manual_seed(0))
    grid = T.uniform_meshgrid([1000])
    th = theta.to(cuda).requires_grad_(True)
    out = T.transform_grid(grid, th)
    _, _, E = N.cell_tables([50], NSTEPS, th.detach(), basis_on(T.params, cuda))
    out_t, cells = N.integrate_trace([50], NSTEPS, grid, E)
    assert torch.equal(out_t, out.detach())
    g = {'nc': np.array([50]), 'B': T.params.basis, 'theta': theta.numpy()}
    clean, ties, n = classify_vs_fp64(g, grid.cpu().numpy(), out_t.cpu().numpy(),
                                      cells.cpu().numpy())
    assert n == 16 * 1000 and ties <= 0.01 * n, (clean, ties)
    # reference-mode dtheta for a random cotangent, all trajectories
    cot = np.random.default_rng(4).standard_normal(out.shape).astype(np.float32)
    (out * torch.tensor(cot, device=cuda)).sum().backward()
    A, _, _ = N.cell_tables([50], NSTEPS, th.detach(), basis_on(T.params, cuda), want_E=False)
    B = T.params.basis
    Bs = B.T.reshape(d, -1, 1, 2).astype(np.float32)
    dth_o = oracle.backward([50], NSTEPS, grid.cpu().numpy(), A.cpu().numpy(), Bs, cot)
    assert rel_err(th.grad.cpu().numpy(), dth_o) <= 1e-4


def headline_inputs(T, cuda):
    d = T.get_theta_dim()
    theta = 0.5 * torch.randn(64, d, generator=torch.Generator().manual_seed(0))
    raw = torch.rand(64, 3, 224, 224, generator=torch.Generator().manual_seed(1))
    data = F.avg_pool2d(raw, kernel_size=5, stride=1, padding=2, count_include_pad=False)
    theta2 = 0.5 * torch.randn(64, d, generator=torch.Generator().manual_seed(2))
    with torch.no_grad():
        target = T.transform_data(data.to(cuda), theta2.to(cuda), [224, 224])
    return theta.to(cuda), data.contiguous().to(cuda), target


def test_cfg2_headline_step_full(cuda, oracle):
    from libcpab_gb300 import Cpab, _native as N
    from libcpab_gb300.functions import basis_on
    T = Cpab([3, 3], backend='pytorch', device='gpu', zero_boundary=True)
    theta, data, target = headline_inputs(T, cuda)
    th = theta.clone().requires_grad_(True)
    dd = data.clone().requires_grad_(True)
    out = T.transform_data(dd, th, [224, 224])
    loss = F.mse_loss(out, target)
    loss.backward()
    assert N.device_status() == 0

    # the fused forward is interpolate(transform_grid(meshgrid)), bit for bit
    mesh = T.uniform_meshgrid([224, 224])
    grid_t = T.transform_grid(mesh, theta)
    assert torch.equal(T.interpolate(data, grid_t, [224, 224]), out.detach())

    # trajectories against the FP64 oracle: 2,048 sampled points of all 64
    # theta, and every point of theta 0 and 63
    B = T.params.basis
    A, _, E = N.cell_tables([3, 3], NSTEPS, theta, basis_on(T.params, cuda))
    cols = np.sort(np.random.default_rng(6).choice(224 * 224, 2048, replace=False))
    pts = mesh[:, torch.tensor(cols, device=cuda)].contiguous()
    out_s, cells_s = N.integrate_trace([3, 3], NSTEPS, pts, E)
    assert torch.equal(out_s, grid_t[:, :, torch.tensor(cols, device=cuda)])
    g = {'nc': np.array([3, 3]), 'B': B, 'theta': theta.cpu().numpy()}
    _, ties, n = classify_vs_fp64(g, pts.cpu().numpy(), out_s.cpu().numpy(),
                                  cells_s.cpu().numpy())
    assert ties <= 1e-3 * n, ties
    for r in (0, 63):
        out_r, cells_r = N.integrate_trace([3, 3], NSTEPS, mesh, E[r:r + 1].contiguous())
        g_r = {'nc': np.array([3, 3]), 'B': B, 'theta': theta[r:r + 1].cpu().numpy()}
        classify_vs_fp64(g_r, mesh.cpu().numpy(), out_r.cpu().numpy(), cells_r.cpu().numpy())

    # gradients of 16 of the 64 images against the reference's algorithm on
    # the GPU's warped grid (each image's gradient depends on it alone)
    rows = torch.arange(0, 64, 4, device=cuda)
    gout = (2.0 / out.numel()) * (out.detach() - target)
    d_np = data[rows].cpu().numpy()
    gt_np = grid_t[rows].cpu().numpy()
    ddata_o, dgrid_o = oracle.interpolate_backward(d_np, gt_np, [224, 224],
                                                   gout[rows].cpu().numpy())
    assert rel_err(dd.grad[rows].cpu().numpy(), ddata_o) <= 1e-5
    nC = B.shape[0] // 6
    Bs = B.T.reshape(B.shape[1], nC, 2, 3).astype(np.float32)
    dth_o = oracle.backward([3, 3], NSTEPS, mesh.cpu().numpy(), A[rows].cpu().numpy(), Bs,
                            dgrid_o)
    assert rel_err(th.grad[rows].cpu().numpy(), dth_o) <= 1e-4

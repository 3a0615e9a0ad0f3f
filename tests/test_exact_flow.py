"""Exact-flow scheme (opt-in; the reference only has the fixed-step scheme).

Gate against its own FP64 oracle (oracle.exact_flow_fp64: the ODE of the
continuous piecewise-affine field integrated by DOP853 at rtol 1e-12, an
independent method): point error <= 1e-5 of the domain width.  Sanity: the
exact flow is the limit of the fixed-step scheme, so the GPU's fixed-step
result with 2000 steps lies within 1e-4 of it.  Its gradient
(cpab_backward_exact) against FP64 forward sensitivities integrated with the
flow (oracle.exact_flow_grad_fp64): dtheta and dpoints within 1e-4 relative.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

CASES = [
    ([50], True, False, 1.0),      # cfg1's tessellation and distribution
    ([100], False, False, 1.0),    # cfg3's
    ([3, 3], True, False, 0.5),    # cfg2's
    ([4, 4], False, False, 0.5),
    ([2, 2, 2], True, True, 1.0),
]


def _setup(nc, zb, vp, std, cuda, n_theta=3, nP=400, seed=0):
    from libcpab_gb300 import _native as N
    from libcpab_gb300.tessellation import make_tessellation
    B = make_tessellation(nc, zb, vp).B
    rng = np.random.default_rng(seed)
    theta = (std * rng.standard_normal((n_theta, B.shape[1]))).astype(np.float32)
    pts = rng.random((len(nc), nP)).astype(np.float32)
    basis = torch.tensor(np.ascontiguousarray(B), dtype=torch.float32, device=cuda)
    th = torch.tensor(theta, device=cuda)
    A, _, _ = N.cell_tables(nc, 50, th, basis, want_E=False)
    return N, B, theta, pts, basis, th, A


@pytest.mark.parametrize('nc,zb,vp,std', CASES)
def test_exact_flow_vs_fp64_oracle(nc, zb, vp, std, cuda):
    from oracle.oracle import exact_flow_fp64
    N, B, theta, pts, basis, th, A = _setup(nc, zb, vp, std, cuda)
    steps = torch.zeros(1, dtype=torch.int64, device=cuda)
    out = N.integrate_exact(nc, torch.tensor(pts, device=cuda), A, steps=steps)
    ref = exact_flow_fp64(B, theta, pts, nc)
    err = np.abs(out.cpu().numpy() - ref).max()
    assert err <= 1e-5, err
    assert N.device_status() == 0
    assert 0 < int(steps.item()) <= 4096 * out.shape[0] * out.shape[-1]


@pytest.mark.parametrize('nc,zb,vp,std', CASES[:4])
def test_exact_flow_is_the_fixed_step_limit(nc, zb, vp, std, cuda):
    N, B, theta, pts, basis, th, A = _setup(nc, zb, vp, std, cuda, nP=2000, seed=1)
    P = torch.tensor(pts, device=cuda)
    out = N.integrate_exact(nc, P, A)
    _, _, E = N.cell_tables(nc, 2000, th, basis)
    fine = N.integrate(nc, 2000, P, E)
    assert float((out - fine).abs().max()) <= 1e-4


@pytest.mark.parametrize('nc,zb,vp,std', CASES)
def test_exact_flow_gradient_vs_fp64_sensitivities(nc, zb, vp, std, cuda):
    """cpab_backward_exact (a reverse sweep that integrates the flow back from
    its result) against FP64 forward sensitivities (oracle.exact_flow_grad_fp64:
    dp/dtheta and dp/dp0 integrated with the flow by DOP853): dtheta and
    dpoints within 1e-4 relative (max |diff| / max |ref|)."""
    from oracle.oracle import exact_flow_grad_fp64
    N, B, theta, pts, basis, th, A = _setup(nc, zb, vp, std, cuda, n_theta=2, nP=48, seed=3)
    P = torch.tensor(pts, device=cuda)
    out = N.integrate_exact(nc, P, A)
    cot = np.random.default_rng(4).standard_normal(out.shape).astype(np.float32)
    dth, dp = N.backward_exact(nc, out, A, basis, torch.tensor(cot, device=cuda),
                               want_dpoints=True)
    assert N.device_status() == 0
    ref_th, ref_p = exact_flow_grad_fp64(B, theta, pts, nc, cot)
    rel = lambda a, b: float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))
    assert rel(dth.cpu().numpy(), ref_th) <= 1e-4, rel(dth.cpu().numpy(), ref_th)
    assert rel(dp.cpu().numpy(), ref_p) <= 1e-4, rel(dp.cpu().numpy(), ref_p)
    # deterministic: the same bits on a second call
    dth2, _ = N.backward_exact(nc, out, A, basis, torch.tensor(cot, device=cuda))
    assert torch.equal(dth, dth2)


def test_exact_flow_public_api(cuda):
    """integration='exact' through the public API: transform_grid and
    transform_data forward and backward (dtheta through autograd equals the
    C ABI's; the data path runs transform_grid then interpolate)."""
    from libcpab_gb300 import Cpab, _native as N
    from libcpab_gb300.functions import basis_on
    T = Cpab([3, 3], backend='pytorch', device='gpu', zero_boundary=True)
    T.set_solver_params(integration='exact')
    g = torch.Generator().manual_seed(2)
    th = (0.5 * torch.randn(2, T.get_theta_dim(), generator=g)).to(cuda).requires_grad_(True)
    grid = T.uniform_meshgrid([20, 20])
    out = T.transform_grid(grid, th)
    data = torch.rand(2, 1, 20, 20, device=cuda)
    img = T.transform_data(data, th, [20, 20])
    assert torch.isfinite(out).all() and torch.isfinite(img).all()
    T2 = Cpab([3, 3], backend='pytorch', device='gpu', zero_boundary=True)
    fixed = T2.transform_grid(grid, th.detach())
    assert float((out.detach() - fixed).abs().max()) < 1e-3     # the schemes differ a little
    w = torch.randn(out.shape, generator=g).to(cuda)
    (out * w).sum().backward()
    A, _, _ = N.cell_tables([3, 3], 50, th.detach(), basis_on(T.params, cuda), want_E=False)
    ref, _ = N.backward_exact([3, 3], out.detach(), A, basis_on(T.params, cuda), w)
    assert torch.equal(th.grad, ref)
    th.grad = None
    img.sum().backward()
    assert th.grad is not None and torch.isfinite(th.grad).all() and th.grad.abs().sum() > 0

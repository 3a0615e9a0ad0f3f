"""CpabSequential (libcpab/sequential.py) and CpabAligner (libcpab/alignment.py).

* The fused composition equals the reference's sequence transform_grid ->
  ... -> transform_grid -> interpolate, bit for bit (same per-stage
  arithmetic), for 2, 3 and 4 stages and in 1D, 2D and 3D.
* Its gradient follows the reference's semantics (the points get no gradient
  from transform_grid, libcpab/pytorch/transformer.py:202): the earlier thetas
  get zeros, the last theta's gradient equals the unfused chain's within the
  summation order tolerance (1e-4 relative), and d(data) is within the
  float-atomic bound.
* With point_gradient the composition runs unfused and every theta gets a
  gradient.
* alignment_by_gradient replayed as a CUDA graph follows the eager loop, and
  both reduce the loss.
"""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _stages(ncs, cuda, zb=True, seed=0, std=0.5):
    from libcpab_gb300 import Cpab
    Ts = [Cpab(list(nc), backend='pytorch', device='gpu', zero_boundary=zb) for nc in ncs]
    g = torch.Generator().manual_seed(seed)
    thetas = [(std * torch.randn(3, T.get_theta_dim(), generator=g)).to(cuda) for T in Ts]
    return Ts, thetas


def _data(shape, cuda, seed=1):
    g = torch.Generator().manual_seed(seed)
    return torch.rand(*shape, generator=g).to(cuda)


def _chain(Ts, thetas, data, outsize):
    grid = Ts[0].uniform_meshgrid(outsize)
    for T, th in zip(Ts, thetas):
        grid = T.transform_grid(grid, th)
    return Ts[-1].interpolate(data, grid, outsize)


@pytest.mark.parametrize('ncs,shape,outsize', [
    ([[2, 2], [3, 3]], (3, 2, 40, 30), (50, 36)),
    ([[3, 3], [2, 2], [4, 4]], (3, 1, 33, 47), (33, 47)),
    ([[2, 2], [2, 3], [3, 2], [4, 4]], (3, 3, 24, 24), (20, 28)),
    ([[10], [20]], (3, 2, 100), (80,)),
    ([[2, 2, 2], [3, 3, 3]], (3, 1, 12, 10, 14), (12, 10, 14)),
])
def test_sequential_fused_forward_matches_chain(ncs, shape, outsize, cuda):
    from libcpab_gb300 import CpabSequential
    Ts, thetas = _stages(ncs, cuda)
    data = _data(shape, cuda)
    S = CpabSequential(*Ts)
    fused = S.transform_data(data, thetas, outsize)
    ref = _chain(Ts, thetas, data, outsize)
    assert torch.equal(fused, ref)
    all_out = S.transform_data(data, thetas, outsize, output_all=True)
    assert len(all_out) == len(Ts) and torch.equal(all_out[-1], ref)


@pytest.mark.parametrize('gradient', ['reference', 'exact'])
def test_sequential_gradient_semantics(gradient, cuda):
    from libcpab_gb300 import CpabSequential
    Ts, thetas = _stages([[2, 2], [3, 3], [2, 3]], cuda)
    for T in Ts:
        T.set_solver_params(nstepsolver=50, gradient=gradient)
    data = _data((3, 3, 40, 30), cuda)
    outsize = (40, 30)
    w = _data((3, 3, 40, 30), cuda, seed=5) - 0.5
    S = CpabSequential(*Ts)
    th_f = [t.clone().requires_grad_(True) for t in thetas]
    d_f = data.clone().requires_grad_(True)
    (S.transform_data(d_f, th_f, outsize) * w).sum().backward()
    th_c = [t.clone().requires_grad_(True) for t in thetas]
    d_c = data.clone().requires_grad_(True)
    (_chain(Ts, th_c, d_c, outsize) * w).sum().backward()
    # the reference's semantics: the earlier thetas receive zero gradients
    for t in th_f[:-1] + th_c[:-1]:
        assert t.grad is not None and torch.count_nonzero(t.grad) == 0
    rel = float((th_f[-1].grad - th_c[-1].grad).abs().max() / th_c[-1].grad.abs().max())
    assert rel <= 1e-4, rel
    # d(data): float-atomic scatter-add, at most 64 terms per element here
    absum = torch.autograd.grad((_chain(Ts, thetas, d_c, outsize) * w.abs()).sum(), d_c)[0]
    assert bool(((d_f.grad - d_c.grad).abs() <= 2 * 64 * 2.0 ** -24 * absum + 1e-12).all())


def test_sequential_point_gradient_trains_every_stage(cuda):
    from libcpab_gb300 import CpabSequential
    Ts, thetas = _stages([[2, 2], [3, 3]], cuda)
    for T in Ts:
        T.set_solver_params(nstepsolver=50, point_gradient=True)
    data = _data((3, 1, 30, 30), cuda)
    th = [t.clone().requires_grad_(True) for t in thetas]
    CpabSequential(*Ts).transform_data(data, th, (30, 30)).sum().backward()
    for t in th:
        assert t.grad is not None and torch.isfinite(t.grad).all() and t.grad.abs().max() > 0


def _pair(cuda):
    from libcpab_gb300 import Cpab
    import torch.nn.functional as F
    T = Cpab([3, 3], backend='pytorch', device='gpu', zero_boundary=True)
    g = torch.Generator().manual_seed(3)
    raw = torch.rand(1, 1, 48, 48, generator=g)
    x1 = F.avg_pool2d(raw, 7, 1, 3, count_include_pad=False).to(cuda).contiguous()
    theta_true = (0.3 * torch.randn(1, T.get_theta_dim(), generator=g)).to(cuda)
    with torch.no_grad():
        x2 = T.transform_data(x1, theta_true, (48, 48))
    return T, x1, x2


def test_aligner_gradient_graph_follows_eager(cuda):
    from libcpab_gb300 import CpabAligner
    T, x1, x2 = _pair(cuda)
    A = CpabAligner(T)
    th_e = A.alignment_by_gradient(x1, x2, maxiter=30, lr=1e-2, graph=False)
    loss_e = A.losses.clone()
    th_g = A.alignment_by_gradient(x1, x2, maxiter=30, lr=1e-2, graph=True)
    loss_g = A.losses.clone()
    assert float(loss_e[-1]) < float(loss_e[0]) and float(loss_g[-1]) < float(loss_g[0])
    assert float((loss_g - loss_e).abs().max() / loss_e.abs().max()) <= 1e-4
    assert float((th_g - th_e).abs().max() / th_e.abs().max()) <= 1e-3


def test_aligner_sampling(cuda):
    from libcpab_gb300 import CpabAligner
    T, x1, x2 = _pair(cuda)
    th = CpabAligner(T).alignment_by_sampling(x1, x2, maxiter=10)
    assert th.shape == (1, T.get_theta_dim()) and torch.isfinite(th).all()

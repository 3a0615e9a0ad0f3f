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
* Against the oracle: each composed stage against the FP64 oracle, the final
  sampling against the oracle's interpolation, the last theta's gradient
  against the reference's algorithm (test_sequential_vs_oracle); three Adam
  iterations of alignment_by_gradient against an FP64 restatement of the
  reference's loop (test_aligner_gradient_vs_oracle).
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


@pytest.mark.parametrize('ncs,shape,outsize', [
    ([[2, 2], [3, 3], [2, 3]], (3, 2, 40, 30), (36, 28)),
    ([[10], [20]], (3, 2, 100), (80,)),
    ([[2, 2, 2], [3, 3, 3]], (3, 1, 12, 10, 14), (12, 10, 14)),
])
def test_sequential_vs_oracle(ncs, shape, outsize, cuda, oracle):
    """Composition against the oracle (libcpab/sequential.py:91-128): every
    stage's map against the FP64 oracle of the same scheme applied to the
    GPU's grid before that stage (<= 1e-5 of the domain width on trajectories
    with the oracle's cells; other trajectories are boundary ties), the final
    sampling bit-identical to the oracle's interpolation of the final grid,
    and the gradient of the last theta (the only one the reference's
    semantics train) within 1e-4 of the reference's algorithm, d(data) within
    1e-5."""
    import numpy as np
    from libcpab_gb300 import CpabSequential, _native as N
    from libcpab_gb300.functions import basis_on
    from oracle.oracle import numpy_transform_grid
    Ts, thetas = _stages(ncs, cuda)
    data = _data(shape, cuda)
    th = [t.clone().requires_grad_(True) for t in thetas]
    dd = data.clone().requires_grad_(True)
    out = CpabSequential(*Ts).transform_data(dd, th, outsize)
    w = torch.randn(out.shape, generator=torch.Generator().manual_seed(9)).to(cuda)
    (out * w).sum().backward()
    grid = Ts[0].uniform_meshgrid(outsize)
    grids = [grid]
    for T, t in zip(Ts, thetas):
        grids.append(T.transform_grid(grids[-1], t))
    ndim = len(outsize)
    for k, (T, t) in enumerate(zip(Ts, thetas)):
        nc = list(ncs[k])
        _, _, E = N.cell_tables(nc, 50, t, basis_on(T.params, cuda))
        src = grids[k]
        out_t, cells = N.integrate_trace(nc, 50, src, E)
        assert torch.equal(out_t, grids[k + 1])
        src_np = src.cpu().numpy()
        for b in range(t.shape[0]):
            p = src_np if src_np.ndim == 2 else src_np[b]
            ref, c64, marg = numpy_transform_grid(T.params.basis, t[b:b + 1].cpu().numpy(), p,
                                                  nc, 50, return_cells=True,
                                                  return_margin='steps', semantics='cpp')
            cg = cells[b:b + 1].cpu().numpy()
            tie = (cg != c64).any(axis=2)
            err = np.abs(out_t[b:b + 1].cpu().numpy() - ref).max(axis=1)
            assert (err[~tie] <= 1e-5).all(), float(err[~tie].max())
            first = (cg != c64).argmax(axis=2)
            ti, pi = np.nonzero(tie)
            assert (marg[ti, pi, first[ti, pi]] < 1e-6).all()
    final = grids[-1].cpu().numpy()
    img_o = oracle.interpolate(data.cpu().numpy(), final, outsize)
    assert np.array_equal(out.detach().cpu().numpy(), img_o)
    ddata_o, dgrid_o = oracle.interpolate_backward(data.cpu().numpy(), final, outsize,
                                                   w.cpu().numpy())
    rel = lambda a, b: float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))
    assert rel(dd.grad.cpu().numpy(), ddata_o) <= 1e-5
    T = Ts[-1]
    B = T.params.basis
    A, _, _ = N.cell_tables(list(ncs[-1]), 50, thetas[-1], basis_on(T.params, cuda),
                            want_E=False)
    Bs = B.T.reshape(B.shape[1], -1, ndim, ndim + 1).astype(np.float32)
    dth_o = oracle.backward(list(ncs[-1]), 50, grids[-2].cpu().numpy(), A.cpu().numpy(), Bs,
                            dgrid_o)
    assert rel(th[-1].grad.cpu().numpy(), dth_o) <= 1e-4
    for t in th[:-1]:
        assert torch.count_nonzero(t.grad) == 0


def test_aligner_gradient_vs_oracle(cuda, oracle):
    """alignment_by_gradient against the reference's loop (libcpab/alignment.py:
    60-87), iteration by iteration on the GPU's own theta path (theta_k from
    runs of k iterations; each starts at identity(1, 1e-6) and is
    deterministic).  At theta_{k-1}: the loss ||transform_data(x1, theta) - x2||
    against the FP64 oracle's warp and the oracle's interpolation (1e-5
    relative), the gradient the loop uses against the reference's algorithm
    (interpolation adjoint, then its analytic gradient, on the GPU's warped
    grid and A table; 1e-4 relative); and
    theta_k against torch's Adam update (betas 0.9 / 0.999, eps 1e-8)
    restated in float64 on the GPU's gradients (1e-5 relative).  Adam's first
    steps are nearly lr * sign(g), so two independent runs would amplify the
    sign of near-zero gradient components; comparing on one theta path
    checks the loss, the gradient and the update each on their own."""
    import numpy as np
    from libcpab_gb300 import CpabAligner, _native as N
    from libcpab_gb300.functions import basis_on
    from oracle.oracle import numpy_transform_grid
    T, x1, x2 = _pair(cuda)
    iters, lr = 3, 1e-2
    path = [T.identity(1, epsilon=1e-6).detach()]
    for k in range(1, iters + 1):
        path.append(CpabAligner(T).alignment_by_gradient(x1, x2, maxiter=k, lr=lr).detach())
    A = CpabAligner(T)
    A.alignment_by_gradient(x1, x2, maxiter=iters, lr=lr)
    losses_gpu = A.losses.cpu().numpy()
    B = T.params.basis
    d = B.shape[1]
    x1n, x2n = x1.cpu().numpy(), x2.cpu().numpy()
    grid = T.uniform_meshgrid((48, 48)).cpu().numpy()
    Bs = B.T.reshape(d, -1, 2, 3).astype(np.float32)
    rel = lambda a, b: float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))
    m = np.zeros(d)
    v = np.zeros(d)
    b1, b2, eps = 0.9, 0.999, 1e-8
    for k in range(1, iters + 1):
        th = path[k - 1]
        t = th.clone().requires_grad_(True)
        torch.norm(T.transform_data(x1, t, outsize=x1.shape[2:]) - x2).backward()
        g_gpu = t.grad.double().cpu().numpy()[0]
        th32 = th.cpu().numpy()
        gt = numpy_transform_grid(B, th32, grid, [3, 3], 50, semantics='cpp').astype(np.float32)
        out = oracle.interpolate(x1n, gt, (48, 48))
        r = out.astype(np.float64) - x2n
        loss = float(np.sqrt((r ** 2).sum()))
        assert abs(losses_gpu[k - 1] - loss) <= 1e-5 * loss, (k, losses_gpu[k - 1], loss)
        # the gradient on the GPU's own warped grid: near the identity every
        # meshgrid point sits on a pixel knot, where the bilinear gradient
        # jumps, so which side a point falls on is decided by its last bits
        gg = T.transform_grid(T.uniform_meshgrid((48, 48)), th).cpu().numpy()
        og = oracle.interpolate(x1n, gg, (48, 48)).astype(np.float64) - x2n
        lg = float(np.sqrt((og ** 2).sum()))
        _, dgrid = oracle.interpolate_backward(x1n, gg, (48, 48), (og / lg).astype(np.float32))
        # the GPU's own A table: near the identity many meshgrid points sit on
        # cell faces at every step, where the reference-mode gradient (which
        # depends on the chosen cell) is decided by the last bits of A
        As, _, _ = N.cell_tables([3, 3], 50, th, basis_on(T.params, cuda), want_E=False)
        g_o = oracle.backward([3, 3], 50, grid, As.cpu().numpy(), Bs, dgrid)[0]
        assert rel(g_gpu, g_o) <= 1e-4, (k, rel(g_gpu, g_o))
        m = b1 * m + (1 - b1) * g_gpu
        v = b2 * v + (1 - b2) * g_gpu * g_gpu
        denom = np.sqrt(v) / np.sqrt(1 - b2 ** k) + eps
        want = th32.astype(np.float64)[0] - (lr / (1 - b1 ** k)) * (m / denom)
        got = path[k].cpu().numpy()[0]
        assert rel(got, want) <= 1e-5, (k, rel(got, want))

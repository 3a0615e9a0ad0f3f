"""GPU parity: the sm_103a kernels (through the C ABI) against the reference's
golden outputs (tests/golden, produced by the reference itself) and against
the CPU oracle.

Tolerances (written where they are used):
  * cell lookup: bit-exact;
  * forward points vs the FP64 oracle of the same scheme: <= 1e-5 of the
    domain width (max over points);
  * dtheta vs the reference's analytic gradient (reference mode) and vs the
    FP64 autograd oracle (exact mode): relative error <= 1e-4, measured as
    max|diff| / max|ref| per config;
  * interpolation: <= 1e-6 absolute for values in [0,1], gradients <= 1e-5
    relative.
"""
import numpy as np
import pytest
import torch

from conftest import SMALL, load_golden

pytestmark = pytest.mark.gpu

NSTEPS = 50


def make_cpab(g, gradient='reference'):
    from libcpab_gb300 import Cpab
    nc = [int(x) for x in g['nc']]
    T = Cpab(nc, backend='pytorch', device='gpu', zero_boundary=bool(g['zero_boundary']),
             volume_perservation=bool(g['volume_perservation']))
    # theta only has a meaning relative to the reference's basis: use it
    T.params.basis = np.asarray(g['B'], dtype=np.float64)
    T.params.D, T.params.d = T.params.basis.shape
    T.set_solver_params(nstepsolver=NSTEPS, gradient=gradient)
    return T


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if b.size == 0:
        assert a.size == 0
        return 0.0
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.mark.parametrize('name', SMALL)
def test_findcellidx_bit_exact(name, cuda):
    from libcpab_gb300 import _native as N
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    P = torch.tensor(g['probe'], device=cuda).contiguous()
    got = N.findcellidx(nc, P).cpu().numpy()
    ref = g['cells_cpp']
    bad = np.nonzero(got != ref)[0]
    assert bad.size == 0, 'cell mismatch at %s: got %s want %s (points %s)' % (
        bad[:5], got[bad[:5]], ref[bad[:5]], g['probe'][:, bad[:5]].T)


@pytest.mark.parametrize('name', SMALL)
def test_findcellidx_random_vs_oracle(name, cuda, oracle):
    from libcpab_gb300 import _native as N
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    rng = np.random.default_rng(7)
    P = rng.uniform(-0.3, 1.3, (len(nc), 200000)).astype(np.float32)
    P[:, :100000] = rng.uniform(0, 1, (len(nc), 100000))
    got = N.findcellidx(nc, torch.tensor(P, device=cuda)).cpu().numpy()
    assert np.array_equal(got, oracle.findcellidx(nc, P))


@pytest.mark.parametrize('name', SMALL)
def test_cell_tables_vs_reference(name, cuda):
    """k_cell_tables against the reference's own tables for the same theta:
    A = B theta (libcpab/pytorch/transformer.py:146-150, an fp32 matmul) and
    the step maps T = expm(A~ / nsteps) (its fp32 Pade expm,
    libcpab/pytorch/expm.py:11-55), and E = T - I against FP64.
    Tolerances: A within 1e-6 of max|A| (fp32 sums in another order); T within
    1e-6 absolute (two fp32 exponentials, entries near 1); E within 1e-5 of
    max|E| of the FP64 step maps minus I (the compensated table keeps the
    increment to full relative precision; T_ref - I loses it to cancellation)."""
    from libcpab_gb300 import _native as N
    from oracle.oracle import step_maps_fp64
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    ndim = len(nc)
    B = np.asarray(g['B'], dtype=np.float64)
    basis = torch.tensor(np.ascontiguousarray(B, dtype=np.float32), device=cuda)
    theta = torch.tensor(np.ascontiguousarray(g['theta'], dtype=np.float32), device=cuda)
    A, T, E = N.cell_tables(nc, NSTEPS, theta, basis, want_T=True)
    A, T, E = A.cpu().numpy(), T.cpu().numpy(), E.cpu().numpy()
    As_ref = np.asarray(g['As_ref'], dtype=np.float64)
    assert A.shape == As_ref.shape
    assert np.abs(A - As_ref).max() <= 1e-6 * max(1.0, np.abs(As_ref).max())
    assert np.abs(T - g['trels_ref']).max() <= 1e-6
    if B.shape[1] == 0:
        assert np.all(E == 0)
        return
    T64 = step_maps_fp64(B, np.asarray(g['theta'], dtype=np.float64), ndim, NSTEPS)
    E64 = T64[:, :, :ndim, :] - np.eye(ndim, ndim + 1)
    assert np.abs(E - E64).max() <= 1e-5 * max(np.abs(E64).max(), 1e-30)


@pytest.mark.parametrize('name', SMALL)
def test_forward_with_reference_step_maps(name, cuda):
    """cpab_forward fed the reference's own fp32 Pade step maps reproduces the
    reference's pytorch-CPU result; differences come only from FMA rounding
    (and from the rare cell choices those roundings flip)."""
    from libcpab_gb300 import _native as N
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    grid = torch.tensor(g['grid'], device=cuda)
    trels = torch.tensor(g['trels_ref'], device=cuda)
    out = N.forward_trels(nc, NSTEPS, grid, trels).cpu().numpy()
    diff = np.abs(out - g['out_cpu32'])
    assert np.quantile(diff, 0.999) <= 1e-5
    assert diff.max() <= 1e-3


TIE_MARGIN = 1e-6     # a step whose FP64 point lies closer than this to a decision boundary is a tie


def traced_forward(T, g, pts, cuda):
    """GPU transform_grid arithmetic (compensated tables) with the cell of every step."""
    from libcpab_gb300 import _native as N
    from libcpab_gb300.functions import basis_on
    nc = [int(x) for x in g['nc']]
    th = torch.tensor(g['theta'], device=cuda)
    _, _, E = N.cell_tables(nc, NSTEPS, th, basis_on(T.params, cuda))
    out, cells = N.integrate_trace(nc, NSTEPS, torch.tensor(pts, device=cuda), E)
    ref_out = T.transform_grid(torch.tensor(pts, device=cuda), th)
    assert torch.equal(out, ref_out)          # the traced kernel is the production arithmetic
    return out.cpu().numpy(), cells.cpu().numpy()


def classify_vs_fp64(g, pts, out, cells, ref=None):
    """Points whose GPU cell sequence equals the FP64 oracle's must agree to
    1e-5 of the domain width.  Every other point must have diverged at a
    boundary tie: at the first step where the cells differ, the FP64 point lay
    within TIE_MARGIN of a decision boundary (the fixed-step scheme is
    discontinuous there, so either cell is a faithful evaluation).  Returns
    (max clean error, tie count, points)."""
    from oracle.oracle import numpy_transform_grid
    nc = [int(x) for x in g['nc']]
    _, cells64, marg = numpy_transform_grid(g['B'], g['theta'], pts, nc, NSTEPS,
                                            return_cells=True, return_margin='steps',
                                            semantics='cpp')
    if ref is None:
        ref = numpy_transform_grid(g['B'], g['theta'], pts, nc, NSTEPS, semantics='cpp')
    diff = cells != cells64                                    # [n_theta, nP, nsteps]
    tie = diff.any(axis=2)
    err = np.abs(out - ref).max(axis=1)                        # [n_theta, nP]
    clean = float(err[~tie].max()) if (~tie).any() else 0.0
    assert clean <= 1e-5, 'max error %.3g on trajectories with the oracle\'s cells' % clean
    first = diff.argmax(axis=2)
    t_idx, p_idx = np.nonzero(tie)
    m = marg[t_idx, p_idx, first[t_idx, p_idx]]
    assert np.all(m < TIE_MARGIN), 'cell divergence away from a boundary (margin %.3g)' % m.max()
    return clean, int(tie.sum()), tie.size


@pytest.mark.parametrize('name', SMALL)
def test_transform_grid_vs_fp64(name, cuda):
    g = load_golden(name)
    T = make_cpab(g)
    out, cells = traced_forward(T, g, g['grid'], cuda)
    classify_vs_fp64(g, g['grid'], out, cells)
    outb, cellsb = traced_forward(T, g, g['grid_b'], cuda)
    _, ties, n = classify_vs_fp64(g, g['grid_b'], outb, cellsb)
    assert ties <= 0.02 * n, 'random points: %d of %d are boundary ties' % (ties, n)


@pytest.mark.parametrize('name', SMALL)
@pytest.mark.parametrize('which', ['grid', 'grid_b'])
@pytest.mark.parametrize('gradient', ['reference', 'reference_map'])
def test_gradient_reference_mode(name, which, gradient, cuda):
    g = load_golden(name)
    T = make_cpab(g, gradient)
    th = torch.tensor(g['theta'], device=cuda, requires_grad=True)
    out = T.transform_grid(torch.tensor(g[which], device=cuda), th)
    (out * torch.tensor(g['cot'], device=cuda)).sum().backward()
    ref = g['dtheta_ref'] if which == 'grid' else g['dtheta_ref_b']
    r = rel_err(th.grad.cpu().numpy(), ref)
    assert r <= 1e-4, 'reference-mode dtheta rel err %.3g' % r


@pytest.mark.parametrize('name', SMALL)
def test_gradient_exact_mode(name, cuda):
    from oracle.oracle import fp64_autograd
    g = load_golden(name)
    T = make_cpab(g, 'exact')
    T.set_solver_params(nstepsolver=NSTEPS, gradient='exact', point_gradient=True)
    nc = [int(x) for x in g['nc']]
    th = torch.tensor(g['theta'], device=cuda, requires_grad=True)
    pts = torch.tensor(g['grid_b'], device=cuda, requires_grad=True)
    out = T.transform_grid(pts, th)
    (out * torch.tensor(g['cot'], device=cuda)).sum().backward()
    # the exact derivative of the map the GPU evaluated: freeze its cells
    _, cells = traced_forward(T, g, g['grid_b'], cuda)
    _, dth, dpts = fp64_autograd(g['B'], g['theta'], g['grid_b'], nc, g['cot'], NSTEPS,
                                 cells=cells)
    r = rel_err(th.grad.cpu().numpy(), dth)
    assert r <= 1e-4, 'exact-mode dtheta rel err %.3g' % r
    rp = rel_err(pts.grad.cpu().numpy(), dpts)
    assert rp <= 1e-4, 'exact-mode dpoints rel err %.3g' % rp


def test_points_get_no_gradient_by_default(cuda):
    """As the reference's analytic gradient (libcpab/pytorch/transformer.py:
    202): transform_grid gives the points no gradient unless point_gradient
    is set."""
    g = load_golden('2d_3x3_zb')
    T = make_cpab(g)
    th = torch.tensor(g['theta'], device=cuda, requires_grad=True)
    pts = torch.tensor(g['grid_b'], device=cuda, requires_grad=True)
    T.transform_grid(pts, th).sum().backward()
    assert pts.grad is None and th.grad is not None
    T.set_solver_params(nstepsolver=NSTEPS, point_gradient=True)
    pts2 = torch.tensor(g['grid_b'], device=cuda, requires_grad=True)
    T.transform_grid(pts2, th).sum().backward()
    assert pts2.grad is not None and torch.isfinite(pts2.grad).all()


@pytest.mark.parametrize('name', SMALL)
def test_backward_deterministic(name, cuda):
    g = load_golden(name)
    res = []
    for mode in ('reference', 'reference_map', 'exact'):
        T = make_cpab(g, mode)
        outs = []
        for _ in range(2):
            th = torch.tensor(g['theta'], device=cuda, requires_grad=True)
            out = T.transform_grid(torch.tensor(g['grid'], device=cuda), th)
            (out * torch.tensor(g['cot'], device=cuda)).sum().backward()
            outs.append(th.grad.cpu().numpy())
        assert np.array_equal(outs[0], outs[1]), mode
        res.append(outs[0])


@pytest.mark.parametrize('name', SMALL)
def test_interpolate_vs_reference(name, cuda):
    g = load_golden(name)
    T = make_cpab(g)
    npts = [int(x) for x in g['npts']]
    data = torch.tensor(g['data'], device=cuda, requires_grad=True)
    grid = torch.tensor(g['out_cpu32'], device=cuda, requires_grad=True)
    out = T.interpolate(data, grid, npts)
    err = np.abs(out.detach().cpu().numpy() - g['interp32']).max()
    assert err <= 1e-6, 'interpolate max abs err %.3g' % err
    (out * torch.tensor(g['icot'], device=cuda)).sum().backward()
    assert rel_err(data.grad.cpu().numpy(), g['interp64_ddata']) <= 1e-5
    assert rel_err(grid.grad.cpu().numpy(), g['interp64_dgrid']) <= 1e-5


@pytest.mark.parametrize('name', SMALL)
@pytest.mark.parametrize('mode', ['reference', 'reference_map', 'exact'])
def test_transform_data_fused_matches_unfused(name, mode, cuda):
    """The fused kernel computes exactly transform_grid followed by
    interpolate; its gradients match the unfused chain."""
    g = load_golden(name)
    T = make_cpab(g, mode)
    osz = [int(x) for x in g['outsize']]
    th = torch.tensor(g['theta'], device=cuda)
    data = torch.tensor(g['data'], device=cuda)
    t1 = th.clone().requires_grad_(True)
    d1 = data.clone().requires_grad_(True)
    fused = T.transform_data(d1, t1, osz)
    t2 = th.clone().requires_grad_(True)
    d2 = data.clone().requires_grad_(True)
    grid = T.uniform_meshgrid(osz)
    unfused = T.interpolate(d2, T.transform_grid(grid, t2), osz)
    assert torch.equal(fused, unfused)
    w = torch.randn(fused.shape, device=cuda, generator=torch.Generator(cuda).manual_seed(3))
    (fused * w).sum().backward()
    (unfused * w).sum().backward()
    assert rel_err(d1.grad.cpu().numpy(), d2.grad.cpu().numpy()) <= 1e-5
    assert rel_err(t1.grad.cpu().numpy(), t2.grad.cpu().numpy()) <= 1e-4


@pytest.mark.parametrize('name', SMALL)
def test_transform_data_vs_reference(name, cuda):
    """End to end against the reference's own transform_data + MSE backward.

    The reference integrates with fp32 T (up to ~3e-5 from FP64), this library
    with compensated increments; bilinear sampling and its gradient are only
    piecewise smooth in the position, so values and gradients differ by more
    than the grids do.  Tolerances: loss 1e-3 relative; dtheta and d(data)
    5e-3 relative (1D, 2D).  In 3D the reference's float clamp puts points at
    exactly x=1 into the cube's first tetrahedron, so zero-boundary points on
    that face follow ulp-dependent paths in both implementations; there only
    the loss is compared (5e-2).  The 1e-4 gradient gate is
    test_transform_data_gradient_chain."""
    g = load_golden(name)
    T = make_cpab(g, 'reference')
    osz = [int(x) for x in g['outsize']]
    th = torch.tensor(g['theta'], device=cuda, requires_grad=True)
    data = torch.tensor(g['data'], device=cuda, requires_grad=True)
    out = T.transform_data(data, th, osz)
    loss = torch.nn.functional.mse_loss(out, torch.tensor(g['td_target'], device=cuda))
    loss.backward()
    ref_loss = float(g['td_loss'])
    if len(osz) == 3:
        assert abs(loss.item() - ref_loss) <= 5e-2 * max(abs(ref_loss), 1e-6)
        return
    assert abs(loss.item() - ref_loss) <= 1e-3 * max(abs(ref_loss), 1e-6)
    assert rel_err(th.grad.cpu().numpy(), g['td_dtheta']) <= 5e-3
    assert rel_err(data.grad.cpu().numpy(), g['td_ddata']) <= 5e-3


@pytest.mark.parametrize('name', SMALL)
def test_transform_data_gradient_chain(name, cuda, oracle):
    """Reference-mode gradients of the fused transform_data against the
    reference's algorithm evaluated on the same transformed grid: the
    interpolation adjoint (C restatement of interpolation.py's autograd) gives
    dL/dgrid, and the reference's analytic gradient (C restatement of
    cpab_ops.cpp's backward) maps it to dtheta.  Gate: dtheta relative error
    <= 1e-4, d(data) <= 1e-5."""
    g = load_golden(name)
    T = make_cpab(g, 'reference')
    nc = [int(x) for x in g['nc']]
    osz = [int(x) for x in g['outsize']]
    theta = g['theta']
    th = torch.tensor(theta, device=cuda, requires_grad=True)
    data = torch.tensor(g['data'], device=cuda, requires_grad=True)
    out = T.transform_data(data, th, osz)
    w = np.random.default_rng(5).standard_normal(out.shape).astype(np.float32)
    (out * torch.tensor(w, device=cuda)).sum().backward()
    grid = T.uniform_meshgrid(osz)
    gt = T.transform_grid(grid, torch.tensor(theta, device=cuda)).cpu().numpy()
    ddata_o, dgrid_o = oracle.interpolate_backward(g['data'], gt, osz, w)
    ndim = len(nc)
    assert rel_err(data.grad.cpu().numpy(), ddata_o) <= 1e-5
    if g['B'].shape[1] == 0:          # empty basis: nothing to differentiate
        assert th.grad.numel() == 0
        return
    nC = g['B'].shape[0] // (ndim * (ndim + 1))
    As = (g['B'] @ theta.astype(np.float64).T).T.reshape(theta.shape[0], nC, ndim, ndim + 1)
    Bs = g['B'].T.reshape(g['B'].shape[1], nC, ndim, ndim + 1)
    dth_o = oracle.backward(nc, NSTEPS, grid.cpu().numpy(), As, Bs, dgrid_o)
    assert rel_err(th.grad.cpu().numpy(), dth_o) <= 1e-4


def test_errors_are_raised(cuda):
    from libcpab_gb300 import Cpab, _native as N
    T = Cpab([2, 2], backend='pytorch', device='gpu')
    th = torch.zeros(2, T.get_theta_dim(), device=cuda)
    with pytest.raises(AssertionError):
        T.transform_grid(torch.zeros(2, 10), th)              # CPU grid
    with pytest.raises(AssertionError):   # one grid per theta (libcpab/cpab.py:271-274)
        T.transform_grid(torch.zeros(3, 2, 10, device=cuda), th)
    with pytest.raises(ValueError):
        T.transform_grid(torch.zeros(3, 10, device=cuda), th)    # 3 coordinates in 2D
    with pytest.raises(ValueError):
        T.interpolate(torch.zeros(2, 1, 5, 5, device=cuda), torch.zeros(2, 2, 7, device=cuda),
                      [3, 3])
    with pytest.raises(N.CpabError):
        N.integrate([2, 2], 0, torch.zeros(2, 4, device=cuda),
                    torch.zeros(1, 16, 2, 3, device=cuda))
    with pytest.raises(NotImplementedError):
        Cpab([2, 2], backend='numpy', device='cpu')
    assert N.device_status() == 0


def test_identity_and_zero_velocity(cuda):
    """theta = 0 is the identity map; points stay where they are."""
    from libcpab_gb300 import Cpab
    for nc in ([5], [3, 3], [2, 2, 2]):
        T = Cpab(nc, backend='pytorch', device='gpu')
        grid = T.uniform_meshgrid([7] * len(nc))
        out = T.transform_grid(grid, T.identity(3))
        assert torch.equal(out, grid.expand(3, *grid.shape))

"""The launch-shape autotuner never changes results.

For transform_grid (integrate + point adjoint), the fused transform_data
forward and backward, and the ragged point-set kernels, every candidate launch
shape is pinned in turn (the tuners' force argument) and its outputs are
compared with the heuristic shape's: point outputs (out, grid, dpoints)
bit for bit, sums over points (dtheta, d(data)) within 1e-5 relative (only
their float summation order changes).  Then a timed tuning run keeps a shape,
and the plain public calls that follow use it and still agree.  Tuning inside
CUDA-graph capture is refused.  Kept shapes are dropped after each test.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NSTEPS = 50


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-30))


@pytest.fixture
def fresh(cuda):
    from libcpab_gb300 import _native as N
    N.tune_reset()
    yield N
    N.tune_reset()


def _forward_shapes(max_ppt=2):
    return [(b, p, 0, -1) for b in (64, 128, 256) for p in (1, 2, 4) if p <= max_ppt]


def _adjoint_shapes(ndim, base_parts):
    out = []
    for g in ((0, 1) if ndim >= 2 else (0,)):
        for b in (64, 128, 256):
            for parts in sorted({base_parts, max(1, base_parts // 2), base_parts * 2}):
                out.append((b, 0, parts, g))
    return out


def _force_or_skip(fn):
    """Run a pinned-shape call; a shape that does not fit the problem
    (CPAB_ERR_UNSUPPORTED) is skipped."""
    from libcpab_gb300._native import CpabError
    try:
        return fn()
    except CpabError as e:
        if 'does not fit' in str(e) or 'too large' in str(e):
            return None
        raise


@pytest.mark.parametrize('nc,mode', [([50], 0), ([3, 3], 0), ([3, 3], 1), ([2, 2, 2], 2)])
def test_transform_grid_shapes(fresh, cuda, nc, mode):
    N = fresh
    from libcpab_gb300 import Cpab
    from libcpab_gb300.functions import basis_on
    T = Cpab(nc, backend='pytorch', device='gpu', zero_boundary=True)
    d = T.get_theta_dim()
    gen = torch.Generator().manual_seed(3)
    theta = (0.5 * torch.randn(12, d, generator=gen)).to(cuda)
    n = {1: 3000, 2: 60, 3: 14}[len(nc)]
    grid = T.uniform_meshgrid([n] * len(nc))
    basis = basis_on(T.params, cuda)
    A, _, E = N.cell_tables(nc, NSTEPS, theta, basis)
    out0 = N.integrate(nc, NSTEPS, grid, E)
    gout = torch.randn(out0.shape, generator=gen).to(cuda)
    dth0, dp0 = N.backward(nc, NSTEPS, mode, grid, A, E, basis, gout, want_dpoints=True)
    for f in _forward_shapes():
        sh, ms, out = N.integrate_tune(nc, NSTEPS, grid, E, force=f)
        assert sh[:2] == f[:2] and ms == 0.0
        assert torch.equal(out, out0), f
    tried = 0
    for f in _adjoint_shapes(len(nc), 8):
        r = _force_or_skip(lambda: N.backward_tune(nc, NSTEPS, mode, grid, A, E, basis, gout,
                                                   want_dpoints=True, force=f))
        if r is None:
            continue
        tried += 1
        sh, _, dth, dp = r
        assert sh[0] == f[0] and sh[3] == f[3]
        assert torch.equal(dp, dp0), f
        assert _rel(dth, dth0) <= 1e-5, f
    assert tried >= 3
    # timed tuning; the plain calls then run the kept shapes
    res = T.tune_transform_grid(grid, theta)
    assert res['forward'][1] > 0 and res['backward'][1] > 0
    assert torch.equal(N.integrate(nc, NSTEPS, grid, E), out0)
    dth, dp = N.backward(nc, NSTEPS, mode, grid, A, E, basis, gout, want_dpoints=True)
    assert torch.equal(dp, dp0) and _rel(dth, dth0) <= 1e-5
    assert N.device_status() == 0


@pytest.mark.parametrize('nc,mode,size', [([3, 3], 0, [48, 40]), ([3, 3], 2, [48, 40]),
                                          ([4], 0, [300]), ([2, 2, 2], 1, [12, 10, 9])])
def test_transform_data_shapes(fresh, cuda, nc, mode, size):
    N = fresh
    from libcpab_gb300 import Cpab
    from libcpab_gb300.functions import basis_on, grid_axes
    T = Cpab(nc, backend='pytorch', device='gpu', zero_boundary=True)
    T.set_solver_params(gradient={0: 'reference', 1: 'exact', 2: 'reference_map'}[mode])
    d = T.get_theta_dim()
    gen = torch.Generator().manual_seed(5)
    nb, C = 6, 2
    theta = (0.5 * torch.randn(nb, d, generator=gen)).to(cuda)
    data = torch.rand(nb, C, *size, generator=gen).to(cuda)
    basis = basis_on(T.params, cuda)
    A, _, E = N.cell_tables(nc, NSTEPS, theta, basis)
    lin = grid_axes(T.params, size, cuda)
    out0, grid0 = N.transform_data(nc, NSTEPS, lin, size, E, data, save_grid=True)
    gout = torch.randn(out0.shape, generator=gen).to(cuda)
    dd0, dth0 = N.transform_data_backward(nc, NSTEPS, mode, lin, size, A, E, grid0, data, basis,
                                          gout)
    for f in _forward_shapes():
        sh, _, out, grid = N.transform_data_tune(nc, NSTEPS, lin, size, E, data, save_grid=True,
                                                 force=f)
        assert sh[:2] == f[:2]
        assert torch.equal(out, out0) and torch.equal(grid, grid0), f
    tried = 0
    for f in _adjoint_shapes(len(nc), 6):
        r = _force_or_skip(lambda: N.transform_data_backward_tune(
            nc, NSTEPS, mode, lin, size, A, E, grid0, data, basis, gout, force=f))
        if r is None:
            continue
        tried += 1
        _, _, dd, dth = r
        assert _rel(dd, dd0) <= 1e-5, f
        assert _rel(dth, dth0) <= 1e-5, f
    assert tried >= 3
    res = T.tune_transform_data(data, theta, size)
    assert res['forward'][1] > 0 and res['backward'][1] > 0
    # the public op after tuning: same forward bits, gradients within the bound
    th = theta.clone().requires_grad_(True)
    dt = data.clone().requires_grad_(True)
    out = T.transform_data(dt, th, size)
    assert torch.equal(out.detach(), out0)
    (out * gout).sum().backward()
    assert _rel(dt.grad, dd0) <= 1e-5 and _rel(th.grad, dth0) <= 1e-5
    assert N.device_status() == 0


@pytest.mark.parametrize('nc,mode', [([20], 0), ([3, 3], 1), ([2, 2, 2], 0)])
def test_ragged_points_shapes(fresh, cuda, nc, mode):
    N = fresh
    from libcpab_gb300 import Cpab
    from libcpab_gb300.functions import basis_on
    T = Cpab(nc, backend='pytorch', device='gpu', zero_boundary=True)
    T.set_solver_params(gradient='exact' if mode == 1 else 'reference', point_gradient=True)
    d = T.get_theta_dim()
    rng = np.random.default_rng(7)
    lengths = [int(x) for x in rng.integers(0, 700, 9)]
    S, total = len(lengths), sum(lengths)
    off = torch.tensor(np.concatenate([[0], np.cumsum(lengths)]), dtype=torch.int64).to(cuda)
    pts = torch.tensor(rng.random((len(nc), total)), dtype=torch.float32).to(cuda)
    theta = torch.tensor(0.5 * rng.standard_normal((S, d)), dtype=torch.float32).to(cuda)
    basis = basis_on(T.params, cuda)
    A, _, E = N.cell_tables(nc, NSTEPS, theta, basis)
    out0 = N.ragged_points_forward(nc, NSTEPS, E, off, pts)
    gout = torch.tensor(rng.standard_normal(pts.shape), dtype=torch.float32).to(cuda)
    Eb = E if mode == 1 else None
    dth0, dp0 = N.ragged_points_backward(nc, NSTEPS, mode, A, Eb, off, pts, basis, gout,
                                         want_dpoints=True)
    for f in _forward_shapes(4):
        sh, _, out, _, _ = N.ragged_points_tune(0, nc, NSTEPS, mode, A, E, off, pts, force=f)
        assert sh[:2] == f[:2]
        assert torch.equal(out, out0), f
    tried = 0
    for b in (64, 128, 256):
        r = _force_or_skip(lambda: N.ragged_points_tune(1, nc, NSTEPS, mode, A, Eb, off, pts,
                                                        basis=basis, grad_out=gout,
                                                        want_dpoints=True, force=(b, 0, 0, -1)))
        if r is None:
            continue
        tried += 1
        _, _, _, dth, dp = r
        assert torch.equal(dp, dp0), b
        assert _rel(dth, dth0) <= 1e-5, b
    assert tried >= 1
    res = T.tune_transform_grid_ragged(pts, off, theta)
    assert res['forward'][1] > 0 and res['backward'][1] > 0
    assert torch.equal(N.ragged_points_forward(nc, NSTEPS, E, off, pts), out0)
    dth, dp = N.ragged_points_backward(nc, NSTEPS, mode, A, Eb, off, pts, basis, gout,
                                       want_dpoints=True)
    assert torch.equal(dp, dp0) and _rel(dth, dth0) <= 1e-5
    assert N.device_status() == 0


def test_tuning_refused_during_capture(fresh, cuda):
    N = fresh
    from libcpab_gb300.functions import basis_on
    from libcpab_gb300 import Cpab
    T = Cpab([3, 3], backend='pytorch', device='gpu', zero_boundary=True)
    theta = torch.zeros(2, T.get_theta_dim(), device=cuda)
    grid = T.uniform_meshgrid([16, 16])
    _, _, E = N.cell_tables([3, 3], NSTEPS, theta, basis_on(T.params, cuda))
    out = torch.empty(2, 2, 256, device=cuda)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    err = None
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            try:
                N.integrate_tune([3, 3], NSTEPS, grid, E)
            except N.CpabError as e:
                err = str(e)
            out.copy_(grid.expand(2, 2, 256))
    assert err is not None and 'capture' in err
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out, grid.expand(2, 2, 256))


def test_forced_shape_validation(fresh, cuda):
    N = fresh
    from libcpab_gb300.functions import basis_on
    from libcpab_gb300 import Cpab
    T = Cpab([3, 3], backend='pytorch', device='gpu', zero_boundary=True)
    theta = torch.zeros(2, T.get_theta_dim(), device=cuda)
    grid = T.uniform_meshgrid([16, 16])
    basis = basis_on(T.params, cuda)
    A, _, E = N.cell_tables([3, 3], NSTEPS, theta, basis)
    for bad in [(48, 1, 0, -1), (512, 1, 0, -1), (128, 3, 0, -1)]:
        with pytest.raises(N.CpabError):
            N.integrate_tune([3, 3], NSTEPS, grid, E, force=bad)
    gout = torch.ones(2, 2, 256, device=cuda)
    for bad in [(96, 0, 4, 0), (128, 0, 0, 0), (128, 0, 4, 2)]:
        with pytest.raises(N.CpabError):
            N.backward_tune([3, 3], NSTEPS, 0, grid, A, E, basis, gout, force=bad)
    assert N.device_status() == 0

"""Ragged point sets (cpab_ragged_points_*): parity on the GPU.

The reference moves each point set with its own theta by one transform_grid
call (libcpab/cpab.py:276-302 -> libcpab/pytorch/transformer.py:72-87).  The
ragged kernels must give, per set, what that per-set path gives:

* forward: bit-identical to cpab_integrate on the set alone (same arithmetic,
  same lookups);
* dtheta: equal to cpab_backward on the set alone within the summation-order
  tolerance (1e-5 relative), and to the golden reference gradients
  (dtheta_ref_b, the reference's analytic gradient with one grid per theta)
  within 1e-4 like the per-set path;
* dpoints: bit-identical to cpab_backward's (each point's adjoint is its own
  computation);
* sorting a set's points by starting cell changes no result bit of the
  forward; empty sets and invalid offsets behave as in the 1D ragged path;
  a CUDA-graph replay equals the eager calls.
"""
import numpy as np
import pytest
import torch

from conftest import SMALL, load_golden

pytestmark = pytest.mark.gpu

NSTEPS = 50


def _cpab(nc, zb=True, seed=0):
    from libcpab_gb300 import Cpab
    T = Cpab(list(nc), backend='pytorch', device='gpu', zero_boundary=zb)
    T.set_solver_params(nstepsolver=NSTEPS)
    return T


def _problem(cuda, nc, lengths, seed=0, zb=True, spread=0.1):
    """S point sets (set s: lengths[s] points in [-spread, 1 + spread]^ndim)
    with theta ~ N(0, I) per set."""
    from libcpab_gb300 import _native as N
    from libcpab_gb300.functions import basis_on
    T = _cpab(nc, zb)
    gen = torch.Generator().manual_seed(seed)
    ndim, S = len(nc), len(lengths)
    theta = torch.randn(S, T.get_theta_dim(), generator=gen).to(cuda)
    off = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    total = int(off[-1])
    pts = (torch.rand(ndim, total, generator=gen) * (1 + 2 * spread) - spread).to(cuda)
    basis = basis_on(T.params, cuda)
    A, _, E = N.cell_tables(list(nc), NSTEPS, theta, basis)
    return dict(T=T, N=N, nc=list(nc), S=S, off=torch.tensor(off, device=cuda), off_h=off,
                pts=pts.contiguous(), theta=theta, basis=basis, A=A, E=E)


def _rel(a, b):
    a, b = a.double().cpu(), b.double().cpu()
    if b.numel() == 0:
        return 0.0
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-30))


LENGTHS = [0, 1, 2, 31, 32, 33, 64, 65, 0, 97, 200, 257, 5, 600]
CASES = [([7], True), ([3, 3], True), ([2, 4], False), ([2, 2, 2], True), ([4, 4, 4], False)]


@pytest.fixture(scope='module', params=CASES, ids=lambda c: 'x'.join(map(str, c[0])))
def prob(request, cuda):
    nc, zb = request.param
    rng = np.random.default_rng(3)
    lengths = LENGTHS + [int(x) for x in rng.integers(1, 300, size=10)]
    return _problem(cuda, nc, lengths, seed=len(nc), zb=zb)


def test_forward_matches_per_set_integrate(prob):
    P, N = prob, prob['N']
    out = N.ragged_points_forward(P['nc'], NSTEPS, P['E'], P['off'], P['pts'])
    for s in range(P['S']):
        a, b = int(P['off_h'][s]), int(P['off_h'][s + 1])
        if a == b:
            continue
        ref = N.integrate(P['nc'], NSTEPS, P['pts'][:, a:b].contiguous(),
                          P['E'][s:s + 1].contiguous())
        assert torch.equal(out[:, a:b], ref[0]), s
    assert N.device_status() == 0


@pytest.mark.parametrize('mode', [0, 1, 2])
def test_backward_matches_per_set_backward(prob, mode):
    P, N = prob, prob['N']
    gen = torch.Generator(device=P['pts'].device).manual_seed(11)
    gout = torch.randn(P['pts'].shape, device=P['pts'].device, generator=gen)
    dth, dp = N.ragged_points_backward(P['nc'], NSTEPS, mode, P['A'], P['E'], P['off'],
                                       P['pts'], P['basis'], gout, want_dpoints=True)
    for s in range(P['S']):
        a, b = int(P['off_h'][s]), int(P['off_h'][s + 1])
        if a == b:
            assert torch.all(dth[s] == 0)
            continue
        rth, rdp = N.backward(P['nc'], NSTEPS, mode, P['pts'][:, a:b].contiguous(),
                              P['A'][s:s + 1].contiguous(), P['E'][s:s + 1].contiguous(),
                              P['basis'], gout[:, a:b][None].contiguous(), want_dpoints=True)
        assert _rel(dth[s], rth[0]) <= 1e-5, (s, _rel(dth[s], rth[0]))
        assert torch.equal(dp[:, a:b], rdp[0]), s
    assert N.device_status() == 0


def test_backward_deterministic(prob):
    P, N = prob, prob['N']
    gout = torch.ones_like(P['pts'])
    r1 = N.ragged_points_backward(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['pts'],
                                  P['basis'], gout)[0]
    r2 = N.ragged_points_backward(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['pts'],
                                  P['basis'], gout)[0]
    assert torch.equal(r1, r2)


@pytest.mark.parametrize('name', SMALL)
def test_golden_reference_gradient(name, cuda):
    """Sets = the golden batched grids (one grid per theta): dtheta in the
    reference's gradient mode against the reference gradient of the
    fixtures."""
    from libcpab_gb300 import Cpab
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    T = Cpab(nc, backend='pytorch', device='gpu', zero_boundary=bool(g['zero_boundary']),
             volume_perservation=bool(g['volume_perservation']))
    T.params.basis = np.asarray(g['B'], dtype=np.float64)
    T.params.D, T.params.d = T.params.basis.shape
    T.set_solver_params(nstepsolver=NSTEPS, gradient='reference')
    grid_b = torch.tensor(g['grid_b'], device=cuda)           # [S, ndim, nP]
    S, ndim, nP = grid_b.shape
    pts = grid_b.permute(1, 0, 2).reshape(ndim, S * nP).contiguous()
    off = torch.arange(S + 1, device=cuda, dtype=torch.int64) * nP
    th = torch.tensor(g['theta'], device=cuda, requires_grad=True)
    out = T.transform_grid_ragged(pts, off, th)
    ref_out = T.transform_grid(grid_b, th.detach())
    assert torch.equal(out.reshape(ndim, S, nP).permute(1, 0, 2), ref_out)
    cot = torch.tensor(g['cot'], device=cuda).permute(1, 0, 2).reshape(ndim, S * nP)
    (out * cot).sum().backward()
    ref = g['dtheta_ref_b']
    assert th.grad.shape == ref.shape
    if ref.size:                       # d = 0 for a fully constrained basis
        err = float(np.abs(th.grad.cpu().numpy() - ref).max() / max(np.abs(ref).max(), 1e-30))
        assert err <= 1e-4, err


def test_sorted_by_cell_and_autograd(cuda):
    """transform_grid_ragged (sorted or not) against a loop of transform_grid
    calls: outputs bit-identical, dtheta within 1e-5."""
    rng = np.random.default_rng(9)
    lengths = [int(x) for x in rng.integers(0, 700, size=12)]
    P = _problem(cuda, [3, 3], lengths, seed=5)
    T = P['T']
    T.set_solver_params(nstepsolver=NSTEPS, point_gradient=True)
    gen = torch.Generator(device=cuda).manual_seed(2)
    cot = torch.randn(P['pts'].shape, device=cuda, generator=gen)
    res = {}
    for sort in (False, True):
        th = P['theta'].clone().requires_grad_(True)
        pts = P['pts'].clone().requires_grad_(True)
        out = T.transform_grid_ragged(pts, P['off'], th, sort_by_cell=sort)
        (out * cot).sum().backward()
        res[sort] = (out.detach(), th.grad, pts.grad)
    th = P['theta'].clone().requires_grad_(True)
    pts = P['pts'].clone().requires_grad_(True)
    outs = []
    for s in range(P['S']):
        a, b = int(P['off_h'][s]), int(P['off_h'][s + 1])
        outs.append(T.transform_grid(pts[:, a:b], th[s:s + 1])[0])
    loop = torch.cat(outs, dim=1)
    (loop * cot).sum().backward()
    for sort in (False, True):
        out, gth, gp = res[sort]
        assert torch.equal(out, loop.detach()), sort
        assert _rel(gth, th.grad) <= 1e-5, (sort, _rel(gth, th.grad))
        assert torch.equal(gp, pts.grad), sort


def test_empty_and_invalid_sets(cuda):
    P = _problem(cuda, [2, 2], [0, 0, 0])
    N = P['N']
    out = N.ragged_points_forward(P['nc'], NSTEPS, P['E'], P['off'], P['pts'])
    assert out.shape == (2, 0)
    dth, _ = N.ragged_points_backward(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['pts'],
                                      P['basis'], torch.zeros_like(P['pts']))
    assert torch.all(dth == 0)
    P = _problem(cuda, [2, 2], [40, 30, 50])
    N = P['N']
    gout = torch.ones_like(P['pts'])
    good, _ = N.ragged_points_backward(P['nc'], NSTEPS, 1, P['A'], P['E'], P['off'], P['pts'],
                                       P['basis'], gout)
    assert N.device_status() == 0
    bad = P['off'].clone()
    bad[2] = 10                        # set 1 = [70, 10): negative length
    dth, dp = N.ragged_points_backward(P['nc'], NSTEPS, 1, P['A'], P['E'], bad, P['pts'],
                                       P['basis'], gout, want_dpoints=True)
    assert N.device_status() == 8      # CPAB_DEV_BAD_OFFSETS
    assert torch.all(dth[1] == 0)
    assert _rel(dth[0], good[0]) <= 1e-6
    fwd = N.ragged_points_forward(P['nc'], NSTEPS, P['E'], bad, P['pts'])
    assert N.device_status() == 8
    ref = N.integrate(P['nc'], NSTEPS, P['pts'][:, :40].contiguous(), P['E'][:1].contiguous())
    assert torch.equal(fwd[:, :40], ref[0])


def test_cuda_graph_replay(cuda):
    rng = np.random.default_rng(4)
    lengths = [int(x) for x in rng.integers(1, 2000, size=64)]
    P = _problem(cuda, [4, 4], lengths, seed=8)
    N = P['N']
    gout = torch.randn_like(P['pts'])
    wsf = N.ragged_points_workspace(P['nc'], P['S'], cuda)
    wsb = N.ragged_points_workspace(P['nc'], P['S'], cuda)
    eager_o = N.ragged_points_forward(P['nc'], NSTEPS, P['E'], P['off'], P['pts'], workspace=wsf)
    eager_t, _ = N.ragged_points_backward(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['pts'],
                                          P['basis'], gout, workspace=wsb)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            o = N.ragged_points_forward(P['nc'], NSTEPS, P['E'], P['off'], P['pts'],
                                        workspace=wsf)
            t, _ = N.ragged_points_backward(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'],
                                            P['pts'], P['basis'], gout, workspace=wsb)
    torch.cuda.current_stream().wait_stream(s)
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    assert torch.equal(o, eager_o)
    assert torch.equal(t, eager_t)
    assert N.device_status() == 0

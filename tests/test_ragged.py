"""Ragged batched 1D series (cpab_ragged1d_*): parity on the GPU.

The reference runs each series as its own transform_data call with outsize
[L_s] (libcpab/cpab.py:304-331).  The ragged kernels must give, per series,
what that per-series path gives:

* forward: bit-identical to torch.linspace(0, 1, L_s) on the GPU ->
  cpab_integrate -> interpolation, and to the C oracle's interpolation of that
  grid (the reference's fp32 formula);
* dtheta / dvalues: equal to the per-series fused transform_data backward
  within the summation-order tolerance (1e-5 relative), and to the oracle's
  reference analytic gradient chain within 1e-4 relative;
* the fused MSE launch equals forward + backward with the MSE cotangent, a
  CUDA-graph replay equals the eager call bit for bit, and the autotuner's
  shape gives the same results.
The full cfg3 workload (4,096 series, lengths U{32..4096}, tess [100]) is
checked on a sample of series against the per-series path.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NSTEPS = 50


def _problem(cuda, nc, lengths, seed=0, zb=False):
    from libcpab_gb300 import Cpab, _native as N
    from libcpab_gb300.functions import basis_on
    T = Cpab([nc], backend='pytorch', device='gpu', zero_boundary=zb)
    gen = torch.Generator().manual_seed(seed)
    S = len(lengths)
    theta = torch.randn(S, T.get_theta_dim(), generator=gen)
    off = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    total = int(off[-1])
    vals = []
    for L in lengths:
        x = np.linspace(0, 1, L)
        v = np.zeros(L)
        for _ in range(3):
            f, ph, a = (torch.rand(3, generator=gen).numpy() * [9, 2 * np.pi, 1] + [1, 0, 0.5])
            v += a * np.sin(2 * np.pi * f * x + ph)
        vals.append(v + 0.1 * torch.randn(L, generator=gen).double().numpy())
    values = torch.tensor(np.concatenate(vals) if total else np.zeros(0), dtype=torch.float32)
    target = values.flip(0).contiguous()
    basis = basis_on(T.params, cuda)
    theta = theta.to(cuda)
    A, _, E = N.cell_tables([nc], NSTEPS, theta, basis)
    return dict(T=T, N=N, nc=[nc], S=S, off=torch.tensor(off, device=cuda), off_h=off,
                values=values.to(cuda), target=target.to(cuda), theta=theta, basis=basis, A=A,
                E=E, lengths=list(lengths))


def _per_series_forward(P, s):
    N = P['N']
    a, b = int(P['off_h'][s]), int(P['off_h'][s + 1])
    L = b - a
    dev = P['values'].device
    lin = torch.linspace(0, 1, L, device=dev)
    grid = N.integrate(P['nc'], NSTEPS, lin[None].contiguous(), P['E'][s:s + 1].contiguous())
    out = N.interpolate(P['values'][a:b].reshape(1, 1, L).contiguous(), grid, [L])
    return out.reshape(-1), grid, lin


def _per_series_backward(P, s, mode, gout):
    N = P['N']
    a, b = int(P['off_h'][s]), int(P['off_h'][s + 1])
    L = b - a
    dev = P['values'].device
    lin = torch.linspace(0, 1, L, device=dev)
    data = P['values'][a:b].reshape(1, 1, L).contiguous()
    _, grid = N.transform_data(P['nc'], NSTEPS, lin, [L], P['E'][s:s + 1].contiguous(), data,
                               save_grid=True)
    ddata, dth = N.transform_data_backward(P['nc'], NSTEPS, mode, lin, [L],
                                           P['A'][s:s + 1].contiguous(),
                                           P['E'][s:s + 1].contiguous(), grid, data, P['basis'],
                                           gout[a:b].reshape(1, 1, L).contiguous())
    absum, _ = N.interpolate_backward(data, grid, [L], gout[a:b].abs().reshape(1, 1, L).contiguous(),
                                      want_dgrid=False)
    return dth[0], ddata.reshape(-1), absum.reshape(-1)


def _rel(a, b):
    a, b = a.double().cpu(), b.double().cpu()
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-30))


def _dv_close(a, b, absum, L=None):
    """d(values) is a float-atomic scatter-add (as in the reference's
    autograd), so two correct results differ by the summation order.  Points
    that leave the domain pile up on the edge samples, so an element can take
    up to n = 2 L contributions.  Recursive summation in float32 is within
    (n - 1) u sum|x_i| (u = 2^-24) of the exact sum, so two results are
    within 2 n u absum, absum = the same scatter with |dL/d(out)|.  L = the
    longest series in a (default: all of a is one series)."""
    n = 2 * (a.numel() if L is None else L)
    a, b, absum = a.double().cpu(), b.double().cpu(), absum.double().cpu()
    return bool(((a - b).abs() <= 2 * n * 2.0 ** -24 * absum + 1e-12).all())


LENGTHS = [0, 1, 2, 3, 31, 32, 33, 63, 64, 65, 0, 97, 128, 129, 200, 257, 511, 600, 5, 1000]


# 20 cells: the adjoint sums per lane in workspace slots; 150 cells (above
# 128): the per-step warp flush into the warp's cell table.
@pytest.fixture(scope='module', params=[20, 150])
def small(cuda, request):
    rng = np.random.default_rng(7)
    lengths = LENGTHS + [int(x) for x in rng.integers(1, 400, size=20)]
    return _problem(cuda, request.param, lengths)


def test_ragged_forward_matches_per_series_path(small, oracle):
    P = small
    N = P['N']
    out = N.ragged_forward(P['nc'], NSTEPS, P['E'], P['off'], P['values'])
    for s in range(P['S']):
        a, b = int(P['off_h'][s]), int(P['off_h'][s + 1])
        if b == a:
            continue
        ref, grid, _ = _per_series_forward(P, s)
        assert torch.equal(out[a:b], ref), s
        # the C oracle's interpolation (reference fp32 formula) of the same grid
        o = oracle.interpolate(P['values'][a:b].cpu().numpy().reshape(1, 1, -1),
                               grid.cpu().numpy(), [b - a])
        assert np.array_equal(out[a:b].cpu().numpy(), o.reshape(-1)), s
    assert N.device_status() == 0


@pytest.mark.parametrize('mode', [0, 1, 2])
def test_ragged_backward_matches_per_series_path(small, mode):
    P = small
    N = P['N']
    gen = torch.Generator(device=P['values'].device).manual_seed(3)
    gout = torch.randn(P['values'].shape, device=P['values'].device, generator=gen)
    dth, dv = N.ragged_backward(P['nc'], NSTEPS, mode, P['A'], P['E'], P['off'], P['values'],
                                P['basis'], gout)
    for s in range(P['S']):
        a, b = int(P['off_h'][s]), int(P['off_h'][s + 1])
        if b == a:
            assert torch.all(dth[s] == 0)
            continue
        rth, rdv, absum = _per_series_backward(P, s, mode, gout)
        assert _rel(dth[s], rth) <= 1e-5, (s, _rel(dth[s], rth))
        assert _dv_close(dv[a:b], rdv, absum), s
    assert N.device_status() == 0


def test_ragged_backward_matches_oracle_gradient(small, oracle):
    """Reference analytic gradient chain on the CPU: interpolation backward ->
    midpoint-rule sensitivity (libcpab/core/cpab_ops.cpp:262-372)."""
    P = small
    N = P['N']
    gen = torch.Generator(device=P['values'].device).manual_seed(4)
    gout = torch.randn(P['values'].shape, device=P['values'].device, generator=gen)
    dth, _ = N.ragged_backward(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['values'],
                               P['basis'], gout)
    nC, d = P['A'].shape[1], P['basis'].shape[1]
    Bs = P['basis'].cpu().numpy().T.reshape(d, nC, 1, 2)
    for s in [4, 9, 14, 16, 17, 19]:
        a, b = int(P['off_h'][s]), int(P['off_h'][s + 1])
        L = b - a
        _, grid, lin = _per_series_forward(P, s)
        data = P['values'][a:b].cpu().numpy().reshape(1, 1, L)
        _, dgrid = oracle.interpolate_backward(data, grid.cpu().numpy(), [L],
                                               gout[a:b].cpu().numpy().reshape(1, 1, L))
        ref = oracle.backward(P['nc'], NSTEPS, lin.cpu().numpy()[None], P['A'][s:s + 1].cpu().numpy(),
                              Bs, dgrid)
        assert _rel(dth[s], torch.tensor(ref[0])) <= 1e-4, (s, _rel(dth[s], torch.tensor(ref[0])))


@pytest.mark.parametrize('mode', [0, 1, 2])
def test_ragged_mse_fused_matches_forward_backward(small, mode):
    P = small
    N = P['N']
    total = P['values'].numel()
    scale = 2.0 / total
    res = N.ragged_mse(P['nc'], NSTEPS, mode, P['A'], P['E'], P['off'], P['values'], P['target'],
                       P['basis'], loss_scale=scale, want_out=True)
    out = N.ragged_forward(P['nc'], NSTEPS, P['E'], P['off'], P['values'])
    assert torch.equal(res['out'], out)
    r = out - P['target']
    gout = scale * r
    dth, dv = N.ragged_backward(P['nc'], NSTEPS, mode, P['A'], P['E'], P['off'], P['values'],
                                P['basis'], gout)
    assert torch.equal(res['dtheta'], dth)
    _, absum = N.ragged_backward(P['nc'], NSTEPS, mode, P['A'], P['E'], P['off'], P['values'],
                                 P['basis'], gout.abs())
    assert _dv_close(res['dvalues'], dv, absum, max(P['lengths']))
    sse = torch.stack([(r[int(P['off_h'][s]):int(P['off_h'][s + 1])].double() ** 2).sum()
                       for s in range(P['S'])])
    assert _rel(res['sse'], sse) <= 1e-5


def test_ragged_autograd_and_public_api(small):
    P = small
    T = P['T']
    th = P['theta'].clone().requires_grad_(True)
    v = P['values'].clone().requires_grad_(True)
    out = T.transform_data_ragged(v, P['off'], th)
    loss = ((out - P['target']) ** 2).mean()
    loss.backward()
    res = T.ragged_mse(P['values'], P['target'], P['off'], P['theta'], want_out=True)
    assert _rel(th.grad, res['dtheta']) <= 1e-5
    gabs = (2.0 / P['values'].numel()) * (res['out'] - P['target']).abs()
    _, absum = P['N'].ragged_backward(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['values'],
                                      P['basis'], gabs)
    assert _dv_close(v.grad, res['dvalues'], absum, max(P['lengths']))
    assert abs(float(loss) - float(res['loss'])) <= 1e-5 * abs(float(loss))


def test_ragged_cuda_graph_replay(small):
    """The plan, fused and finalize kernels are captured once and replayed:
    the replay reproduces the eager results bit for bit (deterministic
    reduction), and a replay after changing theta in place follows it."""
    P = small
    N = P['N']
    dev = P['values'].device
    ws = N.ragged_workspace(20, NSTEPS, P['S'], dev)
    theta = P['theta'].clone()
    eager = N.ragged_mse(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['values'], P['target'],
                         P['basis'], workspace=ws)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):     # warm-up on the capture stream
        for _ in range(2):
            A, _, E = N.cell_tables(P['nc'], NSTEPS, theta, P['basis'])
            N.ragged_mse(P['nc'], NSTEPS, 0, A, E, P['off'], P['values'], P['target'],
                         P['basis'], workspace=ws)
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        A, _, E = N.cell_tables(P['nc'], NSTEPS, theta, P['basis'])
        res = N.ragged_mse(P['nc'], NSTEPS, 0, A, E, P['off'], P['values'], P['target'],
                           P['basis'], workspace=ws)
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(res['dtheta'], eager['dtheta'])
        assert torch.equal(res['sse'], eager['sse'])
    theta.mul_(0.5)
    g.replay()
    A2, _, E2 = N.cell_tables(P['nc'], NSTEPS, theta, P['basis'])
    ref = N.ragged_mse(P['nc'], NSTEPS, 0, A2, E2, P['off'], P['values'], P['target'], P['basis'],
                       workspace=ws)
    torch.cuda.synchronize()
    assert torch.equal(res['dtheta'], ref['dtheta'])
    assert N.device_status() == 0


def test_ragged_autotune(cuda):
    P = _problem(cuda, 20, [int(x) for x in np.random.default_rng(1).integers(1, 3000, 64)])
    N = P['N']
    base = N.ragged_mse(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['values'], P['target'],
                        P['basis'], want_out=True)
    for kind in (0, 1):
        shape, ms, res = N.ragged_tune(kind, P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'],
                                       P['values'], P['target'], P['basis'])
        assert shape[0] in (64, 128, 256) and shape[1] in (1, 2, 4) and ms > 0
        assert torch.equal(res['out'], base['out'])
        if kind == 1:
            assert _rel(res['dtheta'], base['dtheta']) <= 1e-5
    # later calls use the tuned shapes and still agree
    again = N.ragged_mse(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['values'], P['target'],
                         P['basis'], want_out=True)
    assert torch.equal(again['out'], base['out'])
    assert _rel(again['dtheta'], base['dtheta']) <= 1e-5
    assert torch.equal(N.ragged_forward(P['nc'], NSTEPS, P['E'], P['off'], P['values']),
                       base['out'])


def test_ragged_every_launch_shape(cuda):
    """Every candidate launch shape of the ragged kernels pinned in turn (the
    tuner's force argument): forward output bit-identical to the default
    shape's; the adjoint's out bit-identical, the squared errors and dtheta
    within 1e-5 (other block sizes and passes per tile change only the order
    of the sums; d(values), a float-atomic scatter like the reference's, is
    checked against its summation bound elsewhere)."""
    P = _problem(cuda, 20, [int(x) for x in np.random.default_rng(2).integers(1, 2500, 48)])
    N = P['N']
    base = N.ragged_mse(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['values'], P['target'],
                        P['basis'], want_out=True)
    for kind in (0, 1):
        for b in (64, 128, 256):
            for ppt in (1, 2, 4):
                shape, ms, res = N.ragged_tune(kind, P['nc'], NSTEPS, 0, P['A'], P['E'],
                                               P['off'], P['values'], P['target'], P['basis'],
                                               force=(b, ppt))
                assert tuple(shape) == (b, ppt) and ms == 0.0
                assert torch.equal(res['out'], base['out']), (kind, b, ppt)
                if kind == 1:
                    assert _rel(res['sse'], base['sse']) <= 1e-5, (b, ppt)
                    assert _rel(res['dtheta'], base['dtheta']) <= 1e-5, (b, ppt)
    with pytest.raises(N.CpabError):
        N.ragged_tune(1, P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['values'],
                      P['target'], P['basis'], force=(96, 1))
    assert N.device_status() == 0


def test_ragged_empty_and_invalid_series(cuda):
    from libcpab_gb300 import _native as N
    P = _problem(cuda, 10, [0, 0, 0])
    res = N.ragged_mse(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['values'], P['target'],
                       P['basis'])
    assert torch.all(res['dtheta'] == 0) and torch.all(res['sse'] == 0)
    # a decreasing offset makes series 1 invalid: it is skipped and flagged,
    # the other series are unaffected
    P = _problem(cuda, 10, [40, 30, 50])
    good = N.ragged_mse(P['nc'], NSTEPS, 1, P['A'], P['E'], P['off'], P['values'], P['target'],
                        P['basis'], want_dvalues=False)
    assert N.device_status() == 0
    bad_off = P['off'].clone()
    bad_off[2] = 10                    # series 1 = [70, 10): negative length
    res = N.ragged_mse(P['nc'], NSTEPS, 1, P['A'], P['E'], bad_off, P['values'], P['target'],
                       P['basis'], want_dvalues=False)
    assert N.device_status() == 8      # CPAB_DEV_BAD_OFFSETS
    assert torch.all(res['dtheta'][1] == 0)
    assert _rel(res['dtheta'][0], good['dtheta'][0]) <= 1e-6


def test_ragged_full_size_workload(cuda):
    """4,096 series, lengths U{32..4096}, tess [100] (zero_boundary False),
    theta ~ N(0, I): the one-launch results agree with the per-series path on a
    sample of series."""
    rng = np.random.default_rng(0)
    lengths = [int(x) for x in rng.integers(32, 4097, size=4096)]
    P = _problem(cuda, 100, lengths, seed=1)
    N = P['N']
    total = P['values'].numel()
    res = N.ragged_mse(P['nc'], NSTEPS, 0, P['A'], P['E'], P['off'], P['values'], P['target'],
                       P['basis'], want_out=True)
    gout = (2.0 / total) * (res['out'] - P['target'])
    for s in rng.choice(4096, size=24, replace=False):
        a, b = int(P['off_h'][s]), int(P['off_h'][s + 1])
        ref, _, _ = _per_series_forward(P, int(s))
        assert torch.equal(res['out'][a:b], ref), s
        rth, rdv, absum = _per_series_backward(P, int(s), 0, gout)
        assert _rel(res['dtheta'][s], rth) <= 1e-5, s
        assert _dv_close(res['dvalues'][a:b], rdv, absum), s
    assert N.device_status() == 0

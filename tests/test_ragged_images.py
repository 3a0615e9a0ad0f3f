"""Images of mixed sizes (transform_data_mixed, cpab_interpolate_ragged*).

The reference warps a batch of images of different sizes with one
transform_data call per image (libcpab/cpab.py:304-331): its interpolator
takes one data size and one outsize per call (libcpab/pytorch/interpolation.py:
39-40).  The mixed path integrates every image's grid in one ragged launch and
samples every image in one more, and must give, per image, what the per-image
call gives:

* forward: bit-identical to transform_data on the image alone (the same
  integration arithmetic and the same sampling helpers);
* dtheta: equal to the per-image gradient within the summation-order
  tolerance (1e-4 relative, as for the fused vs unfused chain);
* d(image): equal within 1e-5 relative (float atomics in both);
* a plan row that does not fit its buffers is skipped and flagged
  (CPAB_DEV_BAD_OFFSETS), never read past.

The CPU tests cover the host plan (cpab_ragged_images_plan: no CUDA call) and
the argument checks.
"""
import numpy as np
import pytest
import torch

NSTEPS = 50


def _cpab(nc, zb=True, gradient='reference'):
    from libcpab_gb300 import Cpab
    T = Cpab(list(nc), backend='pytorch', device='gpu', zero_boundary=zb)
    T.set_solver_params(nstepsolver=NSTEPS, gradient=gradient)
    return T


def _rel(a, b):
    a, b = a.double().cpu(), b.double().cpu()
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-30))


def _images(cuda, C, sizes, seed=1):
    gen = torch.Generator().manual_seed(seed)
    return [torch.rand(C, *s, generator=gen).to(cuda) for s in sizes]


def _check_mixed(T, cuda, C, sizes, outsize, scale=0.5, seed=0, ddata_tol=1e-5):
    gen = torch.Generator().manual_seed(seed)
    S = len(sizes)
    theta = (torch.randn(S, T.get_theta_dim(), generator=gen) * scale).to(cuda)
    ims = _images(cuda, C, sizes, seed + 1)
    t1 = theta.clone().requires_grad_(True)
    d1 = [im.clone().requires_grad_(True) for im in ims]
    outs = T.transform_data_mixed(d1, t1, outsize)
    assert len(outs) == S
    from libcpab_gb300.functions import _mixed_outsizes
    osz = _mixed_outsizes(len(sizes[0]), sizes, outsize)
    ws = [torch.randn(o.shape, generator=gen).to(cuda) for o in outs]
    sum((o * w).sum() for o, w in zip(outs, ws)).backward()
    for s in range(S):
        t2 = theta[s:s + 1].clone().requires_grad_(True)
        d2 = ims[s][None].clone().requires_grad_(True)
        ref = T.transform_data(d2, t2, list(osz[s]))
        assert outs[s].shape == ref.shape[1:]
        assert torch.equal(outs[s], ref[0]), 'image %d' % s
        (ref[0] * ws[s]).sum().backward()
        assert _rel(t1.grad[s], t2.grad[0]) <= 1e-4, 'dtheta of image %d' % s
        assert _rel(d1[s].grad, d2.grad[0]) <= ddata_tol, 'd(image) of image %d' % s


# ------------------------------------------------------------------- GPU ---
@pytest.mark.gpu
@pytest.mark.parametrize('gradient', ['reference', 'exact'])
@pytest.mark.parametrize('outsize', [None, (20, 30), 'each'])
def test_mixed_2d_matches_per_image(gradient, outsize, cuda):
    from libcpab_gb300 import _native as N
    sizes = [(17, 23), (32, 32), (1, 5), (40, 9), (64, 48)]
    if outsize == 'each':
        outsize = [(9, 40), (32, 32), (3, 3), (1, 1), (70, 33)]
    T = _cpab([3, 3], gradient=gradient)
    N.device_status()
    _check_mixed(T, cuda, 3, sizes, outsize)
    assert N.device_status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize('C', [1, 2])
def test_mixed_3d_matches_per_image(C, cuda):
    from libcpab_gb300 import _native as N
    T = _cpab([2, 2, 2])
    N.device_status()
    _check_mixed(T, cuda, C, [(9, 10, 11), (16, 8, 12), (1, 1, 1)],
                 [(9, 10, 11), (12, 9, 40), (2, 3, 4)])
    assert N.device_status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize('zb,ddata_tol', [(True, 1e-5), (False, 1e-3)])
def test_mixed_1d_matches_per_image(zb, ddata_tol, cuda):
    """Without the zero boundary and with theta ~ N(0, I), most points of the
    257-point series leave the domain and clamp to the edge pixel, where the
    reference's weights (1 - xd, xd) reach about -164 and 165 (xd is taken
    after the clamp) and cancel: ~400 float atomics of such terms into one
    pixel differ with their order by ~1e-4 of the largest gradient, so d(image)
    gets 1e-3 there (forward and dtheta keep their gates)."""
    from libcpab_gb300 import _native as N
    T = _cpab([10], zb=zb)
    N.device_status()
    _check_mixed(T, cuda, 2, [(50,), (300,), (1,), (257,)], None, scale=1.0,
                 ddata_tol=ddata_tol)
    assert N.device_status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize('nc,sizes,outsizes', [
    ([3, 3], [(17, 23), (64, 48), (1, 5)], [(9, 40), (64, 48), (3, 3)]),
    ([2, 2, 2], [(9, 10, 11), (16, 8, 12)], [(9, 10, 11), (12, 9, 40)]),
])
def test_mixed_sampling_matches_c_oracle(nc, sizes, outsizes, cuda, oracle):
    """Each image's output is the C oracle's interpolation (the reference's
    fp32 formula, libcpab/pytorch/interpolation.py:18-172) of that image at
    its warped grid, bit for bit."""
    from libcpab_gb300 import _native as N
    from libcpab_gb300.functions import basis_on, image_layout
    T = _cpab(nc)
    gen = torch.Generator().manual_seed(6)
    theta = (torch.randn(len(sizes), T.get_theta_dim(), generator=gen) * 0.5).to(cuda)
    ims = _images(cuda, 2, sizes, 7)
    outs = T.transform_data_mixed(ims, theta, outsizes)
    lay = image_layout(T.params, sizes, outsizes, cuda)
    _, _, E = N.cell_tables(nc, NSTEPS, theta, basis_on(T.params, cuda))
    grid = N.ragged_points_forward(nc, NSTEPS, E, lay.offsets, lay.points).cpu().numpy()
    off = lay.offsets.cpu().numpy()
    for s, (im, osz) in enumerate(zip(ims, outsizes)):
        g = grid[:, off[s]:off[s + 1]][None]
        ref = oracle.interpolate(im[None].cpu().numpy(), g, list(osz))
        assert np.array_equal(outs[s].cpu().numpy(), ref[0]), 'image %d' % s
    assert N.device_status() == 0


@pytest.mark.gpu
def test_packed_matches_mixed(cuda):
    """transform_data_packed on the concatenated images gives the
    concatenated outputs of transform_data_mixed, and the same gradients."""
    T = _cpab([3, 3])
    sizes = [(17, 23), (32, 32), (1, 5)]
    outsizes = [(9, 40), (32, 32), (3, 3)]
    ims = _images(cuda, 3, sizes, 9)
    gen = torch.Generator().manual_seed(10)
    theta = (torch.randn(3, T.get_theta_dim(), generator=gen) * 0.5).to(cuda)
    t1 = theta.clone().requires_grad_(True)
    d1 = [im.clone().requires_grad_(True) for im in ims]
    outs = T.transform_data_mixed(d1, t1, outsizes)
    flat = torch.cat([o.reshape(-1) for o in outs])
    w = torch.randn(flat.shape, generator=gen).to(cuda)
    (flat * w).sum().backward()
    t2 = theta.clone().requires_grad_(True)
    p2 = torch.cat([im.reshape(-1) for im in ims]).requires_grad_(True)
    packed = T.transform_data_packed(p2, sizes, t2, outsizes)
    assert torch.equal(packed, flat.detach())
    (packed * w).sum().backward()
    assert torch.equal(t1.grad, t2.grad)
    assert _rel(torch.cat([d.grad.reshape(-1) for d in d1]), p2.grad) <= 1e-5


@pytest.mark.gpu
def test_mixed_layout_is_cached_and_theta_only(cuda):
    """Repeated calls with the same sizes reuse the device plan; theta without
    grad and images without grad run forward only."""
    T = _cpab([3, 3])
    ims = _images(cuda, 1, [(8, 8), (16, 4)])
    theta = torch.zeros(2, T.get_theta_dim(), device=cuda)
    a = T.transform_data_mixed(ims, theta)
    lay = next(iter(T.params._layout_cache.values()))
    b = T.transform_data_mixed(ims, theta)
    assert next(iter(T.params._layout_cache.values())) is lay
    for x, y, im in zip(a, b, ims):
        assert torch.equal(x, y)
        # the identity transformation samples every pixel at itself
        assert (x - im).abs().max() <= 1e-5


@pytest.mark.gpu
def test_mixed_cuda_graph_replay(cuda):
    """Forward + backward of transform_data_mixed captured in a CUDA graph
    (after an eager call has cached the layout): the replay reproduces the
    eager outputs and dtheta bit for bit, and d(images) to float-atomic order."""
    from libcpab_gb300 import _native as N
    T = _cpab([3, 3])
    sizes = [(17, 23), (32, 32), (40, 9)]
    ims = _images(cuda, 2, sizes)
    gen = torch.Generator().manual_seed(4)
    theta = (torch.randn(3, T.get_theta_dim(), generator=gen) * 0.5).to(cuda)
    ws = [torch.randn(2, *sz, generator=gen).to(cuda) for sz in sizes]

    def step():
        th = theta.detach().requires_grad_(True)
        dd = [im.detach().requires_grad_(True) for im in ims]
        outs = T.transform_data_mixed(dd, th)
        torch.autograd.backward(outs, ws)
        return [o.detach() for o in outs], th.grad, [d.grad for d in dd]

    e_out, e_dth, e_dd = step()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        step()
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        g_out, g_dth, g_dd = step()
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    for x, y in zip(g_out, e_out):
        assert torch.equal(x, y)
    assert torch.equal(g_dth, e_dth)
    for x, y in zip(g_dd, e_dd):
        assert _rel(x, y) <= 1e-5
    assert N.device_status() == 0


@pytest.mark.gpu
def test_bad_plan_rows_are_flagged_not_read(cuda):
    from libcpab_gb300 import _native as N
    plan, totals = N.ragged_images_plan(2, [(4, 4), (4, 4)])
    bad = plan.copy()
    bad[1, 1] = 15   # image 0 would own 15 points, image 1 17: neither fits 4 x 4
    data = torch.rand(2 * 16, device=cuda)
    grid = torch.rand(2, 32, device=cuda)
    N.device_status()
    out = N.interpolate_ragged(2, torch.from_numpy(bad).to(cuda), totals, data, grid, 1)
    assert out.numel() == 32
    assert N.device_status() == 8       # CPAB_DEV_BAD_OFFSETS
    ok = N.interpolate_ragged(2, torch.from_numpy(plan).to(cuda), totals, data, grid, 1)
    torch.cuda.synchronize()
    assert N.device_status() == 0
    assert torch.isfinite(ok).all()


# ------------------------------------------------------------------- CPU ---
def _plan_restated(ndim, sizes, outsizes):
    rows, d, p, t = [], 0, 0, 0
    for sz, osz in zip(sizes, outsizes):
        ext = lambda v: list(v) + [1] * (3 - ndim)
        if ndim == 1:
            tiles = -(-osz[0] // 256)
        else:
            tiles = -(-osz[0] // 8) * -(-osz[-1] // 32) * (osz[1] if ndim == 3 else 1)
        rows.append([d, p, t] + ext(sz) + ext(osz) + [0])
        d += int(np.prod(sz))
        p += int(np.prod(osz))
        t += tiles
    rows.append([d, p, t] + [0] * 7)
    return np.array(rows, dtype=np.int64), (d, p, t)


@pytest.mark.parametrize('ndim,sizes,outsizes', [
    (2, [(17, 23), (32, 32), (1, 5)], None),
    (2, [(17, 23), (224, 224)], [(9, 40), (224, 225)]),
    (3, [(9, 10, 11), (16, 8, 12)], [(9, 10, 11), (12, 9, 40)]),
    (1, [(50,), (300,), (1,), (256,), (257,)], None),
    (2, [], None),
])
def test_plan_matches_restatement(ndim, sizes, outsizes):
    from libcpab_gb300 import _native as N
    plan, totals = N.ragged_images_plan(ndim, sizes, outsizes)
    ref, rtot = _plan_restated(ndim, sizes, outsizes if outsizes is not None else sizes)
    assert np.array_equal(plan, ref)
    assert totals == rtot


def test_plan_rejects_bad_sizes():
    from libcpab_gb300 import _native as N
    with pytest.raises(N.CpabError, match='image 1'):
        N.ragged_images_plan(2, [(4, 4), (0, 4)])
    with pytest.raises(N.CpabError, match='2\\^31'):
        N.ragged_images_plan(2, [(40000, 40000), (40000, 40000)])
    with pytest.raises(ValueError):
        N.ragged_images_plan(2, [(4, 4, 4)])
    with pytest.raises(ValueError):
        N.ragged_images_plan(2, [(4, 4)], [(4, 4), (4, 4)])


def test_mixed_outsizes_forms():
    from libcpab_gb300.functions import _mixed_outsizes
    sizes = [(3, 4), (5, 6)]
    assert _mixed_outsizes(2, sizes, None) == sizes
    assert _mixed_outsizes(2, sizes, (7, 8)) == [(7, 8), (7, 8)]
    assert _mixed_outsizes(2, sizes, [[1, 2], (3, 4)]) == [(1, 2), (3, 4)]
    with pytest.raises(ValueError):
        _mixed_outsizes(2, sizes, [(1, 2)])
    with pytest.raises(ValueError):
        _mixed_outsizes(2, sizes, [(1, 2, 3), (3, 4)])


def test_mixed_argument_checks():
    from libcpab_gb300 import functions as F
    from libcpab_gb300.cpab import Cpab
    T = Cpab([3, 3], backend='pytorch', device='gpu', zero_boundary=True)
    theta = torch.zeros(2, T.get_theta_dim())
    with pytest.raises(ValueError, match='theta'):
        F.transform_data_mixed([torch.zeros(1, 4, 4)], theta, T.params)
    assert F.transform_data_mixed([], torch.zeros(0, T.get_theta_dim()), T.params) == []
    with pytest.raises(ValueError, match='CUDA'):
        F.transform_data_mixed([torch.zeros(1, 4, 4)] * 2, theta, T.params)
    with pytest.raises(ValueError, match='same C'):
        F.transform_data_mixed([torch.zeros(1, 4, 4), torch.zeros(2, 4, 4)], theta, T.params)
    with pytest.raises(ValueError, match='fewer than'):
        F.transform_data_mixed([torch.zeros(1, 4, 4)] * 2, theta, T.params, (2048, 2048))
    T.params.integration = 'exact'
    with pytest.raises(ValueError, match='fixed-step'):
        F.transform_data_mixed([torch.zeros(1, 4, 4)] * 2, theta, T.params)


def test_packed_argument_checks():
    from libcpab_gb300 import functions as F
    from libcpab_gb300.cpab import Cpab
    T = Cpab([3, 3], backend='pytorch', device='gpu', zero_boundary=True)
    theta = torch.zeros(2, T.get_theta_dim())
    with pytest.raises(ValueError, match='theta'):
        F.transform_data_packed(torch.zeros(32), [(4, 4)], theta, T.params)
    with pytest.raises(ValueError, match='2 extents'):
        F.transform_data_packed(torch.zeros(32), [(4, 4), (4,)], theta, T.params)
    with pytest.raises(ValueError, match='1D'):
        F.transform_data_packed(torch.zeros(2, 16), [(4, 4), (4, 4)], theta, T.params)
    with pytest.raises(ValueError, match='pixels'):
        F.transform_data_packed(torch.zeros(33), [(4, 4), (4, 4)], theta, T.params)
    with pytest.raises(ValueError, match='CUDA'):
        F.transform_data_packed(torch.zeros(64), [(4, 4), (4, 4)], theta, T.params)
    assert F.transform_data_packed(torch.zeros(0), [], torch.zeros(0, T.get_theta_dim()),
                                   T.params).numel() == 0

"""Host-staged transform_data (host_io.HostUpload, transform_data_from_host):
the chunked copy overlapped with the forward must not change any result bit."""
import pytest
import torch


def test_chunk_bounds():
    from libcpab_gb300.host_io import chunk_bounds
    assert chunk_bounds(10, 4) == [(0, 3), (3, 6), (6, 8), (8, 10)]
    assert chunk_bounds(3, 8) == [(0, 1), (1, 2), (2, 3)]
    assert chunk_bounds(5, 1) == [(0, 5)]
    assert chunk_bounds(0, 4) == [(0, 0)]
    for n in range(1, 40):
        for c in range(1, 9):
            b = chunk_bounds(n, c)
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(x[1] == y[0] for x, y in zip(b, b[1:]))
            assert max(x[1] - x[0] for x in b) - min(x[1] - x[0] for x in b) <= 1


def test_from_host_refuses_device_data():
    from libcpab_gb300 import Cpab
    T = Cpab([2, 2], backend='pytorch', device='gpu')
    with pytest.raises(ValueError):                 # theta must be on the GPU
        T.backend.transform_data_from_host(torch.zeros(2, 1, 8, 8), torch.zeros(2, 4),
                                           T.params, [8, 8])


@pytest.mark.gpu
@pytest.mark.parametrize('gradient', ['reference', 'exact'])
def test_from_host_matches_device_path(cuda, gradient):
    import torch.nn.functional as F
    from libcpab_gb300 import Cpab
    from libcpab_gb300.host_io import HostUpload
    T = Cpab([3, 3], backend='pytorch', device='gpu', zero_boundary=True)
    T.set_solver_params(gradient=gradient)
    g = torch.Generator().manual_seed(0)
    nb = 10
    theta_h = 0.5 * torch.randn(nb, T.get_theta_dim(), generator=g)
    data_h = torch.rand(nb, 3, 64, 48, generator=g).pin_memory()
    target_h = torch.rand(nb, 3, 64, 48, generator=g).pin_memory()
    th1 = theta_h.to(cuda).requires_grad_(True)
    out1, dd1 = T.transform_data_from_host(data_h, th1, [64, 48], requires_grad=True)
    F.mse_loss(out1, HostUpload(target_h, cuda).wait()).backward()
    th2 = theta_h.to(cuda).requires_grad_(True)
    dd2 = data_h.to(cuda).requires_grad_(True)
    out2 = T.transform_data(dd2, th2, [64, 48])
    F.mse_loss(out2, target_h.to(cuda)).backward()
    assert torch.equal(dd1.detach(), dd2.detach())
    assert torch.equal(out1, out2)
    assert torch.equal(th1.grad, th2.grad)
    # d(data) is a float-atomic scatter (summation order varies between runs)
    err = (dd1.grad - dd2.grad).abs().max() / dd2.grad.abs().max()
    assert float(err) <= 1e-5, float(err)


@pytest.mark.gpu
@pytest.mark.parametrize('nc,size,outsize', [([3, 3], [40, 30], [40, 30]),
                                             ([2, 4], [31, 17], [20, 45]),
                                             ([6], [50], [77]),
                                             ([2, 2, 2], [9, 10, 11], [8, 12, 7])])
def test_split_forward_is_bit_identical(cuda, nc, size, outsize):
    """cpab_transform_grid_image + cpab_sample_grid == cpab_transform_data."""
    from libcpab_gb300 import Cpab, _native as N
    from libcpab_gb300.functions import basis_on
    T = Cpab(nc, backend='pytorch', device='gpu', zero_boundary=True)
    g = torch.Generator().manual_seed(1)
    nb = 3
    theta = torch.randn(nb, T.get_theta_dim(), generator=g).to(cuda)
    data = torch.rand(nb, 2, *size, generator=g).to(cuda)
    A, _, E = N.cell_tables(nc, 50, theta, basis_on(T.params, cuda))
    lin = torch.cat([torch.linspace(0, 1, o, device=cuda) for o in outsize]).contiguous()
    out, grid = N.transform_data(nc, 50, lin, outsize, E, data, save_grid=True)
    grid2 = N.transform_grid_image(nc, 50, lin, outsize, E)
    out2 = N.sample_grid(data, grid2, outsize)
    assert torch.equal(grid, grid2)
    assert torch.equal(out, out2)

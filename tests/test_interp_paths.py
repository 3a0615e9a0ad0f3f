"""Bilinear and trilinear sampling through each forward kernel, against the C
oracle.

cpab_interpolate in 2D and 3D stages the grid tile with the tensor memory
accelerator (k_interpolate_tma) when the grid is 16-byte aligned, W_out is a
multiple of 4 and C <= 4 (2D) or C <= 3 (3D), and otherwise uses the tiled
kernel (k_interpolate_tiled).  Both must give the C restatement of
libcpab/pytorch/interpolation.py bit for bit: partial tiles at the x and last
-axis edges (the accelerator's zero fill), blocks that take several images
(both mbarrier phases in 3D), one to five channels, coordinates outside
[0, 1], huge ones and NaN.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

# (nb, C, size, outsize); comment: the kernel taken
CASES = [
    (4, 3, [30, 41], [64, 48]),           # 2D accelerator, partial last-axis tile
    (3, 1, [17, 9], [36, 70]),            # 2D accelerator, partial tiles on both axes
    (5, 2, [64, 64], [32, 32]),           # 2D accelerator, one tile, images shared by blocks
    (2, 4, [12, 13], [40, 33]),           # 2D accelerator, four channels
    (2, 5, [12, 13], [40, 33]),           # 2D tiled kernel: five channels
    (3, 3, [20, 21], [42, 50]),           # 2D tiled kernel: W_out not a multiple of 4
    (3, 1, [20, 17, 24], [40, 36, 44]),   # 3D accelerator, partial x and z tiles
    (2, 2, [9, 33, 16], [36, 5, 70]),     # 3D accelerator, two channels
    (5, 3, [12, 6, 40], [64, 3, 32]),     # 3D accelerator, three channels, 2 images per block
    (9, 1, [16, 16, 16], [32, 2, 32]),    # 3D accelerator, three images per block
    (1, 1, [128, 1, 3], [4, 1, 4]),       # 3D accelerator, image smaller than the box
    (2, 4, [10, 11, 12], [40, 6, 36]),    # 3D tiled kernel: four channels
    (2, 5, [10, 11, 12], [40, 6, 36]),    # 3D tiled kernel: any channel count
    (3, 1, [14, 9, 30], [30, 7, 33]),     # 3D tiled kernel: W_out not a multiple of 4
]


def _grid(nb, outsize, seed):
    rng = np.random.default_rng(seed)
    g = rng.uniform(-0.2, 1.2, size=(nb, len(outsize), int(np.prod(outsize)))).astype(np.float32)
    flat = g.reshape(-1)
    idx = rng.choice(flat.size, size=min(64, flat.size), replace=False)
    # NaN and huge finite coordinates (clamped to the edges); not +-inf, whose
    # conversion to an integer index is undefined in the C oracle
    flat[idx[:16]] = np.nan
    flat[idx[16:32]] = 3e9
    flat[idx[32:48]] = -3e9
    flat[idx[48:]] = rng.choice([1 - 2 ** -24, 0.0, 1.0, 1.0 + 2 ** -23], size=idx[48:].size)
    return g


@pytest.mark.parametrize('nb,C,size,outsize', CASES)
def test_interpolate_matches_oracle(nb, C, size, outsize, cuda, oracle):
    from libcpab_gb300 import _native as N
    rng = np.random.default_rng(nb * 100 + C)
    data = rng.standard_normal((nb, C, *size)).astype(np.float32)
    grid = _grid(nb, outsize, nb + C)
    ref = oracle.interpolate(data, grid, outsize)
    out = N.interpolate(torch.tensor(data, device=cuda), torch.tensor(grid, device=cuda),
                        outsize).cpu().numpy()
    assert np.array_equal(out, ref, equal_nan=True)
    assert N.device_status() == 0


@pytest.mark.parametrize('nb,C,size,outsize', [(2, 3, [30, 41], [64, 48]),
                                               (2, 1, [20, 17, 24], [40, 36, 44])])
def test_interpolate_unaligned_grid(nb, C, size, outsize, cuda, oracle):
    """A grid that starts 4 bytes past a 16-byte boundary takes the tiled
    kernel and gives the same values."""
    from libcpab_gb300 import _native as N
    rng = np.random.default_rng(7)
    data = rng.standard_normal((nb, C, *size)).astype(np.float32)
    grid = _grid(nb, outsize, 8)
    buf = torch.empty(grid.size + 1, device=cuda)
    buf[1:] = torch.tensor(grid.reshape(-1), device=cuda)
    g_dev = buf[1:].view(grid.shape)
    assert g_dev.data_ptr() % 16 != 0
    out = N.interpolate(torch.tensor(data, device=cuda), g_dev, outsize).cpu().numpy()
    assert np.array_equal(out, oracle.interpolate(data, grid, outsize), equal_nan=True)
    aligned = N.interpolate(torch.tensor(data, device=cuda), torch.tensor(grid, device=cuda),
                            outsize).cpu().numpy()
    assert np.array_equal(out, aligned, equal_nan=True)
    assert N.device_status() == 0

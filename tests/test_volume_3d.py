"""3D volume warp at full size: tess [4,4,4] with zero boundary and volume
preservation (d = 20, the reference's basis from tests/golden), 8 theta ~
N(0, I), volumes [8, 1, 128, 128, 128] = sums of 32 isotropic Gaussian blobs
(centres uniform in the volume, sigma ~ U[2, 8] voxels, amplitude ~ U[0.5, 1]);
trilinear transform_data forward and dtheta / d(data) backward
(16.8 M trajectories).

* fused forward == meshgrid -> cpab_integrate -> cpab_interpolate, bit for bit;
* fused backward vs the unfused chain (interpolation adjoint -> cpab_backward):
  dtheta relative error <= 1e-4 (summation order), d(data) within the float
  atomic-order bound;
* on sampled trajectories: GPU cells/points vs the FP64 oracle (C++ cell
  rules) with boundary ties classified, trilinear values bit-identical to the
  C oracle's, and reference-mode dtheta vs the reference's analytic gradient
  (C oracle) within 1e-4.
"""
import numpy as np
import pytest
import torch

from conftest import load_golden

pytestmark = pytest.mark.gpu

NSTEPS = 50
NC = [4, 4, 4]
SIZE = 128
TIE_MARGIN = 1e-6


@pytest.fixture(scope='module')
def volume(cuda):
    from libcpab_gb300 import _native as N
    B = load_golden('L_3d_4x4x4_zb_vp')['B']
    basis = torch.tensor(np.ascontiguousarray(B), dtype=torch.float32, device=cuda)
    theta = torch.randn(8, B.shape[1], generator=torch.Generator().manual_seed(0)).to(cuda)
    from bench import make_volumes
    data = make_volumes(cuda)
    A, _, E = N.cell_tables(NC, NSTEPS, theta, basis)
    lin = torch.cat([torch.linspace(0, 1, SIZE, device=cuda)] * 3).contiguous()
    from libcpab_gb300.functions import uniform_meshgrid
    mesh = uniform_meshgrid(3, [0, 0, 0], [1, 1, 1], [SIZE] * 3, cuda).contiguous()
    return dict(N=N, B=B, basis=basis, theta=theta, data=data, A=A, E=E, lin=lin, mesh=mesh)


def _dv_close(a, b, absum, n):
    # float-atomic scatter-add, at most n terms per element: |a - b| <= 2 n u absum
    a, b, absum = a.double(), b.double(), absum.double()
    return bool(((a - b).abs() <= 2 * n * 2.0 ** -24 * absum + 1e-12).all())


def test_volume_fused_forward_matches_unfused(volume):
    V = volume
    N = V['N']
    out, _ = N.transform_data(NC, NSTEPS, V['lin'], [SIZE] * 3, V['E'], V['data'])
    grid = N.integrate(NC, NSTEPS, V['mesh'], V['E'])
    ref = N.interpolate(V['data'], grid, [SIZE] * 3)
    assert torch.equal(out, ref)
    assert torch.isfinite(out).all()
    assert N.device_status() == 0


@pytest.mark.parametrize('mode', [0, 1, 2])
def test_volume_fused_backward_matches_unfused(volume, mode):
    V = volume
    N = V['N']
    osz = [SIZE] * 3
    out, gsave = N.transform_data(NC, NSTEPS, V['lin'], osz, V['E'], V['data'], save_grid=True)
    w = torch.randn(out.shape, device=out.device, generator=torch.Generator(out.device).manual_seed(2))
    ddata, dth = N.transform_data_backward(NC, NSTEPS, mode, V['lin'], osz, V['A'], V['E'], gsave,
                                           V['data'], V['basis'], w)
    grid = N.integrate(NC, NSTEPS, V['mesh'], V['E'])
    ddata_u, dgrid = N.interpolate_backward(V['data'], grid, osz, w)
    dth_u, _ = N.backward(NC, NSTEPS, mode, V['mesh'], V['A'], V['E'], V['basis'], dgrid)
    rel = float((dth - dth_u).abs().max() / dth_u.abs().max())
    assert rel <= 1e-4, rel
    absum, _ = N.interpolate_backward(V['data'], grid, osz, w.abs(), want_dgrid=False)
    # zero boundary keeps the points inside and the field is volume preserving,
    # so a voxel collects the corner weights of a few output points: n <= 64
    assert _dv_close(ddata, ddata_u, absum, 64)
    assert N.device_status() == 0


def test_volume_sampled_trajectories_vs_oracle(volume, oracle):
    from oracle.oracle import numpy_transform_grid
    V = volume
    N = V['N']
    rng = np.random.default_rng(4)
    idx = np.sort(rng.choice(SIZE ** 3, size=4096, replace=False))
    pts = np.ascontiguousarray(V['mesh'].cpu().numpy()[:, idx])
    th = V['theta'][:2].contiguous()
    theta = th.cpu().numpy()
    P = torch.tensor(pts, device=V['data'].device)
    out, cells = N.integrate_trace(NC, NSTEPS, P, V['E'][:2].contiguous())
    out, cells = out.cpu().numpy(), cells.cpu().numpy()
    ref, cells64, marg = numpy_transform_grid(V['B'], theta, pts, NC, NSTEPS, return_cells=True,
                                              return_margin='steps', semantics='cpp')
    diff = cells != cells64
    tie = diff.any(axis=2)
    err = np.abs(out - ref).max(axis=1)
    assert (~tie).any()
    assert err[~tie].max() <= 1e-5, err[~tie].max()
    first = diff.argmax(axis=2)
    ti, pi = np.nonzero(tie)
    if ti.size:
        assert marg[ti, pi, first[ti, pi]].max() < TIE_MARGIN
    assert tie.sum() <= 0.02 * tie.size
    # trilinear values of these points, bit-identical to the C oracle
    n = pts.shape[1]
    data = V['data'][:2].contiguous()
    vals = N.interpolate(data, torch.tensor(out, device=data.device), [n, 1, 1])
    vref = oracle.interpolate(data.cpu().numpy(), out, [n, 1, 1])
    assert np.array_equal(vals.cpu().numpy(), vref)
    # reference-mode dtheta of a loss on these points vs the reference's analytic gradient
    cot = rng.standard_normal(out.shape).astype(np.float32)
    d0, _ = N.backward(NC, NSTEPS, 0, P, V['A'][:2].contiguous(), V['E'][:2].contiguous(),
                       V['basis'], torch.tensor(cot, device=P.device))
    Bs = V['B'].T.reshape(V['B'].shape[1], -1, 3, 4).astype(np.float32)
    ref0 = oracle.backward(NC, NSTEPS, pts, V['A'][:2].cpu().numpy(), Bs, cot)
    rel = float(np.abs(d0.cpu().numpy() - ref0).max() / np.abs(ref0).max())
    assert rel <= 1e-4, rel

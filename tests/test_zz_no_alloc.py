"""cpab_backward_noalloc: the gradient entry point for callers that cannot
allocate device memory (their runtime owns the device memory, or allocation is
not allowed where they run), so they cannot pass cpab_backward a workspace.

It keeps its scratch in a fixed array inside the library.  These tests call it
through the C ABI and check it against cpab_backward (same inputs, workspace
allocated here) within the gradient tolerance used elsewhere (1e-5 relative:
only the number of CTAs per theta, and so the summation order, differs), on
two calls in a row, and check that oversized problems are refused.  The file
runs last so that a failure here does not hide the other tests' results; it
also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import load_golden

pytestmark = pytest.mark.gpu

NSTEPS = 50


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _inputs(cuda, name='2d_3x3_zb', mode=0):
    from libcpab_gb300 import _native as N
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    theta = torch.tensor(g['theta'], device=cuda)
    basis = torch.tensor(np.ascontiguousarray(g['B']), dtype=torch.float32, device=cuda)
    A, _, E = N.cell_tables(nc, NSTEPS, theta, basis)
    pts = torch.tensor(g['grid_b'], device=cuda)
    cot = torch.tensor(g['cot'], device=cuda)
    return N, nc, pts, A, E, basis, cot


def _noalloc(N, nc, mode, pts, A, E, basis, cot, want_dpoints=True):
    """pts: [n_theta, ndim, nP] (one point set per theta) or [ndim, nP]
    (shared by all theta); dpoints come back [n_theta, ndim, nP] either way."""
    ndim = len(nc)
    n_theta, d = A.shape[0], basis.shape[1]
    broadcast = int(pts.dim() == 3)
    nP = pts.shape[-1]
    dtheta = torch.full((n_theta, d), float('nan'), device=pts.device)
    dpoints = torch.full((n_theta, ndim, nP), float('nan'), device=pts.device) \
        if want_dpoints else None
    rc = N.load().cpab_backward_noalloc(
        ndim, N._ints(nc), NSTEPS, mode, _ptr(pts), broadcast, nP, _ptr(A), _ptr(E), n_theta,
        _ptr(basis), d, _ptr(cot), _ptr(dtheta), _ptr(dpoints), None,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, dtheta, dpoints


def _rel(a, b):
    a, b = a.double().cpu(), b.double().cpu()
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-30))


@pytest.mark.parametrize('mode', [0, 1, 2])
def test_noalloc_matches_workspace_backward_twice(mode, cuda):
    N, nc, pts, A, E, basis, cot = _inputs(cuda)
    ref_dth, ref_dpts = N.backward(nc, NSTEPS, mode, pts, A, E, basis, cot, want_dpoints=True)
    for _ in range(2):          # the shared scratch keeps the previous call's values
        rc, dth, dpts = _noalloc(N, nc, mode, pts, A, E, basis, cot)
        assert rc == 0, N.load().cpab_last_error()
        torch.cuda.synchronize()
        assert _rel(dth, ref_dth) <= 1e-5
        assert torch.equal(dpts, ref_dpts)      # per-point adjoint: same arithmetic
    assert N.device_status() == 0


def test_noalloc_3d_and_large_batch(cuda):
    """A 3D case, and a batch large enough that the CTA count is capped by the
    fixed scratch."""
    N, nc, pts, A, E, basis, cot = _inputs(cuda, '3d_2x2x2_zb_vp')
    ref_dth, _ = N.backward(nc, NSTEPS, 0, pts, A, E, basis, cot)
    rc, dth, _ = _noalloc(N, nc, 0, pts, A, E, basis, cot, want_dpoints=False)
    assert rc == 0, N.load().cpab_last_error()
    assert _rel(dth, ref_dth) <= 1e-5
    # 2D [8,8]: 1536 floats per theta; 1024 theta -> at most 1 CTA slice fits
    from libcpab_gb300.tessellation import make_tessellation
    B = make_tessellation([8, 8], False, False).B
    basis = torch.tensor(np.ascontiguousarray(B), dtype=torch.float32, device=cuda)
    gen = torch.Generator(device=cuda).manual_seed(0)
    theta = torch.randn(1024, B.shape[1], device=cuda, generator=gen)
    A, _, E = N.cell_tables([8, 8], NSTEPS, theta, basis)
    pts = torch.rand(1024, 2, 3000, device=cuda, generator=gen)
    cot = torch.randn(1024, 2, 3000, device=cuda, generator=gen)
    ref_dth, _ = N.backward([8, 8], NSTEPS, 0, pts, A, E, basis, cot)
    for _ in range(2):
        rc, dth, _ = _noalloc(N, [8, 8], 0, pts, A, E, basis, cot, want_dpoints=False)
        assert rc == 0, N.load().cpab_last_error()
        assert _rel(dth, ref_dth) <= 1e-5


@pytest.mark.parametrize('mode', [0, 1, 2])
def test_noalloc_capped_blocks_shared_points(mode, cuda):
    """Points shared by all theta ([ndim, nP]), dpoints wanted, on a problem
    where the fixed scratch holds one CTA slice per theta while cpab_backward
    plans more: 1D with 4,096 cells (8,192 floats per theta), 200 theta.  The
    tables come from a random basis (the kernels do not need a CPAB basis)."""
    from libcpab_gb300 import _native as N
    nc, n_theta, nP, d = [4096], 200, 3000, 6
    gen = torch.Generator(device=cuda).manual_seed(5)
    basis = 0.3 * torch.randn(4096 * 2, d, device=cuda, generator=gen)
    theta = torch.randn(n_theta, d, device=cuda, generator=gen)
    A, _, E = N.cell_tables(nc, NSTEPS, theta, basis)
    pts = torch.rand(1, nP, device=cuda, generator=gen)
    cot = torch.randn(n_theta, 1, nP, device=cuda, generator=gen)
    slice_bytes = n_theta * 4096 * 2 * 4
    assert (1 << 21) * 4 < 2 * slice_bytes                # one slice per theta fits
    ws = N.load().cpab_backward_workspace(1, N._ints(nc), NSTEPS, nP, n_theta)
    assert ws >= 2 * slice_bytes                          # cpab_backward: >= 2 CTAs per theta
    ref_dth, ref_dp = N.backward(nc, NSTEPS, mode, pts, A, E, basis, cot, want_dpoints=True)
    for _ in range(2):
        rc, dth, dp = _noalloc(N, nc, mode, pts, A, E, basis, cot)
        assert rc == 0, N.load().cpab_last_error()
        torch.cuda.synchronize()
        assert torch.equal(dp, ref_dp)
        assert _rel(dth, ref_dth) <= 1e-5
    assert N.device_status() == 0


@pytest.mark.parametrize('mode', [0, 1, 2])
def test_3d_global_warp_tables_match_shared(mode, cuda):
    """3D [4,4,4] (320 cells): cpab_backward keeps its per-warp gradient tables
    in the workspace (more warps per SM); the no-alloc entry point keeps them
    in shared memory.  Same dpoints bit for bit, dtheta to summation order."""
    from libcpab_gb300 import _native as N
    from libcpab_gb300.tessellation import make_tessellation
    g = load_golden('L_3d_4x4x4_zb_vp')
    B = np.ascontiguousarray(g['B'])
    basis = torch.tensor(B, dtype=torch.float32, device=cuda)
    gen = torch.Generator(device=cuda).manual_seed(3)
    theta = torch.randn(8, B.shape[1], device=cuda, generator=gen)
    A, _, E = N.cell_tables([4, 4, 4], NSTEPS, theta, basis)
    pts = torch.rand(8, 3, 20000, device=cuda, generator=gen)
    cot = torch.randn(8, 3, 20000, device=cuda, generator=gen)
    ws_glob = N.load().cpab_backward_workspace(3, N._ints([4, 4, 4]), NSTEPS, 20000, 8)
    assert ws_glob > 8 * 320 * 12 * 4 * 4        # partials plus per-warp tables
    ref_dth, ref_dp = N.backward([4, 4, 4], NSTEPS, mode, pts, A, E, basis, cot, want_dpoints=True)
    rc, dth, dp = _noalloc(N, [4, 4, 4], mode, pts, A, E, basis, cot)
    assert rc == 0, N.load().cpab_last_error()
    assert torch.equal(dp, ref_dp)
    assert _rel(dth, ref_dth) <= 1e-5
    assert N.device_status() == 0


def test_noalloc_rejects_oversized_problem(cuda):
    """n_theta * nC * ndim*(ndim+1) above the fixed scratch is refused with a
    clear error, before any work is enqueued."""
    from libcpab_gb300 import _native as N
    nc = [8, 8]                               # 256 cells * 6 = 1536 floats per theta
    n_theta = (1 << 21) // 1536 + 1
    lib = N.load()
    dummy = torch.zeros(16, device=cuda)
    rc = lib.cpab_backward_noalloc(2, N._ints(nc), NSTEPS, 0, _ptr(dummy), 0, 4, _ptr(dummy),
                                   None, n_theta, _ptr(dummy), 10, _ptr(dummy), _ptr(dummy),
                                   None, None, None)
    assert rc == 4                            # CPAB_ERR_WORKSPACE
    assert b'no-alloc scratch' in lib.cpab_last_error()
    assert N.device_status() == 0

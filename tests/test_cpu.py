"""CPU tests (no GPU): the oracle against the reference's golden vectors, the
tessellation/basis against the reference, the C-ABI library's exports, the
host-side API guards, and the multi-rank timing reduction (gloo)."""
import hashlib
import os
import platform
import re

import numpy as np
import pytest

from conftest import REPO, SMALL, load_golden

NSTEPS = 50


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def rel(a, b):
    b = np.asarray(b, dtype=np.float64)
    if b.size == 0:
        return 0.0
    return float(np.abs(np.asarray(a, dtype=np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


# ----------------------------------------------------------------- basis --
@pytest.mark.parametrize('name', SMALL)
def test_tessellation_matches_reference(name):
    from libcpab_gb300.tessellation import make_tessellation
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    t = make_tessellation(nc, bool(g['zero_boundary']), bool(g['volume_perservation']))
    assert tuple(t.L.shape) == tuple(g['L_shape'])
    assert sha(t.L) == str(g['L_sha']), 'constraint matrix differs from the reference'
    if platform.machine() == 'x86_64':
        assert np.array_equal(t.B, g['B']), 'basis differs from the reference'
    else:   # another LAPACK build may pick another orthonormal basis of the same space
        P1 = t.B @ t.B.T
        P2 = g['B'] @ g['B'].T
        assert np.abs(P1 - P2).max() < 1e-9


@pytest.mark.parametrize('name', ['L_2d_8x8_free', 'L_3d_4x4x4_zb_vp'])
def test_large_constraint_matrix_matches_reference(name):
    from libcpab_gb300.tessellation import make_tessellation
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    t = make_tessellation(nc, bool(g['zero_boundary']), bool(g['volume_perservation']),
                          basis=False)
    assert tuple(t.L.shape) == tuple(g['L_shape'])
    assert sha(t.L) == str(g['L_sha'])


def test_basis_cache_roundtrip(tmp_path):
    """The pickle cache uses libcpab's file names and content."""
    from libcpab_gb300.tessellation import make_tessellation, basis_file_name
    t1 = make_tessellation([2, 3], True, False, direc=str(tmp_path))
    f = tmp_path / (basis_file_name([2, 3], True, False) + '.pkl')
    assert f.exists() and f.name == 'cpab_basis_dim2_tess2_3_vo0_zb1_vp0.pkl'
    t2 = make_tessellation([2, 3], True, False, direc=str(tmp_path))
    assert np.array_equal(t1.B, t2.B)


# ---------------------------------------------------------------- oracle --
@pytest.mark.parametrize('name', SMALL)
def test_oracle_cell_lookup_matches_reference(name, oracle):
    from oracle.oracle import numpy_findcellidx
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    assert np.array_equal(oracle.findcellidx(nc, g['probe']), g['cells_cpp'])
    assert np.array_equal(numpy_findcellidx(len(nc), g['probe'], nc), g['cells_np'])


@pytest.mark.parametrize('nc', [[50], [3, 3], [8, 8], [2, 2, 2], [4, 4, 4], [3, 5, 2]])
def test_fp64_cpp_lookup_matches_oracle_except_ties(nc, oracle):
    """The FP64 lookup with the C++ rules (used to follow trajectories in
    double) gives the C oracle's cell for float inputs, except at points whose
    decision margin marks them as ties."""
    from oracle.oracle import numpy_findcellidx
    rng = np.random.default_rng(11)
    P = rng.uniform(-0.5, 1.5, (len(nc), 300000)).astype(np.float32)
    P[:, :100000] = rng.uniform(0, 1, (len(nc), 100000))
    got, margin = numpy_findcellidx(len(nc), P, nc, semantics='cpp', return_margin=True)
    ref = oracle.findcellidx(nc, P)
    bad = got != ref
    assert np.all(margin[bad] < 1e-6), margin[bad].max()
    assert bad.mean() < 1e-3


@pytest.mark.parametrize('name', SMALL)
def test_oracle_forward_matches_reference(name, oracle):
    """C restatement fed the reference's step maps: bit-identical to the
    reference's pytorch-CPU (C++) output; numpy FP64 restatement: identical
    to the reference's numpy backend."""
    from oracle.oracle import numpy_transform_grid
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    assert np.array_equal(oracle.forward(nc, NSTEPS, g['grid'], g['trels_ref']), g['out_cpu32'])
    assert np.abs(numpy_transform_grid(g['B'], g['theta'], g['grid'], nc, NSTEPS)
                  - g['out_np64']).max() <= 1e-12
    assert np.abs(numpy_transform_grid(g['B'], g['theta'], g['grid_b'], nc, NSTEPS)
                  - g['out_np64_b']).max() <= 1e-12


@pytest.mark.parametrize('name', SMALL)
def test_oracle_gradient_matches_reference(name, oracle):
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    As = g['As_ref']
    Bs = g['B'].T.reshape(g['B'].shape[1], *As.shape[1:])
    dth = oracle.backward(nc, NSTEPS, g['grid'], As, Bs, g['cot'])
    assert rel(dth, g['dtheta_ref']) <= 1e-5   # reference sums in fp32, the oracle in fp64
    dthb = oracle.backward(nc, NSTEPS, g['grid_b'], As, Bs, g['cot'])
    assert rel(dthb, g['dtheta_ref_b']) <= 1e-5


@pytest.mark.parametrize('name', SMALL)
def test_oracle_interpolation_matches_reference(name, oracle):
    g = load_golden(name)
    npts = [int(x) for x in g['npts']]
    assert np.array_equal(oracle.interpolate(g['data'], g['out_cpu32'], npts), g['interp32'])
    dd, dg = oracle.interpolate_backward(g['data'], g['out_cpu32'], npts, g['icot'])
    assert rel(dd, g['interp64_ddata']) <= 1e-5
    assert rel(dg, g['interp64_dgrid']) <= 1e-5


@pytest.mark.parametrize('name', ['1d_50_zb', '2d_3x3_zb', '3d_2x2x2_zb_vp'])
def test_fp64_autograd_matches_finite_differences(name):
    """The exact-gradient oracle: central differences of the FP64 forward with
    the cell sequence frozen agree with its autograd."""
    from oracle.oracle import fp64_autograd, numpy_transform_grid
    g = load_golden(name)
    nc = [int(x) for x in g['nc']]
    B, th = g['B'], g['theta'][:1].astype(np.float64)
    pts = g['grid'][:, :64]
    cot = g['cot'][:1, :, :64]
    _, cells = numpy_transform_grid(B, th, pts, nc, NSTEPS, return_cells=True)
    _, dth, _ = fp64_autograd(B, th, pts, nc, cot, NSTEPS, cells=cells)
    h = 1e-6
    for k in range(min(4, th.shape[1])):
        e = np.zeros_like(th)
        e[0, k] = h
        fp = fp64_autograd(B, th + e, pts, nc, cot, NSTEPS, cells=cells)[0]
        fm = fp64_autograd(B, th - e, pts, nc, cot, NSTEPS, cells=cells)[0]
        fd = ((fp - fm) * cot).sum() / (2 * h)
        assert abs(fd - dth[0, k]) <= 1e-6 * max(1.0, abs(fd))


def test_reference_library_matches_golden():
    """The reference's own cpab_ops.cpp, compiled here, regenerates the
    golden fp32 outputs (only where the reference checkout exists)."""
    from oracle.oracle import RefLib
    try:
        ref = RefLib()
    except FileNotFoundError:
        pytest.skip('reference checkout not present')
    for name in SMALL:
        g = load_golden(name)
        nc = [int(x) for x in g['nc']]
        assert np.array_equal(ref.forward(nc, NSTEPS, g['grid'], g['trels_ref']), g['out_cpu32'])
        assert np.array_equal(ref.findcellidx(nc, g['probe']), g['cells_cpp'])


# ----------------------------------------------------------------- C ABI --
def header_functions():
    src = open(os.path.join(REPO, 'include', 'cpab_gb300.h')).read()
    return sorted(set(re.findall(r'CPAB_API\s+[\w\s\*]*?\b(cpab_\w+)\s*\(', src)))


def test_library_exports_every_declared_symbol():
    import ctypes
    from libcpab_gb300 import _native
    names = header_functions()
    assert len(names) >= 15
    assert sorted(_native.EXPORTED) == names
    lib = ctypes.CDLL(_native.LIB_PATH)
    for n in names:
        assert hasattr(lib, n), n


def test_capi_argument_errors_without_gpu():
    """Argument validation runs before any device work."""
    import ctypes
    from libcpab_gb300 import _native as N
    lib = N.load()
    assert lib.cpab_num_cells(2, N._ints([3, 3])) == 36
    assert lib.cpab_num_cells(3, N._ints([4, 4, 4])) == 320
    assert lib.cpab_num_cells(4, N._ints([1, 1, 1, 1])) == -1
    assert b'ndim' in lib.cpab_last_error()
    rc = lib.cpab_integrate(2, N._ints([3, 3]), 0, None, 0, 10, None, 1, None, None, None)
    assert rc == 1 and b'nsteps' in lib.cpab_last_error()
    rc = lib.cpab_backward(2, N._ints([3, 3]), 50, 7, None, 0, 10, None, None, 1, None, 34,
                           None, None, None, None, 0, None, None)
    assert rc == 1 and b'mode' in lib.cpab_last_error()
    rc = lib.cpab_ragged1d_forward(0, 50, None, 1, None, 10, None, None, None, 0, None, None)
    assert rc == 1 and b'nc' in lib.cpab_last_error()
    rc = lib.cpab_ragged1d_mse(10, 50, 0, None, None, -1, None, 0, None, 10, None, None, 1.0,
                               None, None, None, None, None, 0, None, None)
    assert rc == 1 and b'S >= 0' in lib.cpab_last_error()
    rc = lib.cpab_ragged1d_backward(10, 50, 5, None, None, 1, ctypes.c_void_p(16), 10, None, 10,
                                    None, None, None, None, None, 0, None, None)
    assert rc == 1 and b'mode' in lib.cpab_last_error()
    rc = lib.cpab_ragged1d_mse(10, 50, 0, None, None, 4, None, 0, None, 10, None, None, 1.0,
                               None, None, None, None, None, 0, None, None)
    assert rc == 1 and b'offsets' in lib.cpab_last_error()


# -------------------------------------------------------------- host API --
def test_cpab_rejects_other_backends_and_cpu():
    from libcpab_gb300 import Cpab
    with pytest.raises(NotImplementedError):
        Cpab([2, 2], backend='numpy', device='cpu')
    with pytest.raises(NotImplementedError):
        Cpab([2, 2], backend='pytorch', device='cpu')
    with pytest.raises(AssertionError):
        Cpab([2, 2, 2, 2], backend='pytorch', device='gpu')


def test_transformer_refuses_cpu_tensors():
    import torch
    from libcpab_gb300 import Cpab, functions
    T = Cpab([2, 2], backend='pytorch', device='gpu')
    with pytest.raises(ValueError):
        functions.transformer(torch.zeros(2, 5), torch.zeros(1, T.get_theta_dim()), T.params)


def test_params_fields_match_reference():
    from libcpab_gb300 import Cpab
    T = Cpab([3, 3], backend='pytorch', device='gpu')
    p = T.get_params()
    for f in ('nc', 'ndim', 'nC', 'Ashape', 'basis', 'nstepsolver', 'use_slow', 'numeric_grad',
              'D', 'd', 'params_pr_cell', 'zero_boundary', 'volume_perservation',
              'domain_min', 'domain_max', 'inc', 'valid_outside', 'constrain_mat'):
        assert hasattr(p, f), f
    assert (p.nC, p.d, p.D) == (36, 34, 216)
    T.set_solver_params(nstepsolver=20, gradient='exact')
    assert p.nstepsolver == 20 and p.gradient == 'exact'


# ------------------------------------------------------ multi-rank (gloo) --
def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench
    q.put((rank, bench.reduce_max([1.0 + rank, 5.0 - rank], 'cpu')))
    dist.destroy_process_group()


def test_rank_time_reduction_gloo():
    """bench.py aggregates per-rank times with a MAX all-reduce."""
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(60)
    res = dict(q.get(timeout=5) for _ in range(2))
    assert res[0] == res[1] == [2.0, 5.0]


def _shard_main(rank, world, port, q):
    """One rank of a theta-sharded step: this rank's theta rows of the golden
    2D [3,3] problem through the oracle's reference forward and analytic
    gradient, then the shards gathered over gloo."""
    import torch
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    from oracle.oracle import Oracle
    out, dth = _shard_step(Oracle(), rank, world)
    outs = [torch.zeros_like(out) for _ in range(world)]
    dths = [torch.zeros_like(dth) for _ in range(world)]
    dist.all_gather(outs, out)
    dist.all_gather(dths, dth)
    if rank == 0:
        q.put((torch.cat(outs).numpy(), torch.cat(dths).numpy()))
    dist.destroy_process_group()


def _shard_step(orc, rank, world):
    """Rows rank*n/world .. (rank+1)*n/world of theta (contiguous shards of
    equal size): forward with the reference step maps and the reference's
    analytic gradient for a fixed cotangent."""
    import torch
    g = load_golden('2d_3x3_zb')
    n = g['theta'].shape[0]
    assert n % world == 0
    lo, hi = rank * n // world, (rank + 1) * n // world
    nc = [int(x) for x in g['nc']]
    out = orc.forward(nc, 50, g['grid'], g['trels_ref'][lo:hi])
    d = g['B'].shape[1]
    Bs = np.asarray(g['B']).T.reshape(d, -1, 2, 3).astype(np.float32)
    dth = orc.backward(nc, 50, g['grid'], g['As_ref'][lo:hi], Bs, g['cot'][lo:hi])
    return torch.tensor(np.asarray(out)), torch.tensor(np.asarray(dth))


def test_theta_sharded_step_gloo(oracle):
    """The path shards by theta with no data-path exchange: two gloo ranks,
    each integrating and differentiating its half of the theta rows, gather
    exactly the single-process results (every trajectory and its gradient
    depend on their own theta only)."""
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    ps = [ctx.Process(target=_shard_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out2, dth2 = q.get(timeout=120)
    for p in ps:
        p.join(60)
    out1, dth1 = _shard_step(oracle, 0, 1)
    assert np.array_equal(out2, out1.numpy())
    assert np.array_equal(dth2, dth1.numpy())

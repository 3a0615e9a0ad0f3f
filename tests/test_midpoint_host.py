"""The reference-mode trajectory of the adjoint kernels, compiled for the host.

The reference's gradient (libcpab/core/cpab_ops.cpp:262-372) differentiates
its midpoint-rule trajectory: v = A[p;1] in float, pMid = p + h v / 2 and
p += h vMid with h a double, each rounded to float.  The kernels evaluate the
double updates in FP32 (cpab_midpoint.cuh: add_mul_f64).  Checked here on the
CPU:
  * add_mul_f64 against numpy's double evaluation on random and adversarial
    operands: equal except in rare double-rounding cases (<= 1e-6 of them);
  * whole trajectories (ref_mid_step with the FP64 lookup replica) against the
    oracle's C restatement of the reference recurrence: cell sequences and end
    points bit-identical for all but a handful of trajectories.
Runs on the CPU; needs nvcc.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO, load_golden

NVCC = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'


@pytest.fixture(scope='module')
def harness(tmp_path_factory):
    if not os.path.exists(NVCC):
        pytest.skip('nvcc not available')
    out = str(tmp_path_factory.mktemp('midpoint') / 'midpoint_check')
    subprocess.check_call([NVCC, '-O2', '-std=c++17', '-Xcompiler', '-ffp-contract=off', '-o',
                           out, os.path.join(REPO, 'tests', 'midpoint_check.cu')])
    return out


def split(H):
    hi = np.float32(H)
    lo = np.float32(H - np.float64(hi))
    return hi, lo


def run_ops(harness, tmp_path, H, p, v):
    hi, lo = split(H)
    fin, fout = str(tmp_path / 'ops.bin'), str(tmp_path / 'ops_out.bin')
    with open(fin, 'wb') as f:
        f.write(np.array([hi, lo], dtype=np.float32).tobytes())
        f.write(np.int64(p.size).tobytes())
        f.write(np.ascontiguousarray(p, dtype=np.float32).tobytes())
        f.write(np.ascontiguousarray(v, dtype=np.float32).tobytes())
    subprocess.check_call([harness, 'ops', fin, fout])
    return np.fromfile(fout, dtype=np.float32)


@pytest.mark.parametrize('nsteps', [50, 37, 100])
def test_add_mul_f64_matches_double(harness, tmp_path, nsteps):
    rng = np.random.default_rng(nsteps)
    n = 2_000_000
    p = np.concatenate([rng.uniform(-0.2, 1.2, n // 2),
                        rng.standard_normal(n // 4) * 10.0 ** rng.integers(-8, 2, n // 4),
                        rng.uniform(0, 1, n // 4) * 2.0 ** -rng.integers(0, 30, n // 4)])
    v = np.concatenate([rng.standard_normal(n // 2) * 3.0,
                        rng.standard_normal(n // 4) * 10.0 ** rng.integers(-9, 3, n // 4),
                        -p[3 * n // 4:] * rng.uniform(0, 60, n // 4)])
    p, v = p.astype(np.float32), v.astype(np.float32)
    for H in (1.0 / nsteps, 0.5 / nsteps):
        got = run_ops(harness, tmp_path, H, p, v)
        want = (p.astype(np.float64) + H * v.astype(np.float64)).astype(np.float32)
        bad = np.count_nonzero(got != want)
        assert bad <= 1e-6 * n, '%d of %d updates differ from the double evaluation' % (bad, n)
        # a difference is one float step at most
        if bad:
            k = got != want
            assert np.all(np.abs(got[k] - want[k]) <= np.spacing(np.abs(want[k])))


def run_traj(harness, tmp_path, nc, nsteps, A, pts):
    ndim = len(nc)
    hdr = np.array([ndim] + list(nc) + [1] * (3 - ndim) + [nsteps], dtype=np.int32)
    fin, fout = str(tmp_path / 'traj.bin'), str(tmp_path / 'traj_out.bin')
    with open(fin, 'wb') as f:
        f.write(hdr.tobytes())
        f.write(np.int64(pts.shape[1]).tobytes())
        f.write(np.ascontiguousarray(A, dtype=np.float32).tobytes())
        f.write(np.ascontiguousarray(pts, dtype=np.float32).tobytes())
    subprocess.check_call([harness, 'traj', fin, fout])
    r = np.fromfile(fout, dtype=np.uint8)
    nP = pts.shape[1]
    end = r[:ndim * nP * 4].view(np.float32).reshape(ndim, nP)
    cells = r[ndim * nP * 4:].view(np.int32).reshape(nP, nsteps)
    return end, cells


def cases():
    """(name, nc, basis B, theta scale, points): the golden tessellations plus
    the strongly expanding [8,8] fields and the free 1D [100] tessellation."""
    from libcpab_gb300.tessellation import make_tessellation
    out = []
    for name in ('1d_50_zb', '2d_3x3_zb', '2d_4x4_free', '3d_2x2x2_free', '3d_2x2x2_zb_vp'):
        g = load_golden(name)
        out.append((name, [int(x) for x in g['nc']], g['B'], 1.0, None))
    out.append(('1d_100_free', [100], make_tessellation([100], False, False).B, 1.0, None))
    out.append(('2d_8x8_free_large', [8, 8], make_tessellation([8, 8], False, False).B, 3.0,
                None))
    return out


@pytest.mark.parametrize('case', cases(), ids=lambda c: c[0])
def test_trajectory_matches_reference_recurrence(harness, tmp_path, oracle, case):
    name, nc, B, scale, _ = case
    ndim = len(nc)
    rng = np.random.default_rng(11)
    nP = 20000
    pts = rng.uniform(-0.1, 1.1, (ndim, nP)).astype(np.float32)
    pts[:, : nP // 2] = rng.uniform(0, 1, (ndim, nP // 2))
    bad_cells = bad_end = 0
    for k in range(3):
        theta = (scale * rng.standard_normal(B.shape[1])).astype(np.float32)
        A = (B @ theta.astype(np.float64)).astype(np.float32)
        end, cells = run_traj(harness, tmp_path, nc, 50, A, pts)
        end_o, cells_o = oracle.midpoint_trajectory(nc, 50, pts, A.reshape(-1, ndim, ndim + 1))
        same = (cells == cells_o).all(axis=1)
        bad_cells += int((~same).sum())
        bad_end += int((end[:, same] != end_o[:, same]).any(axis=0).sum())
    # each trajectory makes 100 * ndim double updates; rare double-rounding
    # differences (add_mul_f64) may move a trajectory by an ulp
    assert bad_cells <= 3 and bad_end <= 5, (bad_cells, bad_end)

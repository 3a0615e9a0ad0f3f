"""The FP32 cell lookup of the kernels, compiled for the host and checked on
adversarial points: wherever the FP32 path answers, it must equal the FP64
replica, and the FP64 replica must equal the C oracle (itself bit-identical to
the reference's cpab_ops.cpp, see test_cpu.py).  Runs on the CPU; needs nvcc.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO

NVCC = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'


@pytest.fixture(scope='module')
def harness(tmp_path_factory):
    if not os.path.exists(NVCC):
        pytest.skip('nvcc not available')
    out = str(tmp_path_factory.mktemp('lookup') / 'lookup_check')
    subprocess.check_call([NVCC, '-O2', '-std=c++17', '-o', out,
                           os.path.join(REPO, 'tests', 'lookup_check.cu')])
    return out


def run(harness, tmp_path, nc, P):
    P = np.ascontiguousarray(P, dtype=np.float32)
    ndim, n = P.shape
    hdr = np.array([ndim] + list(nc) + [1] * (3 - len(nc)), dtype=np.int32)
    fin, fout = str(tmp_path / 'in.bin'), str(tmp_path / 'out.bin')
    with open(fin, 'wb') as f:
        f.write(hdr.tobytes())
        f.write(np.int64(n).tobytes())
        f.write(P.tobytes())
    subprocess.check_call([harness, fin, fout])
    r = np.fromfile(fout, dtype=np.int32)
    return r[:n], r[n:]


def adversarial(nc, rng, n=400000):
    """Faces (exact float multiples of the reference's float inc and of k/nc,
    +-1..3 ulp), sub-cell diagonals/planes, corners, and out-of-domain points."""
    ndim = len(nc)
    P = rng.uniform(-0.2, 1.2, (ndim, n)).astype(np.float32)
    m = n // 6
    for j in range(ndim):
        inc32 = np.float32(1.0 / nc[j])
        k = rng.integers(0, nc[j] + 1, m)
        base = np.where(rng.random(m) < 0.5, (k * inc32).astype(np.float32),
                        (k / nc[j]).astype(np.float32))
        steps = rng.integers(-3, 4, m)
        v = base.copy()
        for s in range(1, 4):
            v = np.where(steps >= s, np.nextafter(v, np.float32(3)), v)
            v = np.where(steps <= -s, np.nextafter(v, np.float32(-3)), v)
        P[j, j * m:(j + 1) * m] = v
    # points on the square diagonals / tet planes: x-frac == y-frac, x+y == 1, ...
    i0 = ndim * m
    t = rng.random(m).astype(np.float64)
    cx = rng.integers(0, nc[0], m)
    cy = rng.integers(0, nc[1] if ndim > 1 else 1, m)
    P[0, i0:i0 + m] = ((cx + t) / nc[0]).astype(np.float32)
    if ndim > 1:
        sel = rng.random(m) < 0.5
        fy = np.where(sel, t, 1 - t)
        P[1, i0:i0 + m] = ((cy + fy) / nc[1]).astype(np.float32)
    if ndim > 2:
        P[2, i0:i0 + m] = ((rng.integers(0, nc[2], m) + np.where(sel, t, 1 - t)) / nc[2]).astype(np.float32)
    # zero-boundary style points hugging the domain faces
    i1 = i0 + m
    P[:, i1:i1 + m] = rng.random((ndim, m)).astype(np.float32)
    face = rng.integers(0, ndim, m)
    val = rng.choice(np.array([0.0, -0.0, 1e-30, 1e-12, -1e-12, 1.0, np.nextafter(np.float32(1), np.float32(0))],
                              dtype=np.float32), m)
    P[face, i1 + np.arange(m)] = val
    # far outside, huge and non-finite coordinates
    i2 = i1 + m
    P[:, i2:i2 + m] = rng.uniform(-6, 7, (ndim, m)).astype(np.float32)
    spec = np.array([np.nan, np.inf, -np.inf, 1e10, -1e10, 3e38, 1e-38], dtype=np.float32)
    k = i2 + rng.choice(m, m // 20, replace=False)
    P[rng.integers(0, ndim, k.size), k] = rng.choice(spec, k.size)
    # out-of-domain diagonal rules: |py/iy| == |px/ix| corners, to the ulp
    if ndim == 2:
        i3 = i2 + m // 2
        s = rng.uniform(0.01, 2, m // 2)
        sx = rng.choice([-1, 1], m // 2)
        sy = rng.choice([-1, 1], m // 2)
        P[0, i3:i2 + m] = np.where(sx < 0, -s / nc[0], 1 + s / nc[0]).astype(np.float32)
        P[1, i3:i2 + m] = np.where(sy < 0, -s / nc[1], 1 + s / nc[1]).astype(np.float32)
    return P


@pytest.mark.parametrize('nc', [[50], [100], [3, 3], [8, 8], [4, 4], [7, 5], [2, 3],
                                [2, 2, 2], [4, 4, 4], [3, 5, 2]])
def test_fp32_lookup_agrees_with_fp64_replica_and_oracle(nc, harness, tmp_path, oracle):
    rng = np.random.default_rng(sum(nc) * 7919 + len(nc))
    P = adversarial(nc, rng)
    fast, exact = run(harness, tmp_path, nc, P)
    ref = oracle.findcellidx(nc, P)
    if len(nc) == 1:
        # floor(p*nc) of a huge or non-finite p has no defined int value in C;
        # the kernels saturate like CUDA's conversion (see cell_1d)
        ok = np.abs(P[0]) < 1e6
        sat = np.where(np.isnan(P[0]) | (P[0] < 0), 0, nc[0] - 1)
        assert np.array_equal(exact[~ok], sat[~ok])
        exact, ref, fast, P = exact[ok], ref[ok], fast[ok], P[:, ok]
    assert np.array_equal(exact, ref), 'FP64 replica differs from the oracle'
    answered = fast >= 0
    bad = np.nonzero(answered & (fast != exact))[0]
    assert bad.size == 0, 'FP32 lookup wrong at %s' % P[:, bad[:5]].T
    # on random in-domain points the FP64 path is (almost) never needed
    U = rng.random((len(nc), 200000)).astype(np.float32)
    f2, _ = run(harness, tmp_path, nc, U)
    assert (f2 < 0).mean() < 1e-4
    if len(nc) == 3:
        # points a few ulp outside the x or y face (zero-boundary trajectories
        # drift there by rounding): the push-inside rule runs in FP32 as well.
        # (Points outside in all three coordinates are pushed onto a domain
        # corner, where every tetrahedron plane meets: those stay FP64 ties.)
        n3 = 200000
        O = rng.random((3, n3)).astype(np.float32)
        face = rng.integers(0, 2, n3)
        drift = rng.choice(np.array([-1e-7, -1e-9, -0.0, 1.0000001, 1.00001, 1.0 + 2 ** -20],
                                    dtype=np.float32), n3)
        O[face, np.arange(n3)] = drift
        f3, e3 = run(harness, tmp_path, nc, O)
        assert np.array_equal(f3[f3 >= 0], e3[f3 >= 0])
        assert (f3 < 0).mean() < 1e-3


@pytest.mark.parametrize('nc', [[3, 3], [8, 8], [4, 4], [7, 5], [5, 5], [6, 6], [16, 16]])
def test_second_tier_ties_2d(nc, harness, tmp_path):
    """2D points on or within a few ulp of the triangle diagonals, and the
    zero-boundary domain corners with the ~1e-17 drift their trajectories
    have: wherever the FP32 tiers answer they equal the FP64 replica, and for
    square cells they answer the corner points (fixed points of the flow, a
    tie at every step) without the replica."""
    rng = np.random.default_rng(sum(nc) * 31 + 5)
    inc = np.float32(1.0) / np.float32(nc[0])
    m = 40000
    # main diagonal px == py and anti-diagonal px + py == inc of square (0, 0),
    # exact and +-1..2 ulp
    a = rng.uniform(0, float(inc), m).astype(np.float32)
    b = rng.uniform(float(inc) / 2, float(inc), m).astype(np.float32)
    anti = (inc - b).astype(np.float32)                 # exact (Sterbenz)
    pts = [np.stack([a, a]), np.stack([b, anti])]
    for k in (1, 2):
        pts.append(np.stack([a, np.nextafter(a, np.float32(2)) if k == 1 else
                             np.nextafter(np.nextafter(a, np.float32(-2)), np.float32(-2))]))
        pts.append(np.stack([b, np.nextafter(anti, np.float32(2 * k - 3))]))
    # the diagonals of other squares: same remainder in both coordinates
    i = rng.integers(0, nc[0], m)
    j = rng.integers(0, nc[1], m)
    r = rng.uniform(0, 1, m)
    pts.append(np.stack([((i + r) / nc[0]).astype(np.float32),
                         ((j + r) / nc[1]).astype(np.float32)]))
    # domain corners with drift
    drift = np.array([0.0, -0.0, 1e-30, -1e-30, 1e-18, -1e-18, 1.3e-17, -7e-17, 1e-12, 1e-7],
                     dtype=np.float32)
    cx = rng.integers(0, 2, m).astype(np.float32)
    cy = rng.integers(0, 2, m).astype(np.float32)
    corner = np.stack([cx + rng.choice(drift, m), cy + rng.choice(drift, m)]).astype(np.float32)
    pts.append(corner)
    P = np.concatenate(pts, axis=1)
    fast, exact = run(harness, tmp_path, nc, P)
    answered = fast >= 0
    bad = np.nonzero(answered & (fast != exact))[0]
    assert bad.size == 0, 'FP32 tiers wrong at %s' % P[:, bad[:5]].T
    fc, _ = run(harness, tmp_path, nc, corner)
    if nc[0] == nc[1]:
        assert (fc >= 0).mean() > 0.99, (fc >= 0).mean()

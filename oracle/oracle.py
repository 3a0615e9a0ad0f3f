"""CPU oracle for the CPAB integration path.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker.  The libcpab_gb300 package never imports it.

Three independent restatements of the reference's algorithm:

* ``Oracle`` -- ctypes front-end of oracle/cpab_oracle.c, a C restatement of
  libcpab/core/cpab_ops.cpp (cell lookup, fixed-step forward, midpoint-rule
  sensitivity gradient) and of libcpab/pytorch/interpolation.py.
* ``numpy_transform_grid`` -- FP64 restatement of the reference's numpy
  backend (libcpab/numpy/transformer.py:22-61, libcpab/numpy/findcellidx.py),
  using scipy.linalg.expm per cell.
* ``fp64_autograd`` -- FP64 torch autograd through the same fixed-step scheme
  (B theta -> matrix_exp(dT [A;0]) -> gather -> affine, nstepsolver times),
  with the cell sequence frozen from the FP64 forward pass.  This is the exact
  derivative of the discrete forward map and the oracle for the exact adjoint.

``RefLib`` loads oracle/_ref/libcpab_ref.so, the reference's own
libcpab/core/cpab_ops.cpp compiled by oracle/build.py (only where the
reference checkout exists).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int)


def _p(a, t):
    return a.ctypes.data_as(t)


def n_cells(nc):
    nc = list(nc)
    if len(nc) == 1:
        return nc[0]
    if len(nc) == 2:
        return 4 * nc[0] * nc[1]
    return 5 * nc[0] * nc[1] * nc[2]


# --------------------------------------------------------------------------- #
# C oracle
# --------------------------------------------------------------------------- #
class Oracle:
    def __init__(self, path=None):
        if path is None:
            from oracle.build import build_oracle
            path = build_oracle()
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.oracle_findcellidx.argtypes = [ctypes.c_int, _i32p, _f32p, ctypes.c_long, _i32p]
        L.oracle_forward.argtypes = [ctypes.c_int, _i32p, ctypes.c_int, _f32p, ctypes.c_int,
                                     ctypes.c_long, _f32p, ctypes.c_int, _f32p, _i32p]
        L.oracle_backward.argtypes = [ctypes.c_int, _i32p, ctypes.c_int, _f32p, ctypes.c_int,
                                      ctypes.c_long, _f32p, ctypes.c_int, _f32p, ctypes.c_int,
                                      _f32p, _f64p]
        L.oracle_interpolate.argtypes = [ctypes.c_int, _f32p, ctypes.c_int, ctypes.c_int, _i32p,
                                         _f32p, _i32p, _f32p]
        L.oracle_interpolate_backward.argtypes = [ctypes.c_int, _f32p, ctypes.c_int, ctypes.c_int,
                                                  _i32p, _f32p, _i32p, _f32p, _f64p, _f32p]
        L.oracle_midpoint_trajectory.argtypes = [ctypes.c_int, _i32p, ctypes.c_int, _f32p,
                                                 ctypes.c_long, _f32p, _f32p, _i32p]
        L.oracle_num_threads.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]

    def num_threads(self):
        return self.lib.oracle_num_threads()

    def set_threads(self, n):
        self.lib.oracle_set_threads(int(n))

    def findcellidx(self, nc, points):
        pts = np.ascontiguousarray(points, dtype=np.float32)
        ndim, nP = pts.shape
        nca = np.asarray(nc, dtype=np.int32)
        out = np.empty(nP, dtype=np.int32)
        self.lib.oracle_findcellidx(ndim, _p(nca, _i32p), _p(pts, _f32p), nP, _p(out, _i32p))
        return out

    def forward(self, nc, nsteps, points, trels, return_cells=False):
        """points [ndim,nP] or [n_theta,ndim,nP]; trels [n_theta,nC,ndim,ndim+1]."""
        pts = np.ascontiguousarray(points, dtype=np.float32)
        tr = np.ascontiguousarray(trels, dtype=np.float32)
        n_theta = tr.shape[0]
        broadcast = int(pts.ndim == 3 and pts.shape[0] == n_theta)
        ndim, nP = pts.shape[-2], pts.shape[-1]
        nca = np.asarray(nc, dtype=np.int32)
        out = np.empty((n_theta, ndim, nP), dtype=np.float32)
        cells = np.empty((n_theta, nP, nsteps), dtype=np.int32) if return_cells else None
        self.lib.oracle_forward(ndim, _p(nca, _i32p), nsteps, _p(pts, _f32p), broadcast, nP,
                                _p(tr, _f32p), n_theta, _p(out, _f32p),
                                _p(cells, _i32p) if return_cells else None)
        return (out, cells) if return_cells else out

    def backward(self, nc, nsteps, points, As, Bs, grad):
        """Reference analytic dtheta [n_theta, d] (float64 accumulation)."""
        pts = np.ascontiguousarray(points, dtype=np.float32)
        A = np.ascontiguousarray(As, dtype=np.float32)
        B = np.ascontiguousarray(Bs, dtype=np.float32)
        g = np.ascontiguousarray(grad, dtype=np.float32)
        n_theta, d = A.shape[0], B.shape[0]
        broadcast = int(pts.ndim == 3 and pts.shape[0] == n_theta)
        ndim, nP = pts.shape[-2], pts.shape[-1]
        nca = np.asarray(nc, dtype=np.int32)
        out = np.zeros((n_theta, d), dtype=np.float64)
        self.lib.oracle_backward(ndim, _p(nca, _i32p), nsteps, _p(pts, _f32p), broadcast, nP,
                                 _p(A, _f32p), n_theta, _p(B, _f32p), d, _p(g, _f32p),
                                 _p(out, _f64p))
        return out

    def midpoint_trajectory(self, nc, nsteps, points, As):
        """The reference's midpoint trajectory of points [ndim, nP] under one
        theta's cell table As [nC, ndim, ndim+1]: (end points [ndim, nP],
        cells [nP, nsteps])."""
        pts = np.ascontiguousarray(points, dtype=np.float32)
        A = np.ascontiguousarray(As, dtype=np.float32)
        ndim, nP = pts.shape
        nca = np.asarray(nc, dtype=np.int32)
        out = np.empty((ndim, nP), dtype=np.float32)
        cells = np.empty((nP, nsteps), dtype=np.int32)
        self.lib.oracle_midpoint_trajectory(ndim, _p(nca, _i32p), nsteps, _p(pts, _f32p), nP,
                                            _p(A, _f32p), _p(out, _f32p), _p(cells, _i32p))
        return out, cells

    def interpolate(self, data, grid, outsize):
        D = np.ascontiguousarray(data, dtype=np.float32)
        G = np.ascontiguousarray(grid, dtype=np.float32)
        ndim = G.shape[1]
        nb, C = D.shape[:2]
        size = np.asarray(D.shape[2:], dtype=np.int32)
        osz = np.asarray(outsize, dtype=np.int32)
        out = np.empty((nb, C, *[int(o) for o in outsize]), dtype=np.float32)
        self.lib.oracle_interpolate(ndim, _p(D, _f32p), nb, C, _p(size, _i32p), _p(G, _f32p),
                                    _p(osz, _i32p), _p(out, _f32p))
        return out

    def interpolate_backward(self, data, grid, outsize, gout):
        D = np.ascontiguousarray(data, dtype=np.float32)
        G = np.ascontiguousarray(grid, dtype=np.float32)
        W = np.ascontiguousarray(gout, dtype=np.float32)
        ndim = G.shape[1]
        nb, C = D.shape[:2]
        size = np.asarray(D.shape[2:], dtype=np.int32)
        osz = np.asarray(outsize, dtype=np.int32)
        ddata = np.zeros(D.shape, dtype=np.float64)
        dgrid = np.empty(G.shape, dtype=np.float32)
        self.lib.oracle_interpolate_backward(ndim, _p(D, _f32p), nb, C, _p(size, _i32p),
                                             _p(G, _f32p), _p(osz, _i32p), _p(W, _f32p),
                                             _p(ddata, _f64p), _p(dgrid, _f32p))
        return ddata, dgrid


class RefLib:
    """The reference's own libcpab/core/cpab_ops.cpp (compiled by oracle/build.py)."""

    def __init__(self, path=None):
        if path is None:
            from oracle.build import build_ref
            path = build_ref()
        if path is None or not os.path.exists(path):
            raise FileNotFoundError('reference CPU library not built (no reference checkout)')
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.ref_findcellidx.argtypes = [ctypes.c_int, _f32p, _i32p]
        L.ref_findcellidx.restype = ctypes.c_int
        L.ref_forward.argtypes = [_f32p, _f32p, _f32p, _i32p, _i32p, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int]
        L.ref_backward.argtypes = [_f32p, _f32p, _f32p, _f32p, _i32p, _i32p, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int]

    def findcellidx(self, nc, points):
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float32).T)
        nca = np.asarray(nc, dtype=np.int32)
        return np.array([self.lib.ref_findcellidx(len(nc), _p(pts[i], _f32p), _p(nca, _i32p))
                         for i in range(pts.shape[0])], dtype=np.int32)

    def forward(self, nc, nsteps, points, trels):
        pts = np.ascontiguousarray(points, dtype=np.float32)
        tr = np.ascontiguousarray(trels, dtype=np.float32)
        n_theta = tr.shape[0]
        broadcast = int(pts.ndim == 3 and pts.shape[0] == n_theta)
        ndim, nP = pts.shape[-2], pts.shape[-1]
        nca = np.asarray(nc, dtype=np.int32)
        ns = np.asarray([nsteps], dtype=np.int32)
        out = np.zeros((n_theta, ndim, nP), dtype=np.float32)
        self.lib.ref_forward(_p(out, _f32p), _p(pts, _f32p), _p(tr, _f32p), _p(ns, _i32p),
                             _p(nca, _i32p), ndim, nP, n_theta, broadcast)
        return out

    def _chunks(self, n_theta, nP, threads):
        per = max(256, -(-nP * n_theta // (4 * threads)))
        return [(t, a, min(nP, a + per)) for t in range(n_theta) for a in range(0, nP, per)]

    def forward_threaded(self, nc, nsteps, points, trels, threads):
        """ref_forward over (theta, point-chunk) slices on `threads` host
        threads (the op itself is single-threaded); points [ndim, nP]."""
        import concurrent.futures
        pts = np.ascontiguousarray(points, dtype=np.float32)
        tr = np.ascontiguousarray(trels, dtype=np.float32)
        n_theta, (ndim, nP) = tr.shape[0], pts.shape
        nca = np.asarray(nc, dtype=np.int32)
        ns = np.asarray([nsteps], dtype=np.int32)
        out = np.zeros((n_theta, ndim, nP), dtype=np.float32)

        def run(job):
            t, a, b = job
            sub = np.ascontiguousarray(pts[:, a:b])
            o = np.zeros((1, ndim, b - a), dtype=np.float32)
            self.lib.ref_forward(_p(o, _f32p), _p(sub, _f32p), _p(tr[t], _f32p), _p(ns, _i32p),
                                 _p(nca, _i32p), ndim, b - a, 1, 0)
            out[t, :, a:b] = o[0]
        with concurrent.futures.ThreadPoolExecutor(threads) as ex:
            list(ex.map(run, self._chunks(n_theta, nP, threads)))
        return out

    def dtheta_threaded(self, nc, nsteps, points, As, Bs, grad, threads):
        """The reference's analytic gradient, dtheta [n_theta, d]: ref_backward
        (the [d, 1, ndim, chunk] sensitivity of one theta's point chunk)
        contracted with grad [n_theta, ndim, nP] (float64 sums), over
        (theta, point-chunk) slices on `threads` host threads."""
        import concurrent.futures
        pts = np.ascontiguousarray(points, dtype=np.float32)
        A = np.ascontiguousarray(As, dtype=np.float32)
        B = np.ascontiguousarray(Bs, dtype=np.float32)
        n_theta, nC = A.shape[0], A.shape[1]
        d = B.shape[0]
        ndim, nP = pts.shape
        nca = np.asarray(nc, dtype=np.int32)
        ns = np.asarray([nsteps], dtype=np.int32)
        jobs = self._chunks(n_theta, nP, threads)

        def run(job):
            t, a, b = job
            sub = np.ascontiguousarray(pts[:, a:b])
            sens = np.zeros((d, 1, ndim, b - a), dtype=np.float32)
            self.lib.ref_backward(_p(sens, _f32p), _p(sub, _f32p), _p(A[t], _f32p),
                                  _p(B, _f32p), _p(ns, _i32p), _p(nca, _i32p), 1, d, ndim,
                                  b - a, nC, 0)
            return t, np.einsum('kjp,jp->k', sens[:, 0].astype(np.float64),
                                grad[t, :, a:b].astype(np.float64))
        dth = np.zeros((n_theta, d))
        with concurrent.futures.ThreadPoolExecutor(threads) as ex:
            for t, part in ex.map(run, jobs):
                dth[t] += part
        return dth

    def backward_sensitivity(self, nc, nsteps, points, As, Bs):
        """The reference's [d, n_theta, ndim, nP] sensitivity tensor."""
        pts = np.ascontiguousarray(points, dtype=np.float32)
        A = np.ascontiguousarray(As, dtype=np.float32)
        B = np.ascontiguousarray(Bs, dtype=np.float32)
        n_theta, nC = A.shape[0], A.shape[1]
        d = B.shape[0]
        broadcast = int(pts.ndim == 3 and pts.shape[0] == n_theta)
        ndim, nP = pts.shape[-2], pts.shape[-1]
        nca = np.asarray(nc, dtype=np.int32)
        ns = np.asarray([nsteps], dtype=np.int32)
        out = np.zeros((d, n_theta, ndim, nP), dtype=np.float32)
        self.lib.ref_backward(_p(out, _f32p), _p(pts, _f32p), _p(A, _f32p), _p(B, _f32p),
                              _p(ns, _i32p), _p(nca, _i32p), n_theta, d, ndim, nP, nC, broadcast)
        return out


# --------------------------------------------------------------------------- #
# FP64 numpy restatement of libcpab/numpy (transformer.py:22-61, findcellidx.py)
# --------------------------------------------------------------------------- #
def _np_round_min(a, b):
    return np.where(a < b, a, np.round(b))


def _lookup_constants(nc, semantics):
    """Cell widths and clamps.  'numpy': double 1/nc (libcpab/numpy/findcellidx.py);
    'cpp': the float values of libcpab/core/cpab_ops.cpp:40-45,108-110,139-141."""
    ndim = len(nc)
    if semantics == 'numpy':
        inc = [1.0 / n for n in nc]
        width = [nc[j] * inc[j] for j in range(ndim)]
        clamp = [width[j] - (1e-8) for j in range(ndim)]
    else:
        f32 = np.float32
        inc = [float(f32(1.0 / n)) for n in nc]
        width = [float(f32(f32(nc[j]) * f32(inc[j]))) for j in range(ndim)]
        if ndim == 2:
            clamp = [width[j] - 0.000000001 for j in range(ndim)]
        else:
            clamp = [float(f32(width[j] - 1e-8)) for j in range(ndim)]
            if ndim == 3:   # z clamp with inc_x (cpab_ops.cpp:141)
                clamp[2] = float(f32(float(f32(f32(nc[2]) * f32(inc[0]))) - 1e-8))
    return inc, width, clamp


def numpy_findcellidx(ndim, p, nc, semantics='numpy', return_margin=False):
    """Vectorised FP64 cell lookup of points p [ndim, n].

    semantics='numpy' follows the reference's numpy backend
    (libcpab/numpy/findcellidx.py:22-150): double cell widths 1/nc, and in 3D
    z takes part in the outside test.  semantics='cpp' applies the rules of
    the reference's C++/CUDA lookup (libcpab/core/cpab_ops.cpp:26-184) to
    double points: float cell widths and clamps, z not tested for the
    push-inside rule and clamped with nz*inc_x.

    return_margin also returns, per point, the distance (domain units) from
    the point to the nearest boundary of any decision the lookup takes: cell
    faces, clamps, sub-cell diagonals / tetrahedron planes, out-of-domain
    rules and the push-inside comparisons.  A float evaluation can only
    decide differently when this margin is below its rounding error."""
    p = np.array(p, dtype=np.float64, copy=True)
    nc = list(nc)
    inc, width, clamp = _lookup_constants(nc, semantics)
    big = np.full(p.shape[1], np.inf)
    margin = big.copy()
    if ndim == 1:
        nx = nc[0]
        q = p[0] * nx
        idx = np.maximum(0.0, np.minimum(np.floor(q), nx - 1)).astype(np.int64)
        if return_margin:
            margin = np.abs(q - np.round(q)) / nx
            return idx, margin
        return idx
    if ndim == 2:
        nx, ny = nc
        ix, iy = inc
        wx, wy = width
        p0 = np.minimum(clamp[0], np.maximum(0.0, p[0]))
        p1 = np.minimum(clamp[1], np.maximum(0.0, p[1]))
        xm, ym = np.fmod(p0, ix), np.fmod(p1, iy)
        x, y = xm / ix, ym / iy
        idx = (_np_round_min(nx - 1, (p0 - xm) / ix) + _np_round_min(ny - 1, (p1 - ym) / iy) * nx) * 4
        ox, oy = p[0] / ix, p[1] / iy
        left, right = p[0] <= 0, p[0] >= wx
        c1 = left & (p[1] <= 0) & (oy < ox)
        c2 = ~c1 & left & (p[1] >= wy) & (oy - ny > -ox)
        c3 = ~c1 & ~c2 & left
        out = c1 | c2 | c3
        c4 = ~out & right & (p[1] <= 0) & (-oy > ox - nx)
        c5 = ~out & ~c4 & right & (p[1] >= wy) & (oy - ny > ox - nx)
        c6 = ~out & ~c4 & ~c5 & right
        out = out | c4 | c5 | c6
        c7 = ~out & (p[1] >= wy)
        out = out | c7
        c8 = ~out & (x < y) & (1 - x < y)
        c9 = ~out & ~c8 & (x < y)
        c10 = ~out & ~c8 & ~c9 & (x >= y) & (1 - x < y)
        idx = idx + 2 * (c2 | c5 | c7 | c8) + 3 * (c3 | c9) + 1 * (c6 | c10)
        if return_margin:
            s = min(ix, iy) / np.sqrt(2)
            for v in (p[0], p[0] - wx, p[1], p[1] - wy):            # branch tests
                margin = np.minimum(margin, np.abs(v))
            inside = ~(left | right | (p[1] <= 0) | (p[1] >= wy))
            face = np.minimum(np.minimum(xm, ix - xm), np.minimum(ym, iy - ym))
            tri = np.minimum(np.abs(x - y), np.abs(x + y - 1)) * s
            margin = np.where(inside, np.minimum(margin, np.minimum(face, tri)), margin)
            for cond, v in ((left & (p[1] <= 0), oy - ox), (left & (p[1] >= wy), oy - ny + ox),
                            (right & (p[1] <= 0), -oy - ox + nx),
                            (right & (p[1] >= wy), oy - ny - ox + nx)):
                margin = np.where(cond, np.minimum(margin, np.abs(v) * s), margin)
            # the edge square along the in-range axis
            margin = np.where(~inside & ~(left | right),
                              np.minimum(margin, np.minimum(xm, ix - xm)), margin)
            margin = np.where(~inside & (left | right) & (p[1] > 0) & (p[1] < wy),
                              np.minimum(margin, np.minimum(ym, iy - ym)), margin)
            return idx.astype(np.int64), margin
        return idx.astype(np.int64)
    nx, ny, nz = nc
    ix, iy, iz = inc
    outside = (p[0] < 0) | (p[0] > 1) | (p[1] < 0) | (p[1] > 1)
    if semantics == 'numpy':
        outside = outside | (p[2] < 0) | (p[2] > 1)
    h = 0.5
    q = p[:, outside] - h
    a = np.abs(q)
    push = [(h * ix) * ((a[0] < a[1]) & (a[0] < a[2])),
            (h * iy) * ((a[1] < a[0]) & (a[0] < a[2])),
            (h * iz) * ((a[2] < a[0]) & (a[0] < a[1]))]
    for j in range(3):
        m = a[j] > h
        q[j, m] = np.copysign(h - push[j][m], q[j, m])
    pp = p.copy()
    pp[:, outside] = q + h
    c = [np.minimum(clamp[j], np.maximum(0.0, pp[j])) for j in range(3)]
    xm = [np.mod(c[j], inc[j]) for j in range(3)]
    i = _np_round_min(nx - 1, (c[0] - xm[0]) / ix)
    j_ = _np_round_min(ny - 1, (c[1] - xm[1]) / iy)
    k = _np_round_min(nz - 1, (c[2] - xm[2]) / iz)
    idx = 5 * (i + j_ * nx + k * nx * ny)
    x, y, z = xm[0] / ix, xm[1] / iy, xm[2] / iz
    flip = (((k % 2 == 0) & (i % 2 == 0) & (j_ % 2 == 1)) | ((k % 2 == 0) & (i % 2 == 1) & (j_ % 2 == 0)) |
            ((k % 2 == 1) & (i % 2 == 0) & (j_ % 2 == 0)) | ((k % 2 == 1) & (i % 2 == 1) & (j_ % 2 == 1)))
    x, y = np.where(flip, y, x), np.where(flip, 1 - x, y)
    t1 = -x - y + z >= 0
    t2 = x + y + z - 2 >= 0
    t3 = -x + y - z >= 0
    t4 = x - y - z >= 0
    idx = idx + 1 * t1 + 2 * (t2 & ~t1) + 3 * (t3 & ~t1 & ~t2) + 4 * (t4 & ~t1 & ~t2 & ~t3)
    if return_margin:
        s = min(inc) / np.sqrt(3)
        for v in (p[0], p[0] - 1, p[1], p[1] - 1):                 # push-inside test
            margin = np.minimum(margin, np.abs(v))
        pm = np.full(p.shape[1], np.inf)                          # push comparisons
        for u, v in ((0, 1), (0, 2), (1, 2)):
            pm[outside] = np.minimum(pm[outside], np.abs(a[u] - a[v]))
        for j in range(3):
            pm[outside] = np.minimum(pm[outside], np.abs(a[j] - h))
        margin = np.minimum(margin, pm)
        for j in range(3):
            margin = np.minimum(margin, np.abs(pp[j] - clamp[j]))
            margin = np.minimum(margin, np.where(pp[j] > 0, np.abs(pp[j]), np.inf))
            margin = np.minimum(margin, np.minimum(xm[j], inc[j] - xm[j]))
        for v in (-x - y + z, x + y + z - 2, -x + y - z, x - y - z):
            margin = np.minimum(margin, np.abs(v) * s)
        return idx.astype(np.int64), margin
    return idx.astype(np.int64)


def step_maps_fp64(basis, theta, ndim, nsteps):
    """T_c = expm(dT [A_c; 0]) in float64, [n_theta, nC, ndim+1, ndim+1]."""
    from scipy.linalg import expm
    B = np.asarray(basis, dtype=np.float64)
    th = np.asarray(theta, dtype=np.float64)
    n_theta = th.shape[0]
    nC = B.shape[0] // (ndim * (ndim + 1))
    A = (B @ th.T).T.reshape(n_theta * nC, ndim, ndim + 1)
    Asq = np.concatenate([A, np.zeros((n_theta * nC, 1, ndim + 1))], axis=1)
    dT = 1.0 / nsteps
    T = np.stack([expm(dT * a) for a in Asq])
    return T.reshape(n_theta, nC, ndim + 1, ndim + 1)


def numpy_transform_grid(basis, theta, points, nc, nsteps=50, return_cells=False,
                         return_margin=False, semantics='numpy'):
    """FP64 fixed-step integration with the numpy backend's semantics
    (semantics='cpp' uses the C++/CUDA cell rules, see numpy_findcellidx).

    return_margin adds, per point, the smallest decision_margin met along the
    trajectory ([n_theta, nP])."""
    nc = list(nc)
    ndim = len(nc)
    th = np.asarray(theta, dtype=np.float64)
    n_theta = th.shape[0]
    pts = np.asarray(points, dtype=np.float64)
    nP = pts.shape[-1]
    T = step_maps_fp64(basis, th, ndim, nsteps)
    nC = T.shape[1]
    P = np.broadcast_to(pts, (n_theta, ndim, nP)) if pts.ndim == 2 else pts
    P = np.ascontiguousarray(np.transpose(P, (0, 2, 1))).reshape(-1, ndim)
    Ph = np.concatenate([P, np.ones((P.shape[0], 1))], axis=1)[:, :, None]
    Tf = T.reshape(n_theta * nC, ndim + 1, ndim + 1)
    base = np.repeat(np.arange(n_theta) * nC, nP)
    cells, margins = [], []
    for _ in range(nsteps):
        if return_margin:
            c, mg = numpy_findcellidx(ndim, Ph[:, :ndim, 0].T, nc, semantics, return_margin=True)
            margins.append(mg)
        else:
            c = numpy_findcellidx(ndim, Ph[:, :ndim, 0].T, nc, semantics)
        cells.append(c)
        Ph = np.matmul(Tf[c + base], Ph)
    out = Ph[:, :ndim, 0].reshape(n_theta, nP, ndim).transpose(0, 2, 1)
    res = [out]
    if return_cells:
        res.append(np.stack(cells, axis=1).reshape(n_theta, nP, nsteps))
    if return_margin == 'steps':
        res.append(np.stack(margins, axis=1).reshape(n_theta, nP, nsteps))
    elif return_margin:
        res.append(np.min(np.stack(margins, axis=1), axis=1).reshape(n_theta, nP))
    return res[0] if len(res) == 1 else tuple(res)


# --------------------------------------------------------------------------- #
# FP64 autograd oracle for gradients
# --------------------------------------------------------------------------- #
def fp64_autograd(basis, theta, points, nc, cotangent, nsteps=50, cells=None):
    """Exact derivative of the discrete forward map, in float64.

    Returns (out [n_theta,ndim,nP], dtheta [n_theta,d], dpoints like points).
    The cell at each step is frozen: from ``cells`` ([n_theta,nP,nsteps]) if
    given, else looked up on the FP64 trajectory with the C++ lookup rules.
    """
    import torch
    nc = list(nc)
    ndim = len(nc)
    B = torch.as_tensor(np.asarray(basis, dtype=np.float64))
    th = torch.tensor(np.asarray(theta, dtype=np.float64), requires_grad=True)
    pts = torch.tensor(np.asarray(points, dtype=np.float64), requires_grad=True)
    n_theta = th.shape[0]
    nC = B.shape[0] // (ndim * (ndim + 1))
    nP = pts.shape[-1]
    A = (B @ th.T).T.reshape(n_theta, nC, ndim, ndim + 1)
    Asq = torch.cat([A, torch.zeros(n_theta, nC, 1, ndim + 1, dtype=A.dtype)], dim=2)
    T = torch.linalg.matrix_exp(Asq / nsteps)[:, :, :ndim, :]          # [n_theta,nC,n,n+1]
    P = pts.expand(n_theta, ndim, nP) if pts.dim() == 2 else pts
    P = P.permute(0, 2, 1)                                               # [n_theta,nP,n]
    ones = torch.ones(n_theta, nP, 1, dtype=P.dtype)
    tidx = torch.arange(n_theta)[:, None].expand(n_theta, nP)
    if cells is None:
        lookup = Oracle()
    for s in range(nsteps):
        if cells is None:
            pf = P.detach().numpy().reshape(-1, ndim).T.astype(np.float32)
            c = torch.as_tensor(lookup.findcellidx(nc, pf).astype(np.int64)).reshape(n_theta, nP)
        else:
            c = torch.as_tensor(np.asarray(cells)[:, :, s].astype(np.int64))
        Tc = T[tidx, c]                                                 # [n_theta,nP,n,n+1]
        Ph = torch.cat([P, ones], dim=2)
        P = (Tc @ Ph[..., None])[..., 0]
    out = P.permute(0, 2, 1)
    w = torch.as_tensor(np.asarray(cotangent, dtype=np.float64))
    (out * w).sum().backward()
    return out.detach().numpy(), th.grad.numpy(), pts.grad.numpy()


# --------------------------------------------------------------------------- #
# FP64 oracle of the exact-flow scheme
# --------------------------------------------------------------------------- #
def exact_flow_fp64(basis, theta, points, nc, rtol=1e-12, atol=1e-13):
    """Flow of the continuous piecewise-affine field for time 1, in float64.

    An independent check of the exact-flow kernels: instead of their
    in-cell analytic steps, the ODE dx/dt = v(x) is integrated for all points
    of one theta at once by scipy's DOP853 with tight tolerances.  v uses the
    C++ cell rules (numpy_findcellidx, semantics='cpp'); the field is
    continuous across faces, so which side a point on a face is given to does
    not matter.  Returns [n_theta, ndim, nP]."""
    from scipy.integrate import solve_ivp
    nc = list(nc)
    ndim = len(nc)
    B = np.asarray(basis, dtype=np.float64)
    th = np.asarray(theta, dtype=np.float64)
    nC = B.shape[0] // (ndim * (ndim + 1))
    pts = np.asarray(points, dtype=np.float64)
    nP = pts.shape[-1]
    out = np.empty((th.shape[0], ndim, nP))
    for k in range(th.shape[0]):
        A = (B @ th[k]).reshape(nC, ndim, ndim + 1)
        p0 = pts[k] if pts.ndim == 3 else pts

        def field(_t, y):
            P = y.reshape(ndim, nP)
            c = numpy_findcellidx(ndim, P.astype(np.float32), nc, semantics='cpp')
            Ph = np.concatenate([P, np.ones((1, nP))], axis=0)
            return np.einsum('nij,jn->in', A[c], Ph).reshape(-1)
        sol = solve_ivp(field, (0.0, 1.0), p0.reshape(-1), method='DOP853', rtol=rtol,
                        atol=atol)
        out[k] = sol.y[:, -1].reshape(ndim, nP)
    return out


def exact_flow_grad_fp64(basis, theta, points, nc, cot, rtol=1e-10, atol=1e-12):
    """Gradient of the exact flow for time 1, in float64: (dtheta [n_theta, d],
    dpoints [n_theta, ndim, nP]) of L = sum(cot * phi_1(points)).

    Forward sensitivities, independent of the kernels' reverse sweep: the
    state of a point is its position p, S = dp/dtheta [ndim, d] and
    J = dp/dp0 [ndim, ndim], integrated together by DOP853:
        dp/dt = A_c p~,   dS/dt = A_c,lin S + dv/dtheta,   dJ/dt = A_c,lin J,
    with dv_i/dtheta_k = sum_j B[c, i, j, k] p~_j (A_c = B_c theta, the cell
    of p by the C++ rules).  The field is continuous across faces, so the
    sensitivities are continuous too and need no jump conditions.  Each point
    is integrated on its own: the right-hand side is discontinuous where the
    point crosses a face, and a joint system would take small steps at every
    crossing of every point."""
    from scipy.integrate import solve_ivp
    nc = list(nc)
    ndim = len(nc)
    B = np.asarray(basis, dtype=np.float64)
    th = np.asarray(theta, dtype=np.float64)
    d = B.shape[1]
    nC = B.shape[0] // (ndim * (ndim + 1))
    Br = B.reshape(nC, ndim, ndim + 1, d)
    pts = np.asarray(points, dtype=np.float64)
    nP = pts.shape[-1]
    cot = np.asarray(cot, dtype=np.float64)
    dth = np.zeros((th.shape[0], d))
    dpts = np.zeros((th.shape[0], ndim, nP))
    n_s = ndim * d
    for k in range(th.shape[0]):
        A = (B @ th[k]).reshape(nC, ndim, ndim + 1)
        p0s = pts[k] if pts.ndim == 3 else pts

        def field(_t, y):
            p = y[:ndim]
            S = y[ndim:ndim + n_s].reshape(ndim, d)
            J = y[ndim + n_s:].reshape(ndim, ndim)
            c = int(numpy_findcellidx(ndim, p.reshape(ndim, 1).astype(np.float32), nc,
                                      semantics='cpp')[0])
            Ac = A[c]
            ph = np.append(p, 1.0)
            return np.concatenate([Ac @ ph, (Ac[:, :ndim] @ S + np.einsum('ijk,j->ik', Br[c], ph))
                                   .reshape(-1), (Ac[:, :ndim] @ J).reshape(-1)])
        for q in range(nP):
            y0 = np.concatenate([p0s[:, q], np.zeros(n_s), np.eye(ndim).reshape(-1)])
            sol = solve_ivp(field, (0.0, 1.0), y0, method='DOP853', rtol=rtol, atol=atol)
            y = sol.y[:, -1]
            S = y[ndim:ndim + n_s].reshape(ndim, d)
            J = y[ndim + n_s:].reshape(ndim, ndim)
            dth[k] += cot[k][:, q] @ S
            dpts[k][:, q] = cot[k][:, q] @ J
    return dth, dpts

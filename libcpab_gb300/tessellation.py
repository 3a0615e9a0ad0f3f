"""Tessellation of the domain [0,1]^ndim and the CPA velocity-field basis B.

A CPA (continuous piecewise-affine) velocity field assigns each cell c an affine
map A_c (ndim x (ndim+1)).  Stacking all cells gives a vector of D = nC*ndim*(ndim+1)
numbers; the admissible fields are the null space of a constraint matrix L
(continuity across shared faces, optional zero normal velocity on the domain
boundary, optional zero trace).  B = null(L) is a [D, d] orthonormal basis and a
parameter vector theta (length d) means A = B @ theta.

theta only has a meaning relative to one specific B.  The null space is
degenerate, so any orthonormal basis of it is "a" basis; to be interchangeable
with libcpab, this module builds *the same* matrix L row for row as
libcpab/core/tesselation.py:37-442 and takes its null space with the same LAPACK
call (libcpab/core/utility.py:27-42: scipy.linalg.svd, gesdd, eps=1e-6).  On the
same numpy/scipy build that yields a bit-identical B.  Pair finding is done with
a vertex->cell index instead of the O(nC^2) double loop of the reference, but the
constraint rows come out in the reference's order, including the order in which
Python sets enumerate the shared vertices (libcpab/core/tesselation.py:119-121).

The pickle cache uses the reference's file name scheme and content
(libcpab/core/tesselation.py:60-98), so a basis file written by libcpab can be
loaded here and vice versa.
"""
from __future__ import annotations

import os
import pickle

import numpy as np
import scipy.linalg as la


def null_space(L: np.ndarray, eps: float = 1e-6) -> np.ndarray:
    """Null space of L as columns, from a full SVD.

    Follows libcpab/core/utility.py:27-42: singular values <= eps, plus the
    rows of Vh beyond len(s), select the null-space rows of Vh.
    """
    _, s, vh = la.svd(L)
    padding = max(0, L.shape[-1] - s.shape[0])
    mask = np.concatenate((s <= eps, np.ones((padding,), dtype=bool)))
    return np.compress(mask, vh, axis=0).T


def _hashable(arr) -> tuple:
    # Same conversion as libcpab/core/utility.py:45-49 (python floats).
    return tuple(tuple(r.tolist()) for r in arr)


def basis_file_name(nc, zero_boundary: bool, volume_perservation: bool) -> str:
    """File stem used by libcpab for a cached basis (tesselation.py:60-65)."""
    return ('cpab_basis_dim' + str(len(nc)) + '_tess' +
            '_'.join(str(e) for e in nc) + '_' +
            'vo' + str(int(not zero_boundary)) + '_' +
            'zb' + str(int(zero_boundary)) + '_' +
            'vp' + str(int(volume_perservation)))


class Tessellation:
    """Base class: builds verts/cells, L and B for one tessellation config.

    Attribute names match libcpab's Tesselation objects (nc, ndim, nC,
    n_params, verts, cells, shared_v, shared_v_idx, L, B) so that the pickled
    __dict__ is interchangeable with libcpab's basis files.
    """
    n_params = 0
    ndim = 0

    def __init__(self, nc, domain_min, domain_max, zero_boundary=True,
                 volume_perservation=False, direc=None, override=False, basis=True):
        self.nc = list(nc)
        self.domain_min = list(domain_min)
        self.domain_max = list(domain_max)
        self.zero_boundary = zero_boundary
        self.volume_perservation = volume_perservation
        self.dir = direc
        stem = basis_file_name(self.nc, zero_boundary, volume_perservation)
        self._basis_file = None if direc is None else os.path.join(direc, stem)

        cached = (self._basis_file is not None and not override and
                  os.path.isfile(self._basis_file + '.pkl'))
        if cached:
            with open(self._basis_file + '.pkl', 'rb') as f:
                state = pickle.load(f)
            self.__dict__.update(state)
            return

        self.find_verts()
        self.find_shared_verts()
        if not zero_boundary:
            self.find_verts_outside()
        rows = [self.create_continuity_constrains()]
        if zero_boundary:
            rows.append(self.create_zero_boundary_constrains())
        if volume_perservation:
            rows.append(self.create_zero_trace_constrains())
        self.L = np.concatenate(rows, axis=0)
        if not basis:           # constraint matrix only (no SVD, nothing cached)
            self.B = None
            return
        self.B = null_space(self.L)

        if self._basis_file is not None:
            os.makedirs(direc, exist_ok=True)
            tmp = self._basis_file + '.pkl.tmp%d' % os.getpid()
            with open(tmp, 'wb') as f:
                pickle.dump(self.__dict__, f, pickle.HIGHEST_PROTOCOL)
            os.replace(tmp, self._basis_file + '.pkl')

    # ------------------------------------------------------------------ #
    def get_cell_centers(self) -> np.ndarray:
        return np.mean(self.verts[:, :, :self.ndim], axis=1)

    def find_verts(self):
        raise NotImplementedError

    def find_verts_outside(self):
        raise NotImplementedError

    def create_zero_boundary_constrains(self):
        raise NotImplementedError

    def find_shared_verts(self):
        """Cell pairs (i<j, lexicographic) sharing exactly ndim vertices.

        Same pairs, order and vertex order as libcpab/core/tesselation.py:109-126;
        candidates come from a vertex -> cells index.
        """
        hv = [_hashable(self.verts[c]) for c in range(self.nC)]
        by_vert: dict = {}
        for c, vs in enumerate(hv):
            for v in vs:
                by_vert.setdefault(v, []).append(c)
        pairs = set()
        for cells in by_vert.values():
            for a in cells:
                for b in cells:
                    if a < b:
                        pairs.add((a, b))
        shared_v, shared_idx = [], []
        for (i, j) in sorted(pairs):
            sv = set(hv[i]).intersection(hv[j])
            if len(sv) == self.ndim:
                shared_v.append(list(sv)[:self.ndim])
                shared_idx.append((i, j))
        self.shared_v = np.asarray(shared_v)
        self.shared_v_idx = shared_idx

    def create_continuity_constrains(self) -> np.ndarray:
        """ndim*ndim rows per shared pair (tesselation.py:134-148)."""
        n, p = self.ndim, self.n_params
        npair = len(self.shared_v_idx)
        L = np.zeros((npair * n * n, p * self.nC))
        r = 0
        for idx in range(npair):
            i, j = self.shared_v_idx[idx]
            i, j = int(i), int(j)
            for vidx in range(n):
                v = self.shared_v[idx][vidx]
                for k in range(n):
                    a = p * i + k * (n + 1)
                    b = p * j + k * (n + 1)
                    L[r, a:a + n + 1] = v
                    L[r, b:b + n + 1] = -v
                    r += 1
        return L

    def create_zero_trace_constrains(self) -> np.ndarray:
        """One row per cell: trace of the linear part is zero (tesselation.py:155-162)."""
        L = np.zeros((self.nC, self.n_params * self.nC))
        row = np.concatenate((np.eye(self.ndim), np.zeros((self.ndim, 1))), axis=1).flatten()
        for c in range(self.nC):
            L[c, self.n_params * c:self.n_params * (c + 1)] = row
        return L


class Tessellation1D(Tessellation):
    """nc intervals on [0,1] (tesselation.py:165-200)."""

    def __init__(self, nc, domain_min, domain_max, zero_boundary=True,
                 volume_perservation=False, direc=None, override=False, basis=True):
        self.n_params = 2
        self.nC = int(np.prod(nc))
        self.ndim = 1
        super().__init__(nc, domain_min, domain_max, zero_boundary,
                         volume_perservation, direc, override, basis)

    def find_verts(self):
        Vx = np.linspace(self.domain_min[0], self.domain_max[0], self.nc[0] + 1)
        verts = [((Vx[i], 1), (Vx[i + 1], 1)) for i in range(self.nc[0])]
        self.verts = np.asarray(verts)
        self.cells = list(range(self.nc[0]))

    def find_verts_outside(self):
        pass

    def create_zero_boundary_constrains(self):
        L = np.zeros((2, 2 * self.nC))
        L[0, :2] = [self.domain_min[0], 1]
        L[1, -2:] = [self.domain_max[0], 1]
        return L


class Tessellation2D(Tessellation):
    """Each of nc[0] x nc[1] squares is split into 4 triangles around its centre
    (top, right, bottom, left: tesselation.py:216-244)."""

    def __init__(self, nc, domain_min, domain_max, zero_boundary=True,
                 volume_perservation=False, direc=None, override=False, basis=True):
        self.n_params = 6
        self.nC = 4 * int(np.prod(nc))
        self.ndim = 2
        super().__init__(nc, domain_min, domain_max, zero_boundary,
                         volume_perservation, direc, override, basis)

    def find_verts(self):
        Vx = np.linspace(self.domain_min[0], self.domain_max[0], self.nc[0] + 1)
        Vy = np.linspace(self.domain_min[1], self.domain_max[1], self.nc[1] + 1)
        cells, verts = [], []
        for i in range(self.nc[1]):
            for j in range(self.nc[0]):
                ul = (Vx[j], Vy[i], 1)
                ur = (Vx[j + 1], Vy[i], 1)
                ll = (Vx[j], Vy[i + 1], 1)
                lr = (Vx[j + 1], Vy[i + 1], 1)
                center = ((Vx[j] + Vx[j + 1]) / 2, (Vy[i] + Vy[i + 1]) / 2, 1)
                verts += [(center, ul, ur), (center, ur, lr),
                          (center, lr, ll), (center, ll, ul)]
                cells += [(j, i, 0), (j, i, 1), (j, i, 2), (j, i, 3)]
        self.verts = np.asarray(verts)
        self.cells = cells

    def find_verts_outside(self):
        """Extra continuity rows that extend the field outside the domain.

        Pairs of boundary triangles in adjacent boundary squares, joined at
        their single shared corner plus an auxiliary vertex 10 units away
        (tesselation.py:246-311).  The reference scans all (i,j) pairs; only
        boundary triangles can qualify, so only those are scanned here, in the
        same (i,j) order.
        """
        nx, ny = self.nc
        shared_v, shared_idx = [], []
        seen = set()

        def side(m):
            # which boundary classes cell m belongs to
            s = []
            if m[0] == 0 and m[2] == 3:
                s.append('l')
            if m[0] == nx - 1 and m[2] == 1:
                s.append('r')
            if m[1] == 0 and m[2] == 0:
                s.append('t')
            if m[1] == ny - 1 and m[2] == 2:
                s.append('b')
            return s

        cand = [c for c in range(self.nC) if side(self.cells[c])]
        hv = {c: _hashable(self.verts[c]) for c in cand}
        for i in cand:
            for j in cand:
                mi, mj = self.cells[i], self.cells[j]
                left = mi[0] == mj[0] == 0 and mi[2] == mj[2] == 3 and abs(mi[1] - mj[1]) == 1
                right = mi[0] == mj[0] == nx - 1 and mi[2] == mj[2] == 1 and abs(mi[1] - mj[1]) == 1
                top = mi[1] == mj[1] == 0 and mi[2] == mj[2] == 0 and abs(mi[0] - mj[0]) == 1
                bottom = mi[1] == mj[1] == ny - 1 and mi[2] == mj[2] == 2 and abs(mi[0] - mj[0]) == 1
                if not (left or right or top or bottom):
                    continue
                sv = set(hv[i]).intersection(hv[j])
                if len(sv) == 1 and (j, i) not in seen:
                    v0 = list(sv)[0]
                    v_aux = list(v0)
                    if left or right:
                        v_aux[0] -= 10
                    else:
                        v_aux[1] -= 10
                    shared_v.append([tuple(sv)[0], tuple(v_aux)])
                    shared_idx.append((i, j))
                    seen.add((i, j))
        if shared_v:
            self.shared_v = np.concatenate((self.shared_v, shared_v))
            self.shared_v_idx = np.concatenate((self.shared_v_idx, shared_idx))

    def create_zero_boundary_constrains(self):
        xmin, ymin = self.domain_min
        xmax, ymax = self.domain_max
        rows = []
        for c in range(self.nC):
            for v in self.verts[c]:
                if v[0] == xmin or v[0] == xmax:
                    row = np.zeros(6 * self.nC)
                    row[6 * c:6 * c + 3] = v
                    rows.append(row)
                if v[1] == ymin or v[1] == ymax:
                    row = np.zeros(6 * self.nC)
                    row[6 * c + 3:6 * c + 6] = v
                    rows.append(row)
        return np.asarray(rows).reshape(-1, 6 * self.nC)


class Tessellation3D(Tessellation):
    """Each cube is split into 5 tetrahedra, with the split mirrored on
    alternating cubes so faces match (tesselation.py:343-386)."""

    def __init__(self, nc, domain_min, domain_max, zero_boundary=True,
                 volume_perservation=False, direc=None, override=False, basis=True):
        self.n_params = 12
        self.nC = 5 * int(np.prod(nc))
        self.ndim = 3
        super().__init__(nc, domain_min, domain_max, zero_boundary,
                         volume_perservation, direc, override, basis)

    def find_verts(self):
        Vx = np.linspace(self.domain_min[0], self.domain_max[0], self.nc[0] + 1)
        Vy = np.linspace(self.domain_min[1], self.domain_max[1], self.nc[1] + 1)
        Vz = np.linspace(self.domain_min[2], self.domain_max[2], self.nc[2] + 1)
        cells, verts = [], []
        for i in range(self.nc[2]):
            for j in range(self.nc[1]):
                for k in range(self.nc[0]):
                    ul0 = (Vx[k], Vy[j], Vz[i], 1)
                    ur0 = (Vx[k + 1], Vy[j], Vz[i], 1)
                    ll0 = (Vx[k], Vy[j + 1], Vz[i], 1)
                    lr0 = (Vx[k + 1], Vy[j + 1], Vz[i], 1)
                    ul1 = (Vx[k], Vy[j], Vz[i + 1], 1)
                    ur1 = (Vx[k + 1], Vy[j], Vz[i + 1], 1)
                    ll1 = (Vx[k], Vy[j + 1], Vz[i + 1], 1)
                    lr1 = (Vx[k + 1], Vy[j + 1], Vz[i + 1], 1)
                    if k % 2 == 0:
                        flip = (i % 2 == 0 and j % 2 == 1) or (i % 2 == 1 and j % 2 == 0)
                    else:
                        flip = (i % 2 == 0 and j % 2 == 0) or (i % 2 == 1 and j % 2 == 1)
                    if flip:
                        ul0, ur0, lr0, ll0 = ur0, lr0, ll0, ul0
                        ul1, ur1, lr1, ll1 = ur1, lr1, ll1, ul1
                    verts += [(ll1, ur1, ul0, lr0), (ul1, ur1, ll1, ul0),
                              (lr1, ur1, ll1, lr0), (ll0, ul0, lr0, ll1),
                              (ur0, ul0, lr0, ur1)]
                    cells += [(k, j, i, l) for l in range(5)]
        self.verts = np.asarray(verts)
        self.cells = cells

    def find_verts_outside(self):
        """Rows tying together tetrahedra of one cube that touch the same
        domain face, through an auxiliary vertex one unit outside
        (tesselation.py:388-421).  Only same-cube pairs can qualify, so only
        those are scanned, in the reference's (i, j, axis) order."""
        shared_verts, shared_idx = [], []
        seen = set()
        for i in range(self.nC):
            base = (i // 5) * 5
            for j in range(base, base + 5):
                if i == j:
                    continue
                for d in range(self.ndim):
                    vi = self.verts[i]
                    vj = self.verts[j]
                    upper = (np.sum(vi[:, d] == self.domain_min[d]) == 3 and
                             np.sum(vj[:, d] == self.domain_min[d]) == 3)
                    lower = (np.sum(vi[:, d] == self.domain_max[d]) == 3 and
                             np.sum(vj[:, d] == self.domain_max[d]) == 3)
                    if (upper or lower) and (j, i) not in seen:
                        hvi, hvj = _hashable(vi), _hashable(vj)
                        sv = set(hvi).intersection(hvj)
                        center = [(a + b) / 2.0 for a, b in zip(hvi[0], hvj[0])]
                        center[d] += (-1) if upper else (+1)
                        shared_verts.append(list(sv.union([tuple(center)])))
                        shared_idx.append((i, j))
                        seen.add((i, j))
        if shared_verts:
            self.shared_v = np.concatenate((self.shared_v, np.asarray(shared_verts)))
            self.shared_v_idx = list(self.shared_v_idx) + shared_idx

    def create_zero_boundary_constrains(self):
        xmin, ymin, zmin = self.domain_min
        xmax, ymax, zmax = self.domain_max
        rows = []
        for c in range(self.nC):
            for v in self.verts[c]:
                if v[0] == xmin or v[0] == xmax:
                    row = np.zeros(12 * self.nC)
                    row[12 * c:12 * c + 4] = v
                    rows.append(row)
                if v[1] == ymin or v[1] == ymax:
                    row = np.zeros(12 * self.nC)
                    row[12 * c + 4:12 * c + 8] = v
                    rows.append(row)
                if v[2] == zmin or v[2] == zmax:
                    row = np.zeros(12 * self.nC)
                    row[12 * c + 8:12 * c + 12] = v
                    rows.append(row)
        return np.asarray(rows).reshape(-1, 12 * self.nC)


def make_tessellation(nc, zero_boundary=True, volume_perservation=False,
                      direc=None, override=False, basis=True) -> Tessellation:
    ndim = len(nc)
    cls = {1: Tessellation1D, 2: Tessellation2D, 3: Tessellation3D}[ndim]
    return cls(list(nc), [0] * ndim, [1] * ndim, zero_boundary,
               volume_perservation, direc, override, basis)

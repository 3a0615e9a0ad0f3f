"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in an environment that has the reference checkout (default
/root/reference, override with CPAB_REFERENCE_ROOT):

    python tests/golden/make_golden.py

The reference is copied to a temporary directory (its basis cache writes next
to the package) and imported with three shims that touch only this process:
matplotlib is stubbed (imported for plotting only), scipy.transpose /
scipy.compress are aliased to numpy's, and torch.solve is mapped to
torch.linalg.solve.  Every number stored here is produced by the reference's
own code: its numpy backend (FP64), its pytorch CPU backend (the C++ op
libcpab/core/cpab_ops.cpp, fp32) with its autograd backward, its pytorch
interpolation, and its C++ cell lookup (via oracle/_ref).

The script also checks that libcpab_gb300.tessellation builds the same
constraint matrix L (bit for bit) and the same basis B as the reference.
"""
import hashlib
import os
import shutil
import sys
import tempfile
import types
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
REFERENCE_ROOT = os.environ.get('CPAB_REFERENCE_ROOT', '/root/reference')

# name, nc, zero_boundary, volume_perservation, n_theta, theta scale,
# meshgrid size, data channels, data size, transform_data outsize
CONFIGS = [
    ('1d_50_zb', [50], True, False, 16, 1.0, [1000], 2, [120], [90]),
    ('1d_100_free', [100], False, False, 4, 1.0, [300], 1, [200], [150]),
    ('1d_7_zb_vp', [7], True, True, 3, 1.0, [64], 1, [40], [33]),
    ('2d_3x3_zb', [3, 3], True, False, 4, 0.5, [24, 20], 3, [40, 36], [32, 28]),
    ('2d_4x4_free', [4, 4], False, False, 3, 1.0, [16, 18], 2, [20, 22], [18, 16]),
    ('2d_2x3_zb_vp', [2, 3], True, True, 2, 1.0, [12, 10], 1, [16, 14], [12, 10]),
    ('3d_2x2x2_zb_vp', [2, 2, 2], True, True, 2, 1.0, [7, 6, 5], 1, [9, 8, 7], [6, 5, 4]),
    ('3d_2x2x2_free', [2, 2, 2], False, False, 2, 0.5, [6, 6, 6], 2, [8, 8, 8], [5, 6, 7]),
]

# Large tessellations: only L (hash) and, where small enough, B are stored.
LARGE = [
    ('L_2d_8x8_free', [8, 8], False, False, False),
    ('L_3d_4x4x4_zb_vp', [4, 4, 4], True, True, True),
]


def import_reference():
    import scipy
    import torch
    tmp = tempfile.mkdtemp(prefix='cpab_ref_')
    shutil.copytree(os.path.join(REFERENCE_ROOT, 'libcpab'), os.path.join(tmp, 'libcpab'),
                    ignore=shutil.ignore_patterns('*.o'))
    mpl = types.ModuleType('matplotlib')
    plt = types.ModuleType('matplotlib.pyplot')
    plt.figure = lambda *a, **k: None
    mpl.pyplot = plt
    sys.modules['matplotlib'] = mpl
    sys.modules['matplotlib.pyplot'] = plt
    scipy.transpose = np.transpose
    scipy.compress = np.compress
    torch.solve = lambda P, Q: (torch.linalg.solve(Q, P), None)
    sys.path.insert(0, tmp)
    import libcpab  # noqa: F401
    return tmp


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def probe_points(nc, rng):
    """Points on faces, corners, diagonals and outside the domain (float32)."""
    ndim = len(nc)
    ticks = []
    for j in range(ndim):
        t = [k / nc[j] for k in range(nc[j] + 1)]
        t += [np.float32(1.0 / nc[j]) * k for k in range(nc[j] + 1)]
        t += [np.nextafter(np.float32(x), np.float32(2)) for x in t[:nc[j] + 1]]
        t += [np.nextafter(np.float32(x), np.float32(-2)) for x in t[:nc[j] + 1]]
        t += [-0.3, -1e-7, 0.5, 1.0 + 1e-7, 1.2, 1.7, -2.0]
        ticks.append(np.asarray(t, dtype=np.float32))
    if ndim == 1:
        P = ticks[0][None]
    else:
        g = np.meshgrid(*ticks, indexing='ij')
        P = np.stack([x.reshape(-1) for x in g])
        if P.shape[1] > 6000:
            P = P[:, rng.choice(P.shape[1], 6000, replace=False)]
    # diagonals of the sub-cell split (x==y, x+y==1 inside a square)
    u = rng.random((ndim, 1500)).astype(np.float32)
    if ndim >= 2:
        s = rng.integers(0, nc[0], 1500)
        t = rng.random(1500).astype(np.float32)
        u[0, :500] = ((s[:500] + t[:500]) / nc[0]).astype(np.float32)
        u[1, :500] = ((np.floor(u[1, :500] * nc[1]) + t[:500]) / nc[1]).astype(np.float32)
        u[0, 500:1000] = ((s[500:1000] + t[500:1000]) / nc[0]).astype(np.float32)
        u[1, 500:1000] = ((np.floor(u[1, 500:1000] * nc[1]) + 1 - t[500:1000]) / nc[1]).astype(np.float32)
    u[:, 1000:] = (rng.random((ndim, 500)) * 1.6 - 0.3).astype(np.float32)
    return np.concatenate([P, u], axis=1).astype(np.float32)


def main():
    import torch
    torch.set_num_threads(min(8, os.cpu_count() or 1))
    tmp = import_reference()
    try:
        from libcpab import Cpab
        import libcpab.pytorch.findcellidx as pt_find
        import libcpab.numpy.findcellidx as np_find
        from libcpab.pytorch.expm import expm as ref_expm
        from libcpab_gb300.tessellation import make_tessellation
        from oracle.oracle import RefLib
        ref = RefLib()

        for (name, nc, zb, vp, n_theta, scale, npts, C, dsize, osize) in CONFIGS:
            print('config', name, flush=True)
            rng = np.random.default_rng(zlib.crc32(name.encode()))
            Tn = Cpab(nc, backend='numpy', device='cpu', zero_boundary=zb, volume_perservation=vp,
                      override=True)
            Tt = Cpab(nc, backend='pytorch', device='cpu', zero_boundary=zb, volume_perservation=vp)
            mine = make_tessellation(nc, zb, vp)
            L_ref, B_ref = Tn.tesselation.L, Tn.params.basis
            assert mine.L.shape == L_ref.shape and np.array_equal(mine.L, L_ref), name + ': L differs'
            assert np.array_equal(mine.B, B_ref), name + ': B differs'
            ndim = len(nc)
            d = B_ref.shape[1]
            nC = Tn.params.nC

            theta = (scale * rng.standard_normal((n_theta, d))).astype(np.float32)
            grid = Tt.uniform_meshgrid(npts).numpy().astype(np.float32)
            lo, hi = (0.0, 1.0) if zb else (-0.2, 1.2)
            grid_b = rng.uniform(lo, hi, (n_theta, ndim, grid.shape[1])).astype(np.float32)

            out_np64 = Tn.transform_grid(grid.astype(np.float64), theta.astype(np.float64))
            out_np64_b = Tn.transform_grid(grid_b.astype(np.float64), theta.astype(np.float64))

            th_t = torch.tensor(theta, requires_grad=True)
            out_t = Tt.transform_grid(torch.tensor(grid), th_t)
            cot = rng.standard_normal(out_t.shape).astype(np.float32)
            (out_t * torch.tensor(cot)).sum().backward()
            dtheta_ref = th_t.grad.numpy().copy()

            th_t2 = torch.tensor(theta, requires_grad=True)
            out_tb = Tt.transform_grid(torch.tensor(grid_b), th_t2)
            (out_tb * torch.tensor(cot)).sum().backward()
            dtheta_ref_b = th_t2.grad.numpy().copy()

            # the reference's own per-cell maps (fp32 Pade-13) and A tables
            Bf = torch.Tensor(B_ref)
            As = (Bf @ torch.tensor(theta).t()).t().reshape(n_theta * nC, ndim, ndim + 1)
            Asq = torch.cat([As, torch.zeros(n_theta * nC, 1, ndim + 1)], dim=1)
            trels = ref_expm((1.0 / 50) * Asq)[:, :ndim, :].reshape(n_theta, nC, ndim, ndim + 1).numpy()
            As = As.reshape(n_theta, nC, ndim, ndim + 1).numpy()

            # interpolation of the reference's transformed grid, fp32 and fp64 autograd
            data = rng.random((n_theta, C, *dsize)).astype(np.float32)
            gt = torch.tensor(out_t.detach().numpy())
            interp32 = Tt.interpolate(torch.tensor(data), gt, npts).numpy()
            d64 = torch.tensor(data.astype(np.float64), requires_grad=True)
            g64 = torch.tensor(gt.numpy().astype(np.float64), requires_grad=True)
            i64 = Tt.backend.interpolate(ndim, d64, g64, npts)
            icot = rng.standard_normal(i64.shape).astype(np.float32)
            (i64 * torch.tensor(icot.astype(np.float64))).sum().backward()

            # transform_data with an MSE loss against a second warp
            theta2 = (scale * rng.standard_normal((n_theta, d))).astype(np.float32)
            with torch.no_grad():
                target = Tt.transform_data(torch.tensor(data), torch.tensor(theta2), osize)
            th3 = torch.tensor(theta, requires_grad=True)
            dd = torch.tensor(data, requires_grad=True)
            td = Tt.transform_data(dd, th3, osize)
            loss = torch.nn.functional.mse_loss(td, target)
            loss.backward()

            P = probe_points(nc, rng)
            cells_cpp = ref.findcellidx(nc, P)
            cells_np = np_find.findcellidx(ndim, P.astype(np.float64), nc).astype(np.int32)
            cells_pt = pt_find.findcellidx(ndim, torch.tensor(P).clone(), nc).numpy().astype(np.int32)

            np.savez_compressed(
                os.path.join(HERE, name + '.npz'),
                nc=np.asarray(nc), zero_boundary=zb, volume_perservation=vp, nstepsolver=50,
                B=B_ref, L_sha=sha(L_ref), L_shape=np.asarray(L_ref.shape),
                theta=theta, grid=grid, grid_b=grid_b, npts=np.asarray(npts),
                out_np64=out_np64, out_np64_b=out_np64_b,
                out_cpu32=out_t.detach().numpy(), out_cpu32_b=out_tb.detach().numpy(),
                cot=cot, dtheta_ref=dtheta_ref, dtheta_ref_b=dtheta_ref_b,
                trels_ref=trels, As_ref=As,
                data=data, interp32=interp32, interp64=i64.detach().numpy(), icot=icot,
                interp64_ddata=d64.grad.numpy(), interp64_dgrid=g64.grad.numpy(),
                theta2=theta2, outsize=np.asarray(osize), td_target=target.numpy(),
                td_out=td.detach().numpy(), td_loss=loss.item(),
                td_dtheta=th3.grad.numpy(), td_ddata=dd.grad.numpy(),
                probe=P, cells_cpp=cells_cpp, cells_np=cells_np, cells_pt=cells_pt,
            )

        for (name, nc, zb, vp, keep_B) in LARGE:
            print('config', name, flush=True)
            mine = make_tessellation(nc, zb, vp)
            Tn = Cpab(nc, backend='numpy', device='cpu', zero_boundary=zb, volume_perservation=vp,
                      override=True)
            L_ref, B_ref = Tn.tesselation.L, Tn.params.basis
            assert np.array_equal(mine.L, L_ref), name + ': L differs'
            assert np.array_equal(mine.B, B_ref), name + ': B differs'
            extra = {'B': B_ref} if keep_B else {}
            np.savez_compressed(os.path.join(HERE, name + '.npz'), nc=np.asarray(nc),
                                zero_boundary=zb, volume_perservation=vp,
                                L_sha=sha(L_ref), L_shape=np.asarray(L_ref.shape),
                                B_sha=sha(B_ref), B_shape=np.asarray(B_ref.shape), **extra)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


if __name__ == '__main__':
    main()

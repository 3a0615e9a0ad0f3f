"""The exact-flow adjoint's algorithm, restated in float64 on the CPU.

k_adjoint_exact (csrc/cpab_exact.cu) integrates the flow backwards from the
forward result in certified in-cell sub-steps; per sub-step it carries the
cotangent back through the in-cell exponential and adds the adjoint Frechet
derivative to the cell's dL/dA, and a sub-step that passed a face is
corrected to first order in the time it spent on the far side.  This test
runs the same sweep in float64 (scipy's expm and expm_frechet) and checks it
against the FP64 forward sensitivities of oracle.exact_flow_grad_fp64: within
1e-5 relative with the crossing correction, and the correction must matter
(the uncorrected sweep is off by more).  The CUDA kernel itself is checked
against the same oracle in tests/test_exact_flow.py.
"""
import numpy as np
import pytest

pytest.importorskip('scipy')


def _face_distance(p, nc):
    """Distance to the face lines of p's cell (domain edges excluded): the
    1D cell ends, the 2D square sides and the two triangle diagonals."""
    ndim = len(nc)
    inc = [1.0 / n for n in nc]
    d, sub = np.inf, []
    for j in range(ndim):
        ci = min(max(np.floor(p[j] / inc[j]), 0), nc[j] - 1)
        x = p[j] / inc[j] - ci
        sub.append(x)
        if ci > 0:
            d = min(d, abs(x) * inc[j])
        if ci < nc[j] - 1:
            d = min(d, abs(1 - x) * inc[j])
    if ndim == 2:
        s = min(inc) / np.sqrt(2.0)
        d = min(d, abs(sub[0] - sub[1]) * s, abs(sub[0] + sub[1] - 1) * s)
    return d


def _reverse_sweep(B, theta, nc, end, cot, correct, overshoot=1e-5):
    from scipy.linalg import expm, expm_frechet
    from oracle.oracle import numpy_findcellidx
    ndim = len(nc)
    nC = B.shape[0] // (ndim * (ndim + 1))
    A = (B @ theta).reshape(nC, ndim, ndim + 1)
    dA = np.zeros_like(A)

    def cell(x):
        return int(numpy_findcellidx(ndim, x.reshape(ndim, 1).astype(np.float32), nc,
                                     semantics='cpp')[0])
    p, lam, tr = end.astype(np.float64), cot.astype(np.float64), 1.0
    c = cell(p)
    for _ in range(100000):
        if tr <= 0:
            break
        M = A[c]
        v = M[:, :ndim] @ p + M[:, ndim]
        reach = _face_distance(p, nc) + overshoot
        bound = np.linalg.norm(v) + np.linalg.norm(M[:, :ndim]) * reach
        dt = min(tr, reach / bound) if bound > 0 else tr
        X = np.zeros((ndim + 1, ndim + 1))
        X[:ndim] = M
        q = (expm(-dt * X) @ np.append(p, 1.0))[:ndim]
        qt = np.append(q, 1.0)
        W = np.zeros((ndim + 1, ndim + 1))
        W[:ndim] = np.outer(lam, qt)
        T, L = expm_frechet(dt * X.T, W)
        dA[c] += dt * L[:ndim]
        nl = T[:ndim, :ndim] @ lam
        cn = cell(q)
        if cn != c and correct:
            Mn = A[cn]
            gq = np.linalg.norm((M - Mn) @ qt)
            gp = np.linalg.norm((M - Mn) @ np.append(p, 1.0))
            tau = dt * gq / (gq + gp) if gq + gp > 0 else 0.0
            nl = nl + tau * (Mn[:, :ndim] - M[:, :ndim]).T @ nl
            w = tau * np.outer(nl, qt)
            dA[c] -= w
            dA[cn] += w
        p, lam, c = q, nl, cn
        tr = 0.0 if dt >= tr else tr - dt
    return B.T @ dA.reshape(-1), lam


@pytest.mark.parametrize('nc,zb,std', [([50], True, 1.0), ([3, 3], True, 0.5)])
def test_reverse_sweep_matches_sensitivities(nc, zb, std):
    from libcpab_gb300.tessellation import make_tessellation
    from oracle.oracle import exact_flow_fp64, exact_flow_grad_fp64
    B = make_tessellation(nc, zb, False).B
    rng = np.random.default_rng(3)
    theta = std * rng.standard_normal(B.shape[1])
    nP = 8
    pts = rng.random((len(nc), nP))
    cot = np.random.default_rng(4).standard_normal((1, len(nc), nP))
    end = exact_flow_fp64(B, theta[None], pts, nc)[0]
    ref_th, ref_p = exact_flow_grad_fp64(B, theta[None], pts, nc, cot)
    errs = {}
    for correct in (True, False):
        g = np.zeros(B.shape[1])
        gp = np.zeros((len(nc), nP))
        for q in range(nP):
            gq, lq = _reverse_sweep(B, theta, nc, end[:, q], cot[0][:, q], correct)
            g += gq
            gp[:, q] = lq
        errs[correct] = (np.abs(g - ref_th[0]).max() / np.abs(ref_th[0]).max(),
                         np.abs(gp - ref_p[0]).max() / np.abs(ref_p[0]).max())
    assert max(errs[True]) <= 1e-5, errs
    assert max(errs[False]) > 2 * max(errs[True]), errs

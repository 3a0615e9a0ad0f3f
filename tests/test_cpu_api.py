"""Host-side checks of the composition, alignment, ragged and exact-flow APIs
(no GPU needed), and a pin of the exact-flow FP64 oracle.

The exact-flow oracle (oracle.exact_flow_fp64) integrates the ODE of the
continuous piecewise-affine field numerically; in 1D the flow also has a
closed form (per cell x(t) = (x0 + b/a) e^{at} - b/a, with the time to reach
a cell boundary log(v(boundary)/v(x0))/a), restated here in float64.  The two
independent methods must agree to 1e-8 (the ODE tolerance).
"""
import math

import numpy as np
import pytest
import torch


def test_sequential_checks():
    from libcpab_gb300 import Cpab, CpabSequential
    T1 = Cpab([2, 2], backend='pytorch', device='gpu')
    T2 = Cpab([3, 3], backend='pytorch', device='gpu')
    T3 = Cpab([4], backend='pytorch', device='gpu')
    with pytest.raises(AssertionError):
        CpabSequential(T1, T3)                      # mixed dimensions
    with pytest.raises(AssertionError):
        CpabSequential(T1, 'not a cpab')
    S = CpabSequential(T1, T2)
    assert S.get_theta_dim() == [T1.get_theta_dim(), T2.get_theta_dim()]
    with pytest.raises(AssertionError):             # one theta per transformation
        S.transform_grid(torch.zeros(2, 5), [torch.zeros(1, T1.get_theta_dim())])
    with pytest.raises(AssertionError):             # equal batch sizes
        S._assert_theta_shape([torch.zeros(1, 3), torch.zeros(2, 3)])


def test_aligner_and_solver_checks():
    from libcpab_gb300 import Cpab, CpabAligner
    with pytest.raises(AssertionError):
        CpabAligner('not a cpab')
    T = Cpab([3, 3], backend='pytorch', device='gpu')
    assert T.params.integration == 'fixed_step' and T.params.point_gradient is False
    with pytest.raises(AssertionError):
        T.set_solver_params(integration='rk4')
    with pytest.raises(AssertionError):
        T.set_solver_params(point_gradient=1)
    T.set_solver_params(integration='exact', point_gradient=True)
    assert T.params.integration == 'exact' and T.params.point_gradient is True


def test_ragged_api_refuses_cpu_tensors():
    from libcpab_gb300 import Cpab, functions
    T = Cpab([10], backend='pytorch', device='gpu', zero_boundary=False)
    values = torch.zeros(20)
    offsets = torch.tensor([0, 8, 20])
    theta = torch.zeros(2, T.get_theta_dim())
    with pytest.raises(ValueError):
        functions.transform_data_ragged(values, offsets, theta, T.params)


def _closed_form_1d(A, x, nc):
    """Exact 1D flow for time 1 of the field v(x) = a_c x + b_c, float64."""
    inc = 1.0 / nc
    t = 1.0
    c = min(max(int(math.floor(x * nc)), 0), nc - 1)
    for _ in range(nc + 2):
        a, b = A[c]
        v = a * x + b
        if v == 0.0:
            break
        right = v > 0
        has_face = c < nc - 1 if right else c > 0
        tb = math.inf
        if has_face:
            xb = (c + 1) * inc if right else c * inc
            vb = a * xb + b
            if vb != 0.0 and (vb > 0) == right:
                tb = math.log(vb / v) / a if a != 0.0 else (xb - x) / v
        if tb >= t:
            x = x + v * (math.expm1(a * t) / a if a != 0.0 else t)
            break
        x, t, c = xb, t - tb, c + (1 if right else -1)
    return x


@pytest.mark.parametrize('nc,zb', [([20], True), ([50], False)])
def test_exact_flow_oracle_matches_closed_form_1d(nc, zb):
    from libcpab_gb300.tessellation import make_tessellation
    from oracle.oracle import exact_flow_fp64
    B = make_tessellation(nc, zb, False).B
    rng = np.random.default_rng(5)
    theta = rng.standard_normal((2, B.shape[1]))
    pts = rng.random((1, 60))
    ode = exact_flow_fp64(B, theta, pts, nc)
    for k in range(theta.shape[0]):
        A = (B @ theta[k]).reshape(nc[0], 2)
        ref = np.array([_closed_form_1d(A, float(x), nc[0]) for x in pts[0]])
        assert np.abs(ode[k, 0] - ref).max() <= 1e-8


def test_ragged_points_argument_checks():
    from libcpab_gb300 import Cpab, functions
    T = Cpab([3, 3], backend='pytorch', device='gpu')
    pts = torch.zeros(2, 20)
    off = torch.tensor([0, 8, 20])
    theta = torch.zeros(2, T.get_theta_dim())
    with pytest.raises(ValueError):                 # CPU tensors: no fallback
        functions.transform_grid_ragged(pts, off, theta, T.params)
    meta = lambda *s, **k: torch.empty(*s, device='meta', **k)
    for p, o, th in ((meta(3, 20), meta(3, dtype=torch.int64), meta(2, 4)),
                     (meta(2, 20), meta(3, dtype=torch.int32), meta(2, 4)),
                     (meta(2, 20), meta(3, dtype=torch.int64), meta(3, 4))):
        with pytest.raises(ValueError):
            functions._check_ragged_points(p, o, th, T.params)


def test_grid_axes_cached_and_equal_to_linspace():
    from libcpab_gb300 import Cpab
    from libcpab_gb300.functions import grid_axes
    T = Cpab([3, 3], backend='pytorch', device='gpu')
    a = grid_axes(T.params, (5, 7), 'cpu')
    assert grid_axes(T.params, (5, 7), 'cpu') is a
    assert torch.equal(a, torch.cat([torch.linspace(0, 1, 5), torch.linspace(0, 1, 7)]))
    assert grid_axes(T.params, (7, 5), 'cpu') is not a


def test_ints_and_cell_counts_are_reused():
    from libcpab_gb300 import _native as N
    assert N._ints([3, 3]) is N._ints((3, 3))
    assert list(N._ints([4, 2, 8])) == [4, 2, 8]

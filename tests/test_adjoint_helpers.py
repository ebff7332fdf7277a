"""Host helpers of the reverse-mode checks (dynearthsol_gb300/adjoint.py):
the fourth-order central difference the gradients are validated against,
the adjoint's directional derivative, and the seeded Gaussian random field
the adjoint workloads draw their viscosity fields from."""
import math

import numpy as np
import pytest

from dynearthsol_gb300.adjoint import adjoint_dot, fd5, grf_log10_visc, top_nodes
from dynearthsol_gb300.mesh import BOUNDZ1, box3d


def test_fd5_is_fourth_order():
    f = lambda t: math.exp(0.7 * t) + math.sin(2.0 * t)
    exact = 0.7 + 2.0
    e1 = abs(fd5(f, 0.1) - exact)
    e2 = abs(fd5(f, 0.05) - exact)
    assert e1 < 2e-4                  # ~h^4 |f^(5)| / 30
    assert 12 < e1 / e2 < 20          # halving h divides the error by ~2^4
    assert fd5(lambda t: 3 * t**3 - t + 5, 0.3) == pytest.approx(-1.0, abs=1e-12)   # exact on cubics


def test_adjoint_dot_sums_state_and_parameter_terms():
    start = {"vel": np.array([[1.0, 2.0], [3.0, 4.0]])}
    grad = {7: np.array([0.5, -1.0])}
    d = adjoint_dot(start, grad, dstate={"vel": np.ones((2, 2))}, dparams={7: np.array([2.0, 1.0])})
    assert d == 10.0 + 0.0


def test_random_field_statistics_and_seeding():
    m = box3d(20, 20, 4, 100e3, 100e3, 10e3)
    a = grf_log10_visc(m, mean=21.0, sd=0.5, corr_len=15e3, seed=3)
    b = grf_log10_visc(m, mean=21.0, sd=0.5, corr_len=15e3, seed=3)
    c = grf_log10_visc(m, mean=21.0, sd=0.5, corr_len=15e3, seed=4)
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    assert a.shape == (m.nelem,)
    # 128 random Fourier features: the sample moments scatter around the
    # requested ones by a fraction of sd
    assert abs(a.mean() - 21.0) < 0.5 and 0.2 < a.std() < 0.8


def test_random_field_is_smooth_on_its_correlation_length():
    m = box3d(40, 4, 2, 100e3, 10e3, 5e3)
    f = grf_log10_visc(m, sd=1.0, corr_len=15e3, seed=5)
    from dynearthsol_gb300.config import elem_center
    x = elem_center(m)
    near = np.linalg.norm(x[1:] - x[:-1], axis=1) < 3e3
    jumps = np.abs(np.diff(f))[near]
    assert np.median(jumps) < 0.2   # neighbours a fraction of a correlation length apart stay close


def test_top_nodes_are_the_z1_boundary():
    m = box3d(3, 2, 2, 1.0, 1.0, 1.0)
    t = top_nodes(m)
    assert len(t) == 4 * 3
    assert (m.coord[t, 2] == 0.0).all() and ((m.bcflag[t] & BOUNDZ1) != 0).all()

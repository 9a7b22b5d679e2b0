"""Properties of the oracle that hold for every path the golden vectors do not
cover (characteristic projection, HLLC star-right branch, sensor blend)."""

import numpy as np
import pytest

from states import noisy, quadrant, smooth

G = 1.4


@pytest.mark.parametrize("cons", [False, True])
@pytest.mark.parametrize("hlle", [False, True])
def test_free_stream_is_steady(orc, cons, hlle):
    q = np.zeros((14, 12, 8))
    rho, u, v, p = 1.3, 0.4, -0.7, 0.9
    q[..., 0], q[..., 1], q[..., 2] = rho, rho * u, rho * v
    q[..., 3] = p / (G - 1) + 0.5 * rho * (u * u + v * v)
    L = orc.l_local_py(q, 0.1, G, hlle, (0.2, 1.0), cons)
    assert np.abs(L).max() < 1e-12


@pytest.mark.parametrize("cons", [False, True])
@pytest.mark.parametrize("hlle", [False, True])
def test_transpose_symmetry(orc, cons, hlle):
    """Swapping the axes and the momentum components maps x fluxes onto y fluxes."""
    rng = np.random.default_rng(3)
    q = quadrant(rng, 11, 11)
    qt = np.ascontiguousarray(q.transpose(1, 0, 2)[:, :, [0, 2, 1, 3]])
    L = orc.l_local_py(q, 0.05, G, hlle, (0.1, 0.6), cons)
    Lt = orc.l_local_py(qt, 0.05, G, hlle, (0.1, 0.6), cons)
    back = Lt.transpose(1, 0, 2)[:, :, [0, 2, 1, 3]]
    np.testing.assert_allclose(back, L, rtol=1e-12, atol=1e-12)


def test_characteristic_equals_componentwise_for_linear_data_at_unit_density(orc):
    """On data linear in x the WENO weights are the linear ones, so the reconstruction
    commutes with a constant projection.  With rho == 1 the reference's left and right
    eigenvector matrices are inverse to each other, and both variants agree."""
    m, n = 14, 11
    q = np.zeros((m, n, 4))
    x = np.arange(m)[:, None] * np.ones((1, n))
    q[..., 0] = 1.0
    q[..., 1] = 0.2 + 0.003 * x
    q[..., 2] = -0.1 + 0.002 * x
    q[..., 3] = 2.5 + 0.02 * x
    a = orc.weno_x_py(q, G, cons=False)
    b = orc.weno_x_py(q, G, cons=True)
    for x1, x2 in zip(a, b):
        np.testing.assert_allclose(x1, x2, rtol=1e-9, atol=1e-12)


def test_reference_eigenvectors_are_not_inverse_off_unit_density(orc):
    """weno.rs:88,103 use 0.5/(rho*c) where the conserved-variable inverse of the right
    eigenvectors (weno.rs:113-131) has 0.5/c, so L*R != I unless rho == 1.  The oracle keeps
    the reference's matrices; at rho != 1 the characteristic reconstruction of linear data
    therefore differs from the component-wise one."""
    m, n = 14, 11
    q = np.zeros((m, n, 4))
    x = np.arange(m)[:, None] * np.ones((1, n))
    q[..., 0] = 1.0 + 0.01 * x
    q[..., 1] = 0.2 + 0.003 * x
    q[..., 2] = -0.1 + 0.002 * x
    q[..., 3] = 2.5 + 0.02 * x
    a = orc.weno_x_py(q, G, cons=False)[0]
    b = orc.weno_x_py(q, G, cons=True)[0]
    assert np.abs(a[..., 0] - b[..., 0]).max() < 1e-12  # density row of R*L is exact
    assert np.abs(a[..., 1] - b[..., 1]).max() > 1e-3


def test_conservation_under_periodic_like_flux(orc):
    """The residual is a flux difference: its interior sum equals the boundary flux balance."""
    rng = np.random.default_rng(5)
    q = smooth(rng, 20, 18)
    dx = 0.1
    L = orc.l_local_py(q, dx, G, True, (0.2, 1.0), True)
    ql, fl, qr, fr = orc.weno_x_py(q, G, cons=True)
    Fx = orc.hlle_x_rs_py(ql, fl, qr, fr, G)
    ql, fl, qr, fr = orc.weno_y_py(q, G, cons=True)
    Fy = orc.hlle_y_rs_py(ql, fl, qr, fr, G)
    total = -(Fx[-1].sum(0) - Fx[0].sum(0) + Fy[:, -1].sum(0) - Fy[:, 0].sum(0)) / dx
    np.testing.assert_allclose(L.sum((0, 1)), total, rtol=1e-10, atol=1e-9)


def test_rejects_small_arrays(orc):
    with pytest.raises(ValueError):
        orc.l_local_py(np.zeros((5, 9, 4)) + 1, 0.1, G, True, (0.2, 1), True)
    with pytest.raises(ValueError):
        orc.l_local_py(np.ones((7, 9, 4)), 0.1, G, False, (0.2, 1), True)


def test_flop_tally_is_stable(orc):
    """Algorithmic operation counts per interior cell for each residual variant."""
    rng = np.random.default_rng(9)
    q = noisy(rng, 22, 22)
    per = {}
    for cons in (False, True):
        for hlle in (False, True):
            t = orc.count_l_local(q, 0.1, G, hlle, (0.2, 1.0), cons)
            cells = 16 * 16
            per[(cons, hlle)] = sum(t.values()) / cells
            assert t["div"] > 0 and t["sqrt"] > 0
    # characteristic reconstruction costs more than component-wise
    assert per[(False, True)] > per[(True, True)]


def test_reference_characteristic_scheme_is_unstable_on_low_density_quadrants(orc):
    """With the reference's eigenvectors (L*R != I off rho = 1) the characteristic
    reconstruction is not consistent, and on four-quadrant data with a rho ~ 0.11
    quadrant the reference algorithm produces NaN within a few steps at CFL 0.5, while
    the component-wise reconstruction and CFL 0.1 stay finite.  The GPU exact path
    reproduces this bit for bit (tests/test_gpu_solver.py)."""
    from states import quadrant
    q = quadrant(np.random.default_rng(9), 40, 56)
    orc.bc_transmissive(q)
    orc.sync_primitives(q, G)

    def first_nan(cfl, cons, steps=12):
        qq = q.copy()
        for k in range(steps):
            dt = cfl / 56 / orc.cfl_cmax(qq, 40, 56, G)
            orc.rk3_step(qq, 40, 56, 1 / 56, dt, G, True, (1e4, 1.1e4), cons)
            if np.isnan(qq).any():
                return k + 1
        return None

    assert first_nan(0.5, False) is not None and first_nan(0.5, False) <= 3
    assert first_nan(0.5, True) is None
    assert first_nan(0.1, False) is None

"""The identities the FAST FP64 forms rest on, checked on the oracle (the
reference's own arithmetic, weno.rs / riemann.rs restated) on the CPU.

* WENO5 and the Gauss-point WENO are homogeneous of degree one when the
  smoothness epsilon scales with the square of the field: reconstructing
  k f with eps k^2 gives k times the reconstruction of f.  For a power of two
  k every operation commutes with the scaling, so the component-wise faces
  agree bit for bit; for other k to rounding.  The FAST characteristic pass 1
  carries the shear field as rho w2 with eps rho^2 on this identity.
* The candidate polynomials of WENO5 less six times the centre value are the
  difference forms the FAST kernels evaluate (left 4 d2 - d3, d1 + 2 d2,
  5 d1 - 2 d0; right their mirror images), exact on integer data.
* HLLE is homogeneous of degree one in (states, fluxes) while the clamps do not
  bind: the FAST pass 2 feeds it the Gauss-point sums (twice the averages)
  and halves the result.
"""

import numpy as np
import pytest

from states import noisy

G = 1.4


@pytest.fixture
def eps_guard(orc):
    yield orc
    orc.set_weno_eps(1e-12)


@pytest.mark.parametrize("ydir", [False, True], ids=["x", "y"])
def test_weno_homogeneous_power_of_two_bit_exact(eps_guard, ydir):
    orc = eps_guard
    rng = np.random.default_rng(41)
    q = np.ascontiguousarray(noisy(rng, 22, 19)[:, :, :4])
    rec = orc.weno_y_py if ydir else orc.weno_x_py
    orc.set_weno_eps(1e-12)
    ql, _, qr, _ = rec(q, G, cons=True)
    for k in (4.0, 0.125):
        orc.set_weno_eps(1e-12 * k * k)
        qlk, _, qrk, _ = rec(q * k, G, cons=True)
        assert np.array_equal(qlk, ql * k) and np.array_equal(qrk, qr * k)


def test_weno_homogeneous_general_factor(eps_guard):
    orc = eps_guard
    rng = np.random.default_rng(42)
    q = np.ascontiguousarray(noisy(rng, 20, 20)[:, :, :4])
    orc.set_weno_eps(1e-12)
    ql, _, qr, _ = orc.weno_x_py(q, G, cons=True)
    for k in (1.37, 0.23, 11.5):
        orc.set_weno_eps(1e-12 * k * k)
        qlk, _, qrk, _ = orc.weno_x_py(q * k, G, cons=True)
        for a, b in ((qlk, ql * k), (qrk, qr * k)):
            assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()


def _candidates(u):
    """The reference's WENO5 candidates (x6) of the left state at the face between
    u2 and u3 (weno.rs:214-233) and of the right state (weno.rs:238-257)."""
    u0, u1, u2, u3, u4, u5 = u
    left = (-u4 + 5 * u3 + 2 * u2, -u1 + 5 * u2 + 2 * u3, 2 * u0 - 7 * u1 + 11 * u2)
    right = (2 * u5 - 7 * u4 + 11 * u3, -u4 + 5 * u3 + 2 * u2, -u1 + 5 * u2 + 2 * u3)
    return left, right


def test_slope_form_candidates_exact():
    rng = np.random.default_rng(43)
    u = rng.integers(-10 ** 6, 10 ** 6, size=(6, 5000)).astype(np.float64)
    d = np.diff(u, axis=0)  # d_m = u_{m+1} - u_m
    (pl0, pl1, pl2), (pr0, pr1, pr2) = _candidates(u)
    sl0, sl1, sl2 = d[3] - 3 * d[2], d[1] + d[2], 3 * d[1] - d[0]
    sr0, sr1, sr2 = d[4] - 3 * d[3], d[2] + d[3], 3 * d[2] - d[1]
    # left, stencils 2-4, 1-3, 0-2, about 6 u2
    assert np.array_equal(pl0 - 6 * u[2], d[2] - sl0)
    assert np.array_equal(pl1 - 6 * u[2], sl1 + d[2])
    assert np.array_equal(pl2 - 6 * u[2], 2 * sl2 - d[1])
    # right, stencils 3-5, 2-4, 1-3, about 6 u3 (the mirror images)
    assert np.array_equal(pr0 - 6 * u[3], 2 * sr0 + d[3])
    assert np.array_equal(pr1 - 6 * u[3], -d[2] - sr1)
    assert np.array_equal(pr2 - 6 * u[3], -d[2] - sr2)


@pytest.mark.parametrize("ydir", [False, True], ids=["x", "y"])
def test_hlle_homogeneous_in_states_and_fluxes(orc, ydir):
    rng = np.random.default_rng(44 + ydir)
    q = np.ascontiguousarray(noisy(rng, 24, 18)[:, :, :4])
    ql, fl, qr, fr = (orc.weno_y_py if ydir else orc.weno_x_py)(q, G, cons=True)
    hlle = orc.hlle_y_rs_py if ydir else orc.hlle_x_rs_py
    half = hlle(ql, fl, qr, fr, G)
    twice = hlle(2 * ql, 2 * fl, 2 * qr, 2 * fr, G)
    assert np.abs(0.5 * twice - half).max() <= 1e-13 * np.abs(half).max()

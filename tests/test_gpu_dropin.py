"""Parity of the twelve drop-in functions (CUDA, through the C ABI) with the CPU
oracle.  Exact mode must be bit-identical; fast mode agrees to 1e-11 of the
largest magnitude per array (the tolerance for one call)."""

import numpy as np
import pytest

from states import noisy, quadrant, smooth

pytestmark = pytest.mark.gpu
G = 1.4
FAST_TOL = 1e-11
# Near-vacuum cells (rho = 1e-13) make the Roe-averaged eigenvector matrices
# ill-conditioned (entries ~ 1/(rho*c)), which amplifies the last-bit differences
# of the fast forms; exact mode stays bit-identical there too.
FAST_TOL_VACUUM = 1e-6


@pytest.fixture(params=["exact", "fast"])
def mode(wx, request):
    wx.set_mode(request.param)
    yield request.param
    wx.set_mode("exact")


def check(got, ref, mode, what="", tol=FAST_TOL):
    got = np.asarray(got)
    ref = np.asarray(ref)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    if mode == "exact":
        bad = ~((got == ref) | (np.isnan(got) & np.isnan(ref)))
        assert not bad.any(), f"{what}: {bad.sum()} of {bad.size} differ, max {np.nanmax(np.abs(got - ref))}"
    else:
        scale = np.nanmax(np.abs(ref)) if ref.size else 1.0
        err = np.nanmax(np.abs(got - ref)) if ref.size else 0.0
        assert err <= tol * max(scale, 1e-300), f"{what}: {err} vs scale {scale}"


def vacuum(rng, m, n):
    q = noisy(rng, m, n)
    q[rng.random((m, n)) < 0.15, 0] = 1e-13  # near-vacuum cells: floors, guards and pp_limit
    q[rng.random((m, n)) < 0.1, 3] = 1e-14
    return q


def tol_for(state):
    return FAST_TOL_VACUUM if state == "vacuum" else FAST_TOL


def skip_ill_conditioned(mode, state, cons, hlle=True):
    """Near vacuum, the characteristic projection (entries ~ 1/(rho*c), results ~ 1e70 in the
    reference itself) and the sensor's hard 0/1 switch turn last-bit differences into O(1)
    ones, so only exact mode -- bit-identical there as everywhere -- is compared.  At 1e22
    and 1e40 the reference's characteristic projection is not scale invariant either (its
    left eigenvectors carry 0.5/(rho c), so L R differs from the identity by a factor of
    order rho): exact(1e40 q)/1e40 differs from exact(q) by O(1), and fast arithmetic is
    compared there on the component-wise path only."""
    if mode == "fast" and state == "vacuum" and (not cons or not hlle):
        pytest.skip("fast arithmetic is not compared on ill-conditioned near-vacuum states")
    if mode == "fast" and state in ("huge", "large") and not cons:
        pytest.skip("fast arithmetic is not compared on the characteristic path at 1e22 and 1e40")


def huge(rng, m, n):
    """Cell-wise random states with every conserved value scaled by 1e40 (same
    velocities and sound speeds, pressures x 1e40): smoothness indicators near
    1e80, outside the range where the fast WENO weights skip their power-of-two
    rescaling."""
    return noisy(rng, m, n) * 1e40


def large(rng, m, n):
    """Every conserved value scaled by 1e22: smoothness indicators near 1e44
    (about 2^146), inside the range where the fast WENO5 weights skip their
    rescaling but where the eighth-power product of the Gauss-point weights
    would overflow without its own, narrower, range."""
    return noisy(rng, m, n) * 1e22


STATES = {
    "quad": lambda rng, m, n: quadrant(rng, m - 6, n - 6),
    "smooth": lambda rng, m, n: smooth(rng, m, n),
    "noisy": lambda rng, m, n: noisy(rng, m, n),
    "vacuum": vacuum,
    "huge": huge,
    "large": large,
}
SHAPES = [(8, 8), (13, 22), (31, 17)]


@pytest.mark.parametrize("state", list(STATES))
@pytest.mark.parametrize("shape", SHAPES)
def test_flux_and_con2primi(wx, orc, mode, state, shape):
    q = STATES[state](np.random.default_rng(1), *shape)
    t = tol_for(state)
    check(wx.flux_x_py(q, G), orc.flux_x_py(q, G), mode, "flux_x", t)
    check(wx.flux_y_py(q, G), orc.flux_y_py(q, G), mode, "flux_y", t)
    for got, ref, nm in zip(wx.con2primi_py(q, G), orc.con2primi_py(q, G), "p a rho u v h".split()):
        check(got, ref, mode, nm, t)


@pytest.mark.parametrize("state", list(STATES))
@pytest.mark.parametrize("shape", SHAPES + [(6, 6)])
@pytest.mark.parametrize("cons", [False, True])
def test_reconstruction(wx, orc, mode, state, shape, cons):
    skip_ill_conditioned(mode, state, cons)
    q = STATES[state](np.random.default_rng(2), *shape)
    for ydir, fw, fo in ((0, wx.weno_x_py, orc.weno_x_py), (1, wx.weno_y_py, orc.weno_y_py)):
        for got, ref, nm in zip(fw(q, G, cons=cons), fo(q, G, cons=cons), ("q_l", "f_l", "q_r", "f_r")):
            check(got, ref, mode, f"{nm} y={ydir}", tol_for(state))


def test_reconstruction_default_is_characteristic(wx, orc):
    q = quadrant(np.random.default_rng(4), 10, 9)
    for got, ref in zip(wx.weno_x_py(q, G), orc.weno_x_py(q, G, cons=False)):
        check(got, ref, "exact")


@pytest.mark.parametrize("state", list(STATES))
@pytest.mark.parametrize("ydir", [0, 1])
def test_riemann_solvers(wx, orc, mode, state, ydir):
    q = STATES[state](np.random.default_rng(3), 24, 19)
    faces = (orc.weno_y_py if ydir else orc.weno_x_py)(q, G, cons=True)
    # plus supersonic faces so every HLLC / HLLE branch is taken
    fast = faces[0].copy()
    fast[::3, :, 1] *= 6.0
    fast[1::3, :, 2] *= -6.0
    for ql, fl, qr, fr in (faces, (fast, faces[1], faces[2], faces[3])):
        xs = "y" if ydir else "x"
        ow = {n: getattr(wx, n.replace("?", xs)) for n in ("hllc_?_rs_py", "hlle_?_rs_py", "hllc_hlle_?_rs_py")}
        oo = {n: getattr(orc, n.replace("?", xs)) for n in ("hllc_?_rs_py", "hlle_?_rs_py", "hllc_hlle_?_rs_py")}
        t = tol_for(state)
        check(ow["hllc_?_rs_py"](ql, fl, qr, fr, G), oo["hllc_?_rs_py"](ql, fl, qr, fr, G), mode, "hllc", t)
        check(ow["hlle_?_rs_py"](ql, fl, qr, fr, G), oo["hlle_?_rs_py"](ql, fl, qr, fr, G), mode, "hlle", t)
        for jp in ((0.05, 0.4), (1e4, 1.1e4), (0.0, 1e-9)):
            for fh in (False, True):
                check(ow["hllc_hlle_?_rs_py"](ql, fl, qr, fr, G, jp[0], jp[1], fh),
                      oo["hllc_hlle_?_rs_py"](ql, fl, qr, fr, G, jp[0], jp[1], fh), mode, f"blend {jp} {fh}", t)


@pytest.mark.parametrize("state", list(STATES))
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("cons", [False, True])
@pytest.mark.parametrize("hlle", [False, True])
def test_l_local(wx, orc, mode, state, shape, cons, hlle):
    skip_ill_conditioned(mode, state, cons, hlle)
    q = STATES[state](np.random.default_rng(5), *shape)
    jp = (0.05, 0.4)
    check(wx.l_local_py(q, 0.01, G, hlle, jp, cons), orc.l_local_py(q, 0.01, G, hlle, jp, cons), mode, "L",
          tol_for(state))


def test_l_local_minimal_and_empty(wx, orc):
    rng = np.random.default_rng(6)
    q = noisy(rng, 6, 6)
    check(wx.l_local_py(q, 0.1, G, True, (0.2, 1), True), orc.l_local_py(q, 0.1, G, True, (0.2, 1), True), "exact")
    assert wx.l_local_py(q, 0.1, G, True, (0.2, 1), False).shape == (0, 0, 4)
    q = noisy(rng, 7, 9)
    check(wx.l_local_py(q, 0.1, G, True, (0.2, 1), False), orc.l_local_py(q, 0.1, G, True, (0.2, 1), False), "exact")


def test_torch_inputs_and_strides(wx, orc):
    import torch
    rng = np.random.default_rng(7)
    big = quadrant(rng, 30, 26)
    t = torch.from_numpy(big).cuda()
    view = t[2:-1, 1:-3, :]  # non-contiguous rows, 8 channels
    ref_in = np.ascontiguousarray(big[2:-1, 1:-3, :])
    L = wx.l_local_py(view, 0.02, G, False, (0.05, 0.4), False)
    assert isinstance(L, torch.Tensor) and L.is_cuda
    check(L.cpu().numpy(), orc.l_local_py(ref_in, 0.02, G, False, (0.05, 0.4), False), "exact")
    got = wx.weno_y_py(view, G)
    for g, r in zip(got, orc.weno_y_py(ref_in, G)):
        check(g.cpu().numpy(), r, "exact")
    # channel-sliced numpy input with 4 channels of an 8-channel array
    q4 = big[:, :, :4]
    check(wx.l_local_py(q4, 0.02, G, True, (0.2, 1), True), orc.l_local_py(q4, 0.02, G, True, (0.2, 1), True), "exact")


def test_inputs_are_not_modified(wx):
    q = quadrant(np.random.default_rng(8), 12, 12)
    keep = q.copy()
    wx.l_local_py(q, 0.1, G, False, (0.05, 0.4), False)
    wx.weno_x_py(q, G)
    wx.con2primi_py(q, G)
    assert np.array_equal(q, keep)


def test_matches_golden_twin(wx, golden_twin):
    for case in ("quad", "smooth", "quad8"):
        u = golden_twin[f"{case}/u"]
        for got, tag in zip(wx.weno_x_py(u, G, cons=True), ("qlx", "flx", "qrx", "frx")):
            check(got, golden_twin[f"{case}/{tag}"], "exact", tag)
        dx = float(golden_twin[f"{case}/dx"])
        check(wx.l_local_py(u, dx, G, True, (0.2, 1.0), True), golden_twin[f"{case}/L_hlle"], "exact", "L")


def test_errors(wx):
    with pytest.raises(TypeError):
        wx.l_local_py(np.ones((10, 10, 8), dtype=np.float32), 0.1, G, True, (0.2, 1), True)
    with pytest.raises(TypeError):
        wx.flux_x_py(np.ones((10, 10)), G)
    with pytest.raises(ValueError):
        wx.l_local_py(np.ones((5, 10, 8)), 0.1, G, True, (0.2, 1), True)
    with pytest.raises(ValueError):
        wx.l_local_py(np.ones((7, 10, 8)), 0.1, G, False, (0.2, 1), True)
    with pytest.raises(ValueError):
        wx.flux_x_py(np.ones((10, 10, 3)), G)
    with pytest.raises(ValueError):
        wx.hllc_hlle_x_rs_py(*[np.ones((1, 5, 4))] * 4, G, 0.1, 0.2, False)


def _signed_nan(sign):
    return np.array([0x7FF8000000000000 if sign > 0 else 0xFFF8000000000000], dtype=np.uint64).view(np.float64)[0]


@pytest.mark.parametrize("sign", [1, -1], ids=["+nan", "-nan"])
@pytest.mark.parametrize("cons", [False, True], ids=["char", "cons"])
def test_nan_density_residual(wx, orc, sign, cons):
    """A NaN density with either sign bit.  Exact mode reproduces the oracle bit for bit,
    NaN positions included (the reference's f64::max clamps turn some NaN faces into finite
    values).  FAST mode's integer-bit clamps let a NaN with the sign bit clear through where
    f64::max returns the bound, so FAST outputs may hold NaN where exact ones are finite,
    never the reverse on the characteristic path, where the projection spreads the NaN
    to all four fields: there the NaN cell's residual is NaN in both modes."""
    q = quadrant(np.random.default_rng(12), 24, 20)
    q[14, 11, 0] = _signed_nan(sign)
    ref = orc.l_local_py(q, 1.0 / 24, G, True, (0.2, 1.0), cons)
    wx.set_mode("exact")
    try:
        got = wx.l_local_py(q, 1.0 / 24, G, True, (0.2, 1.0), cons)
        check(got, ref, "exact", "l_local exact")
        wx.set_mode("fast")
        fast = wx.l_local_py(q, 1.0 / 24, G, True, (0.2, 1.0), cons)
    finally:
        wx.set_mode("exact")
    if not cons:
        assert np.isnan(ref[11, 8]).all() and np.isnan(fast[11, 8]).all()
        assert not (np.isnan(ref) & ~np.isnan(fast)).any()
    fin = np.isfinite(fast) & np.isfinite(ref)
    far = np.ones(ref.shape[:2], dtype=bool)
    far[11 - 4:11 + 5, 8 - 4:8 + 5] = False  # cells whose stencils reach the NaN cell
    assert fin[far].all()
    check(fast[far], ref[far], "fast", "l_local fast away from the NaN cell")


@pytest.mark.parametrize("sign", [1, -1], ids=["+nan", "-nan"])
@pytest.mark.parametrize("smode", ["exact", "fast"])
def test_nan_density_stops_the_solver(wx, orc, sign, smode):
    """The driver's CFL divides by np.maximum(rho, 1e-14), which is NaN for a NaN density,
    so dt and the whole next state are NaN (Rie_prob_2d_rs.py:311-319).  The solver does
    the same in both modes, and reports it (status bit 1, non-finite wave speed)."""
    q = quadrant(np.random.default_rng(13), 24, 20)
    q[14, 11, 0] = _signed_nan(sign)
    assert np.isnan(orc.cfl_cmax(q, 24, 20, G))
    s = wx.Solver(24, 20, 1.0 / 24, G, mode=smode, cons=False, force_hlle=True, cfl=0.45)
    s.set_state(q)
    s.run(1)
    t, n, st = s.info()
    assert st & 1
    assert np.isnan(s.state()[3:-3, 3:-3, :4]).all()
    s.close()


@pytest.mark.parametrize("ydir", [0, 1], ids=["x", "y"])
def test_fast_riemann_on_mirror_faces(wx, orc, ydir):
    """At a reflecting wall the two face states are mirror images (normal momentum
    negated).  Where the energy has gone negative the Roe sound speed is zero, and the
    reference flux switches from F_L to F_R with the sign of the Roe-averaged normal
    velocity, which its arithmetic makes exactly +0.0.  FAST mode must land on the same
    side: every solver agrees with the oracle to the one-call tolerance."""
    rng = np.random.default_rng(21 + ydir)
    m, n = 16, 24
    ql = np.ascontiguousarray(noisy(rng, m, n)[:, :, :4])
    ql[rng.random((m, n)) < 0.4, 3] *= -1.0  # negative energy: zero Roe sound speed
    qr = ql.copy()
    qr[:, :, 2 if ydir else 1] *= -1.0
    flux = orc.flux_y_py if ydir else orc.flux_x_py
    fl, fr = flux(ql, G), flux(qr, G)
    solvers = ((wx.hlle_y_rs_py, orc.hlle_y_rs_py), (wx.hllc_y_rs_py, orc.hllc_y_rs_py)) if ydir else \
              ((wx.hlle_x_rs_py, orc.hlle_x_rs_py), (wx.hllc_x_rs_py, orc.hllc_x_rs_py))
    wx.set_mode("fast")
    try:
        for fw, fo in solvers:
            check(fw(ql, fl, qr, fr, G), fo(ql, fl, qr, fr, G), "fast", fw.__name__)
        bw = wx.hllc_hlle_y_rs_py if ydir else wx.hllc_hlle_x_rs_py
        bo = orc.hllc_hlle_y_rs_py if ydir else orc.hllc_hlle_x_rs_py
        check(bw(ql, fl, qr, fr, G, 0.05, 0.4, False), bo(ql, fl, qr, fr, G, 0.05, 0.4, False), "fast", "blend")
    finally:
        wx.set_mode("exact")


@pytest.mark.parametrize("cons", [True], ids=["cons"])
def test_fast_reconstruction_mirror_exact(wx, cons):
    """Mirror-image stencils (the reflecting wall): FAST's left and right face states of
    a face whose six cells are mirror images are themselves exact mirrors (normal
    momentum negated), as the reference's arithmetic makes them."""
    rng = np.random.default_rng(33)
    m, n = 12, 10
    half = noisy(rng, m, n // 2)
    q = np.concatenate([half[:, ::-1], half], axis=1)  # columns j and n-1-j mirror each other
    q[:, : n // 2, 2] *= -1.0  # the normal (y) momentum flips across the wall
    q = np.ascontiguousarray(q)
    wx.set_mode("fast")
    try:
        ql, fl, qr, fr = wx.weno_y_py(q, G, cons=cons)
    finally:
        wx.set_mode("exact")
    # the wall face is face column n//2 - 3 of the (m-6, n-5) face arrays
    c = n // 2 - 3
    sign = np.array([1.0, 1.0, -1.0, 1.0])
    assert np.array_equal(ql[:, c, :], qr[:, c, :] * sign)

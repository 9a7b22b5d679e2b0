"""The CPU oracle against golden vectors made by the reference's own Python code
(tests/golden/make_golden.py): the numpy twin WENO_HLLC_2d.py for the
component-wise + HLLE path and the drivers for BC fills, RK3 and CFL.  Every
comparison is bit-exact."""

import numpy as np
import pytest

CASES = ["quad", "smooth", "quad8"]
G = 1.4


def same(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape
    assert np.array_equal(a, b), f"max |diff| = {np.nanmax(np.abs(a - b))}"


@pytest.mark.parametrize("case", CASES)
def test_reconstruct_cons_matches_twin(orc, golden_twin, case):
    u = golden_twin[f"{case}/u"]
    ql, fl, qr, fr = orc.weno_x_py(u, G, cons=True)
    for got, tag in ((ql, "qlx"), (fl, "flx"), (qr, "qrx"), (fr, "frx")):
        same(got, golden_twin[f"{case}/{tag}"])
    ql, fl, qr, fr = orc.weno_y_py(u, G, cons=True)
    for got, tag in ((ql, "qly"), (fl, "fly"), (qr, "qry"), (fr, "fry")):
        same(got, golden_twin[f"{case}/{tag}"])


@pytest.mark.parametrize("case", CASES)
def test_flux_con2primi_match_twin(orc, golden_twin, case):
    u = golden_twin[f"{case}/u"]
    same(orc.flux_x_py(u, G), golden_twin[f"{case}/flux_x"])
    same(orc.flux_y_py(u, G), golden_twin[f"{case}/flux_y"])
    p, a, rho, uu, vv, h = orc.con2primi_py(u, G)
    for got, tag in ((p, "p"), (a, "a"), (rho, "rho"), (uu, "uu"), (vv, "vv")):
        same(got, golden_twin[f"{case}/c2p_{tag}"])
    same(h, (u[:, :, 3] + p) / rho)


@pytest.mark.parametrize("case", CASES)
def test_riemann_matches_twin(orc, golden_twin, case):
    u = golden_twin[f"{case}/u"]
    qlx, flx, qrx, frx = orc.weno_x_py(u, G, cons=True)
    qly, fly, qry, fry = orc.weno_y_py(u, G, cons=True)
    same(orc.hlle_x_rs_py(qlx, flx, qrx, frx, G), golden_twin[f"{case}/hlle_x"])
    same(orc.hlle_y_rs_py(qly, fly, qry, fry, G), golden_twin[f"{case}/hlle_y"])
    # The twin's HLLC differs from the Rust one only in the star-right branch.
    mx = golden_twin[f"{case}/hllc_x_mask"]
    my = golden_twin[f"{case}/hllc_y_mask"]
    assert mx.mean() > 0.2 and my.mean() > 0.2
    same(orc.hllc_x_rs_py(qlx, flx, qrx, frx, G)[mx], golden_twin[f"{case}/hllc_x"][mx])
    same(orc.hllc_y_rs_py(qly, fly, qry, fry, G)[my], golden_twin[f"{case}/hllc_y"][my])


@pytest.mark.parametrize("case", CASES)
def test_sensor_and_residual_match_twin(orc, golden_twin, case):
    same(orc.shock_sensor(golden_twin[f"{case}/sensor_pbar_x"], 0.05, 0.4), golden_twin[f"{case}/sensor_x"])
    u = golden_twin[f"{case}/u"]
    dx = float(golden_twin[f"{case}/dx"])
    same(orc.l_local_py(u, dx, G, True, (0.2, 1.0), True), golden_twin[f"{case}/L_hlle"])


def test_bc_fills_match_drivers(orc, golden_drivers):
    g = golden_drivers
    a = g["bc/rand"].copy()
    same(orc.bc_transmissive(a), g["bc/zero_gradient"])
    a = g["bc/rand_sq"].copy()
    same(orc.bc_reflecting(a), g["bc/reflecting"])
    for bnd in (3, 9, 30, 40):
        a = g["bc/rand_dmr"].copy()
        same(orc.bc_dmr(a, 40, 10, bnd), g[f"bc/dmr_{bnd}"])


def test_rk3_step_matches_driver(orc, golden_drivers):
    q = golden_drivers["rk3/q_in"].copy()
    orc.rk3_step(q, 13, 10, 0.05, 1e-3, G, True, (0.2, 1.0), True)
    same(q, golden_drivers["rk3/q_out"])


def _run(orc, q, nx, ny, dx, cfl, nstep, t_final=None, bc="transmissive", bound=0, jp=(0.5, 2)):
    T, step = 0.0, 0
    while (t_final is None and step < nstep) or (t_final is not None and T < t_final - 1e-12 and step < nstep):
        dt = cfl * dx / orc.cfl_cmax(q, nx, ny, G)
        if t_final is not None:
            dt = min(dt, t_final - T)
        orc.rk3_step(q, nx, ny, dx, dt, G, True, jp, True, bc=bc, bound=bound)
        T += dt
        step += 1
    return q


def test_driver_runs_match(orc, golden_drivers):
    g = golden_drivers
    same(_run(orc, g["rie/q0"].copy(), 16, 16, 1 / 16, 0.3, 3), g["rie/q_nstep3"])
    same(_run(orc, g["rie/q0"].copy(), 16, 16, 1 / 16, 0.3, 50, t_final=0.02), g["rie/q_tfinal"])
    same(_run(orc, g["dmr/q0"].copy(), 40, 10, 0.1, 0.1, 4, t_final=0.01, bc="dmr", bound=int(g["dmr/bound"]),
              jp=(10000, 11000)), g["dmr/q_final"])

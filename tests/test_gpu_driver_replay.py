"""The unchanged reference drivers, call by call, on this package.

``Rie_prob_2d_rs.main_rs`` (rk3_cc: six-argument l_local_py, con2primi_py in
_sync_primitives) and ``double_mach_reflection.main_rs`` (rk3_refac:
five-argument l_local_py with cons_switch at its default, con2primi_py) were run
with a recording weno_ext (tests/golden/make_driver_trace.py).  Here the same
loop runs with this package as weno_ext, numpy arrays in and out as the drivers
pass them, in exact mode: every input must equal the driver's (digest), every
output the recorded one, and the final array the one main_rs returned -- 64^2
four-quadrant runs of 10 steps in the component-wise + HLLE (identical to the
reference's own numpy twin), characteristic + HLLE and characteristic + blend
schemes, and a 128 x 32 oblique-shock run of 10 steps (characteristic + HLLC).
"""

import pytest

import driver_replay

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("run", ["rie_cons_hlle", "rie_char_hlle", "rie_char_blend", "dmr_char_hllc"])
def test_driver_runs_unchanged_on_package(wx, run):
    wx.set_mode("exact")
    z, meta = driver_replay.load_trace()
    q, ncalls = driver_replay.replay(wx, run)
    assert ncalls == len(meta[run]["calls"])

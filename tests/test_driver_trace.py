"""The recorded calls of the unchanged reference drivers (tests/golden/driver_trace.npz)
against the oracle, on the CPU: the replay loop reproduces every recorded input digest
and the oracle every output digest, and a one-ulp change in a residual is caught."""

import types

import numpy as np
import pytest

import driver_replay

RUNS = ("rie_cons_hlle", "rie_char_hlle", "rie_char_blend", "dmr_char_hllc")


@pytest.mark.parametrize("run", RUNS)
def test_oracle_replays_driver_trace(orc, run):
    z, meta = driver_replay.load_trace()
    q, ncalls = driver_replay.replay(orc, run)
    assert ncalls == len(meta[run]["calls"]) >= 40
    assert np.isfinite(q[:, :, :4]).all()


def test_trace_call_forms():
    """The drivers call l_local_py with six positional arguments (rk3_cc) and with five
    (rk3_refac, cons_switch left at its default), and con2primi_py with two."""
    z, meta = driver_replay.load_trace()
    forms = {(c["fn"], c["npos"]) for run in RUNS for c in meta[run]["calls"]}
    assert forms == {("l_local_py", 6), ("l_local_py", 5), ("con2primi_py", 2)}


def test_replay_detects_one_ulp(orc):
    """A module whose residual differs by one ulp in one element fails the replay."""
    def l_local_py(u, dx, gamma, force_hlle, jp_cri, cons_switch=False):
        out = orc.l_local_py(u, dx, gamma, force_hlle, jp_cri, cons_switch)
        out[5, 7, 2] = np.nextafter(out[5, 7, 2], np.inf)
        return out

    planted = types.SimpleNamespace(l_local_py=l_local_py, con2primi_py=orc.con2primi_py)
    with pytest.raises(driver_replay.TraceMismatch):
        driver_replay.replay(planted, "rie_char_hlle")

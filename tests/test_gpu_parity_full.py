"""FP64 GPU solver against the oracle, bit for bit, on the benchmark cases at
their own sizes.

* The 4 x 13 cosine-spaced AR-4 wing (200 steps, the whole near-wake sheet
  kept), under the PC2 and AM2 schemes: the whole trajectory.
* The 2-blade hover rotor with its 260 near-wake rows and truncation after
  432 steps (2 x 6,240 rings + 2 x 172 far filaments at the end): the
  oracle needs minutes per hundred steps of this wake, so it checks three
  windows -- the first 24 steps from the start, the steps 255-266 around the
  start of the roll-up into the far wake, and the steps 427-440 through the
  first truncations -- each window starting from the GPU's own FP64 state
  (oracle/handoff.py) and then stepping independently.  Every step of the
  solver is deterministic given its state, so per-step bit equality from the
  GPU's states shows the trajectories are the same.
"""
import threading

import numpy as np
import pytest

from oracle import handoff
from oracle import oracle as O
from volcanor_gb300 import cases as C
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu

CHUNK = 256
ARRAYS = ("gam", "waN_gam", "waN_rvc", "waN_age", "waF", "waF_gam", "waF_rvc", "waF_age", "waF_l0", "waF_lc",
          "velN", "velN1", "velF", "velF1")


def snapshot(case, nb):
    snap = {"ct": case.ct_hist(), "gamVec": case.get("gamVec")}
    for b in range(1, nb + 1):
        snap[("waN", b)] = case.get("waN", b).reshape(-1, 4, 3)
        for name in ARRAYS:
            snap[(name, b)] = case.get(name, b)
    return snap


def assert_matches_oracle(snap, sim, nb, rows):
    np.testing.assert_array_equal(snap["ct"][-rows:], sim.ct_hist()[-rows:])
    np.testing.assert_array_equal(snap["gamVec"], sim.get("gamVec"))
    for b in range(1, nb + 1):
        np.testing.assert_array_equal(snap[("waN", b)], sim.get("waN", b).reshape(-1, 4, 2, 3)[:, :, 0])
        for name in ARRAYS:
            np.testing.assert_array_equal(snap[(name, b)], sim.get(name, b), err_msg=f"{name} blade {b}")


@pytest.mark.parametrize("fd", [1, 3])
def test_wing_ar4_full_trajectory_bitwise(fd):
    """4 x 13 cosine wing, alpha 5 deg, 200 steps, all 200 near-wake rows."""
    c = C.wing_ar4(nt=200, fd_scheme=fd)
    g = lib.Case(c.config, c.geom, precision=lib.PREC_FP64, sum_chunk=CHUNK)
    g.start()
    g.step(200)
    r = O.Sim(c.config, c.geom)
    r.set_sum_chunk(CHUNK)
    r.start()
    r.step(200)
    assert g.ct_hist().shape == (201, 10)
    assert_matches_oracle(snapshot(g, 1), r, 1, 201)


def test_hover_2blade_full_size_windows_bitwise():
    c = C.rotor_2blade_hover(nt=440)
    nb = 2
    g = lib.Case(c.config, c.geom, precision=lib.PREC_FP64, sum_chunk=CHUNK)
    g.start()
    assert g.geti("nNwake") == 260 and g.geti("nFwake") == 172
    errors, threads, checks = [], [], []

    def oracle_window(sim, nsteps, snap, rows):
        try:
            sim.step(nsteps)
            assert_matches_oracle(snap, sim, nb, rows)
            checks.append(rows)
        except BaseException as e:  # reported on the main thread
            errors.append(e)

    def window(start, nsteps):
        # the GPU runs on to `start`, the oracle takes its state there, both
        # advance nsteps; the oracle's steps run in the background while the
        # GPU goes on to the next window
        done = g.geti("iter")
        if start > done:
            g.step(start - done, with_ct=False)
        sim = O.Sim(c.config, c.geom)
        sim.set_sum_chunk(CHUNK)
        sim.start()
        if start > 0:
            assert handoff.load_case_state(sim, g) == start
        g.step(nsteps)
        t = threading.Thread(target=oracle_window, args=(sim, nsteps, snapshot(g, nb), nsteps))
        t.start()
        threads.append(t)

    window(0, 24)      # from the start
    window(254, 12)    # rowNear reaches 1 at step 260: roll-up into the far wake
    window(426, 14)    # rowFar reaches 1 at step 432: truncation from step 433
    assert g.geti("rowNear") == 1 and g.geti("rowFar") == 1
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    assert sorted(checks) == [12, 14, 24]

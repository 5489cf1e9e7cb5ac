"""The reference's predictor on the oracle (CPU): its 'P' convection loop
(`do i = 1, rowNear, nNwake`, src/classdef.f90:1549-1575) visits the first
near-wake node row only, so in a steady truncated wake the predicted wake
differs from the current one in ring rows 1 and 2 of each blade and in every
far-wake filament -- the sets the library's incremental predicted-wake
evaluation recomputes (volcanor_gb300/csrc/incr.cu)."""
import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C


@pytest.mark.parametrize("fd", [1, 3, 5])
def test_predictor_moves_the_first_row_and_the_far_wake(fd):
    # near wake 12 rows, truncation at 24: steady (rowNear 1, rowFar 1) from step 25
    c = C.rotor_2blade_hover(nt=40, n_nwake=12, truncate_nt=24, fd_scheme=fd)
    sim = O.Sim(c.config, c.geom)
    sim.start()
    sim.step(30)
    sim.step_open()  # iteration 31 up to its loads: the current wake of the step
    nb, ns, NW = sim.geti("nb"), sim.geti("ns"), sim.geti("nNwake")
    rn, rf, NF = sim.geti("rowNear"), sim.geti("rowFar"), sim.geti("nFwake")
    assert (rn, rf) == (1, 1)
    cur = [dict(n=sim.get("waN", b).reshape(ns, NW, 24), f=sim.get("waF", b).reshape(NF, 6),
                ng=sim.get("waN_gam", b).reshape(ns, NW), nr=sim.get("waN_rvc", b).reshape(ns, NW, 4),
                fg=sim.get("waF_gam", b), fr=sim.get("waF_rvc", b)) for b in range(1, nb + 1)]
    # an unmoved node (row 6 of blade 1) and its current-wake velocity
    P = cur[0]["n"][3, 5, 3:6][None, :]
    v_cur = sim.vind_points(P, predicted=False)
    sim.step_close()  # the predictor and the corrector
    v_pred = sim.vind_points(P, predicted=True)
    delta = np.zeros_like(P)
    for b in range(1, nb + 1):
        w = cur[b - 1]
        pn, pf = sim.get("waNP", b).reshape(ns, NW, 24), sim.get("waFP", b).reshape(NF, 6)
        ring_moved = np.any(pn != w["n"], axis=2)  # (span, row)
        assert ring_moved[:, :2].all() and not ring_moved[:, 2:].any()
        assert np.all(np.any(pf[rf - 1:] != w["f"][rf - 1:], axis=1))
        # the changed sources' new-minus-old share at the unmoved node (the
        # predicted wake carries the current wake's circulation and cores)
        corners = lambda a: a[:, :2].reshape(-1, 4, 6)[:, :, :3]
        rv, gm = w["nr"][:, :2].reshape(-1, 4), w["ng"][:, :2].reshape(-1)
        delta += O.vind_rings(corners(pn), rv, gm, P) - O.vind_rings(corners(w["n"]), rv, gm, P)
        act = slice(rf - 1, NF)
        delta += (O.vind_filaments(pf[act], w["fr"][act], w["fg"][act], P) -
                  O.vind_filaments(w["f"][act], w["fr"][act], w["fg"][act], P))
    # the incremental evaluation's identity, here in FP64 on the oracle
    assert np.max(np.abs(v_pred - (v_cur + delta))) <= 1e-12 * np.max(np.abs(v_cur))
    assert np.max(np.abs(delta)) > 1e-9 * np.max(np.abs(v_cur))  # the moved sources do contribute

"""Hand a product case's flow state to the oracle (TEST INFRASTRUCTURE ONLY).

The oracle steps a case at the cost of the reference's CPU algorithm, which
is minutes per hundred steps once the wake is long.  To compare the GPU
solver with the oracle late in a long run, or to time the oracle on a
late-run state, the GPU case runs to iteration k, and the oracle is brought
to the same iteration: its prescribed kinematics are advanced without flow
(``Sim.skip_to``) and every flow-state array is copied in from the case's
public getters (``vlm_case_get``).  From there both step independently; with
FP64 and equal summation blocks the GPU state and the oracle state stay
bit-identical step after step (``tests/test_gpu_parity_full.py``).

Only tests/ and bench.py's CPU legs use this module.
"""
from __future__ import annotations

import numpy as np

# per-blade arrays copied unchanged (same layouts on both sides)
_SAME = ("gam", "gamPrev", "waN_gam", "waN_rvc", "waN_age", "waF_gam", "waF_rvc", "waF_rvc0", "waF_l0", "waF_lc",
         "waF_age", "velN", "velN1", "velN2", "velN3", "velF", "velF1", "velF2", "velF3")


def ring_filaments(corners: np.ndarray) -> np.ndarray:
    """Ring corners [ring][corner][xyz] -> filaments [ring][k][fc1, fc2][xyz],
    filament k running from corner k to corner k+1 (the reference's vr_class)."""
    c = np.asarray(corners, dtype=np.float64).reshape(-1, 4, 3)
    return np.stack([c, np.roll(c, -1, axis=1)], axis=2)


def load_case_state(sim, case) -> int:
    """Bring oracle ``sim`` (created from the same case files, not yet
    stepped past the case's iteration) to the flow state of GPU ``case`` at
    its current iteration.  Returns that iteration."""
    k = case.geti("iter")
    sim.skip_to(k)
    nb = case.geti("nb")
    sim.set("gamVec", 1, case.get("gamVec"))
    for b in range(1, nb + 1):
        for name in _SAME:
            sim.set(name, b, case.get(name, b))
        sim.set("waN", b, ring_filaments(case.get("waN", b)))
        sim.set("waF", b, case.get("waF", b))
    return k

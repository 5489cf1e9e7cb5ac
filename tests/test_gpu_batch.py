"""Many uneven cases in one batch: each case's results equal its solo run's
bits (same precision and chunk plan), through the eager steps and the
steady-state steps replayed as one CUDA graph for the whole batch."""
import numpy as np
import pytest

from volcanor_gb300 import cases as C
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu


def uneven_cases():
    out = []
    for i, (nw, trunc, theta) in enumerate([(8, 12, 6.0), (12, 20, 8.0), (16, 22, 10.0), (10, 14, 4.0)]):
        c = C.rotor_2blade_hover(nt=60, n_nwake=nw, truncate_nt=trunc)
        out.append((c.config, c.geom.replace("theta0 = 8.0", f"theta0 = {theta}"), ""))
    w = C.wing_ar4(nt=60)
    out.append((w.config, w.geom, ""))
    return out


@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_FP32_NEAR64])
def test_batch_matches_solo_runs(prec):
    cases = uneven_cases()
    b = lib.Batch(cases, precision=prec, nbody_slots=16)
    b.start()
    rows = np.concatenate([b.step(10), b.step(50)], axis=1)
    assert b.last_step_ms() > 0
    for i, (cfg, geo, base) in enumerate(cases):
        g = lib.Case(cfg, geo, base, precision=prec, nbody_slots=16)
        g.start()
        solo = g.step(60)
        assert np.array_equal(rows[i], solo), i
        assert np.array_equal(b.case(i).get("waN", 1), g.get("waN", 1))

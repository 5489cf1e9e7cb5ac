"""Incremental predicted-wake evaluation (FP32 precisions): the predicted-wake
velocities as the current-wake ones plus the changed sources' new-minus-old
sum, and the full sum at the moved wake nodes only.  It must agree with the
full predicted-wake evaluation up to the grouping of FP32 pairs into tile
sums, find exactly the
sources and nodes the predictor moves, and give the same bits however the
steps are driven."""
import numpy as np
import pytest

from volcanor_gb300 import cases as C
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu

NT = 270
STEADY = 241  # first step of the steady signature (rowNear 1, rowFar 1)


def hover(fd_scheme=3, nt=NT):
    # near wake 160 rows, far wake from step 160, truncation at 240: one
    # signature from step 241 to NT, large enough for the incremental form
    # to pay (a few hundred changed records against ~8k)
    return C.rotor_2blade_hover(nt=nt, n_nwake=160, truncate_nt=240, fd_scheme=fd_scheme)


def run(prec, incremental=True, fd_scheme=3, lattice=None, use_graph=True, steps=NT):
    c = hover(fd_scheme)
    g = lib.Case(c.config, c.geom, precision=prec, incremental=incremental, lattice=lattice, use_graph=use_graph)
    g.start()
    rows = g.step(steps)
    return g, rows


def plan_rows(g):
    v = g.get("incremental")
    return v.reshape(-1, 9) if v.size else v.reshape(0, 9)


@pytest.mark.parametrize("prec,lattice,fd", [(lib.PREC_FP32_NEAR64, None, 3), (lib.PREC_FP32, None, 3),
                                             (lib.PREC_FP32_NEAR64, False, 3), (lib.PREC_FP32_NEAR64, None, 1),
                                             (lib.PREC_FP32, None, 5)])
def test_incremental_matches_the_full_predicted_evaluation(prec, lattice, fd):
    gi, ri = run(prec, True, fd, lattice)
    gf, rf = run(prec, False, fd, lattice)
    p = plan_rows(gi)
    assert p.shape[0] == 1 and plan_rows(gf).shape[0] == 0
    rn, rfar, on, changed, moved, dcap, mcap, nrec, M = p[0]
    assert (rn, rfar, on) == (1, 1, 1)
    ns, nb = gi.geti("ns"), gi.geti("nb")
    nfar = gi.geti("nFwake")
    # the predictor moves node row 1 and the far wake: ring rows 1 and 2 of
    # every blade and every far-wake filament change; node row 1 and every
    # far-wake node move
    far_fils = nb * (nfar - int(rfar) + 1)
    print("changed", changed, "moved", moved, "records", nrec, "targets", M, "far filaments", far_fils)
    assert changed == 2 * ns * nb + far_fils
    assert moved == (ns + 1) * nb + far_fils
    assert 2 * changed <= dcap and moved <= mcap
    # before the steady signature: the same path, the same bits
    assert np.array_equal(ri[:STEADY - 1], rf[:STEADY - 1])
    # after it: the same FP32 pairs grouped into other FP32 tile sums (as
    # another chunking groups them)
    ct_i, ct_f = ri[:, 1], rf[:, 1]
    print("max CT rel diff", np.max(np.abs(ct_i - ct_f) / np.abs(ct_f)))
    assert np.max(np.abs(ct_i - ct_f) / np.abs(ct_f)) < 2e-6


def test_incremental_same_bits_with_and_without_graphs_and_phases():
    prec = lib.PREC_FP32_NEAR64
    _, r1 = run(prec, True, use_graph=True)
    _, r2 = run(prec, True, use_graph=False)
    assert np.array_equal(r1, r2)
    # the step driven phase by phase
    c = hover()
    g = lib.Case(c.config, c.geom, precision=prec)
    g.start()
    rows = []
    for _ in range(NT):
        g.solve_circulation()
        rows.append(g.loads())
        g.wake_step()
    assert np.array_equal(np.array(rows), r1)


def test_incremental_resumed_run_gives_the_same_bits(tmp_path):
    prec = lib.PREC_FP32_NEAR64
    _, full = run(prec, True)
    c = hover()
    g = lib.Case(c.config, c.geom, precision=prec)
    g.start()
    g.step(STEADY + 9)
    ck = tmp_path / "mid.ckpt"
    g.checkpoint_save(ck)
    h = lib.Case(c.config, c.geom, precision=prec)
    h.checkpoint_load(ck)
    rest = h.step(NT - STEADY - 9)
    assert plan_rows(h)[0, 2] == 1
    assert np.array_equal(rest, full[STEADY + 9:])


def test_incremental_not_used_where_it_does_not_apply():
    # FP64 keeps the full evaluation
    c = C.rotor_2blade_hover(nt=60, n_nwake=20, truncate_nt=36)
    g = lib.Case(c.config, c.geom, precision=lib.PREC_FP64)
    g.start()
    g.step(60, with_ct=False)
    assert plan_rows(g).shape[0] == 0
    # a small wake: measured, but the full evaluation is cheaper
    h = lib.Case(c.config, c.geom, precision=lib.PREC_FP32_NEAR64)
    h.start()
    h.step(60, with_ct=False)
    p = plan_rows(h)
    assert p.shape[0] == 1 and p[0, 2] == 0


def test_incremental_in_a_batch():
    """Cases of a batch (one graph launch per step) take the same plans as
    lone cases; their loads agree with the full evaluation's."""
    cs = [hover(3), hover(1)]
    rows = {}
    for inc in (True, False):
        b = lib.Batch([(c.config, c.geom, "") for c in cs], precision=lib.PREC_FP32_NEAR64, incremental=inc)
        b.start()
        rows[inc] = b.step(NT)
        for i in range(len(cs)):
            p = plan_rows(b.case(i))
            assert p.shape[0] == (1 if inc else 0)
            if inc:
                assert p[0, 2] == 1
    ri, rf = rows[True], rows[False]
    assert np.array_equal(ri[:, :STEADY - 1], rf[:, :STEADY - 1])
    assert np.max(np.abs(ri[..., 1] - rf[..., 1]) / np.abs(rf[..., 1])) < 2e-6

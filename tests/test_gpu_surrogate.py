"""The learned far-wake surrogate inside the solver: collection, GPU training,
per-step FP64 audits, revert on a failed audit, and what it gains."""
import tempfile

import numpy as np
import pytest

from volcanor_gb300 import cases as C
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu


def forward_case(nt, prec, surr=None, use_graph=True):
    c = C.rotor_4blade_forward(nt=nt, n_nwake=24)
    with tempfile.TemporaryDirectory() as d:
        c.write(d)
        g = lib.Case.from_case_dir(d, precision=prec, use_graph=use_graph)
    if surr is not None:
        g.set_surrogate(**surr)
    g.start()
    return g


def test_surrogate_trains_audits_and_gains_over_omission():
    """After training on solver-generated pairs, the network's audit error (the
    relative rms error of the old-far-wake velocity at the audited targets,
    against the direct FP64 sum) is far below that of the method without it,
    leaving the old far wake out (error 1 by definition), and the audited
    steps use it."""
    nt = 240
    opts = dict(young_far=48, min_far=24, collect_steps=24, sample_stride=2, train_iters=2000, audit_tol=0.2)
    g = forward_case(nt, lib.PREC_FP32_NEAR64, opts)
    ct = g.step(nt)[:, 1]
    st = g.surrogate_stats()
    print(st)
    assert st["trainings"] >= 1 and st["audits"] > 0
    assert st["active_steps"] + st["reverts"] == st["audits"]
    # most audited steps passed (error <= 0.2, five times below omission's 1)
    assert st["active_steps"] >= 0.5 * st["audits"]
    assert np.all(np.isfinite(ct))


def test_surrogate_reverts_when_the_audit_fails():
    # an untrained network (no Adam steps) cannot pass a tight audit: every
    # audit reverts to the direct sum and retrains, and the results equal
    # the direct run's bits on the reverted steps' inputs
    nt = 120
    opts = dict(young_far=48, min_far=8, collect_steps=8, sample_stride=4, train_iters=0, audit_tol=1e-6)
    g = forward_case(nt, lib.PREC_FP32_NEAR64, opts, use_graph=False)
    ct = g.step(nt)[:, 1]
    st = g.surrogate_stats()
    assert st["audits"] > 0 and st["reverts"] == st["audits"] and st["active_steps"] == 0
    ref = forward_case(nt, lib.PREC_FP32_NEAR64, use_graph=False).step(nt)[:, 1]
    assert np.array_equal(ct, ref)

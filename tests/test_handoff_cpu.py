"""The oracle's state hand-off (kinematics-only advance + flow-state setters)
is complete: an oracle brought to iteration k from another oracle's state
continues bit for bit.  The GPU parity tests at full case size rely on it
(tests/test_gpu_parity_full.py)."""
import numpy as np
import pytest

from oracle import handoff
from oracle import oracle as O
from volcanor_gb300 import cases as C


class OracleAsCase:
    """An oracle Sim seen through the product case's getter names: the
    near-wake array as ring corners (the product's layout)."""

    def __init__(self, sim):
        self.s = sim

    def geti(self, name):
        return self.s.geti(name)

    def get(self, name, b=1):
        if name == "waN":
            return self.s.get("waN", b).reshape(-1, 4, 2, 3)[:, :, 0, :].ravel()
        return self.s.get(name, b)


@pytest.mark.parametrize("fd", [1, 3, 5])
def test_handoff_continues_bit_for_bit(fd):
    c = C.rotor_2blade_hover(nt=60, n_nwake=10, truncate_nt=22, fd_scheme=fd)
    a = O.Sim(c.config, c.geom)
    a.set_sum_chunk(16)
    a.start()
    a.step(26)  # past the roll-up (step 10) and the truncation (step 22)
    b = O.Sim(c.config, c.geom)
    b.set_sum_chunk(16)
    b.start()
    assert handoff.load_case_state(b, OracleAsCase(a)) == 26
    a.step(8)
    b.step(8)
    np.testing.assert_array_equal(a.ct_hist()[-8:], b.ct_hist()[-8:])
    for bl in (1, 2):
        for name in ("waN", "waN_gam", "waN_rvc", "waF", "waF_gam", "waF_rvc", "velN", "velF", "gam"):
            np.testing.assert_array_equal(a.get(name, bl), b.get(name, bl), err_msg=name)


def test_skip_to_reaches_the_stepped_geometry():
    c = C.rotor_4blade_forward(nt=30, n_nwake=6)
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        c.write(d)
        a = O.Sim.from_case_dir(d)
        b = O.Sim.from_case_dir(d)
    a.start()
    a.step(12)
    b.start()
    b.skip_to(12)
    for bl in range(1, 5):
        for name in ("PC", "vr", "CP", "nCap", "secCP"):
            np.testing.assert_array_equal(a.get(name, bl), b.get(name, bl), err_msg=name)
    assert a.geti("rowNear") == b.geti("rowNear") and a.geti("rowFar") == b.geti("rowFar")

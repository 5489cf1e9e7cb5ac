"""The oracle's coupled rotors (nr > 1) on the CPU: a lone rotor as a system
is the single-rotor oracle bit for bit; two rotors that map onto each other
by a half turn about the shaft carry equal loads while the coupling moves
them away from an isolated rotor's."""
import numpy as np

from oracle import oracle as O
from volcanor_gb300 import cases as C


def test_lone_rotor_system_is_the_single_rotor_oracle():
    O.set_threads(4)
    c = C.rotor_2blade_hover(nt=24, n_nwake=8, truncate_nt=12)
    s = O.Sim(c.config, c.geom)
    s.set_sum_chunk(16)
    s.start()
    s.step(24)
    y = O.System(c.config, [c.geom])
    y.set_sum_chunk(16)
    y.start()
    y.step(24)
    assert np.array_equal(s.ct_hist(), y.rotors[0].ct_hist())
    assert np.array_equal(s.get("waN", 2), y.rotors[0].get("waN", 2))


def test_half_turn_symmetric_pair():
    O.set_threads(4)
    sc = C.rotor_pair(nt=30, n_nwake=12, truncate_nt=18, hub1=(1.3, 0.0, 0.0), hub2=(-1.3, 0.0, 0.0), omega2=100.0)
    y = O.System(sc.config, sc.geoms)
    y.start()
    y.step(30)
    a, b = y.rotors[0].ct_hist()[:, 1], y.rotors[1].ct_hist()[:, 1]
    assert np.max(np.abs(a - b) / np.abs(a)) < 1e-12
    iso = O.Sim(sc.config.replace("nr = 2", "nr = 1"), sc.geoms[0])
    iso.start()
    iso.step(30)
    assert np.max(np.abs(iso.ct_hist()[:, 1] - a) / np.abs(a)) > 1e-3


def test_system_input_checks():
    sc = C.rotor_pair(nt=4)
    try:
        O.System(sc.config, sc.geoms[:1])
    except O.OracleError as e:
        assert "nr" in str(e)
    else:
        raise AssertionError("nr mismatch accepted")
    try:
        O.Sim(sc.config, sc.geoms[0])
    except O.OracleError as e:
        assert "system" in str(e)
    else:
        raise AssertionError("nr = 2 accepted by a lone rotor")


def test_ground_effect_image_rotor():
    """A hover rotor at h = 0.5 R and its image in the ground plane
    (surfaceType -1, imagePlane 3): the image's circulation and wake are the
    exact mirror of the rotor's, and the ground raises its thrust against the
    same rotor in free air, less so higher up."""
    O.set_threads(4)
    gains = []
    for h in (0.5, 1.5):
        sc = C.rotor_ground_effect(height=h, nt=30, n_nwake=12, truncate_nt=18)
        y = O.System(sc.config, sc.geoms)
        y.start()
        y.step(30)
        a, b = y.rotors
        assert np.array_equal(b.get("gamVec"), -a.get("gamVec"))
        wa, wb = a.get("waN", 1).reshape(-1, 3), b.get("waN", 1).reshape(-1, 3)
        assert np.array_equal(wb[:, :2], wa[:, :2]) and np.array_equal(wb[:, 2], -wa[:, 2])
        iso = O.Sim(sc.config.replace("nr = 2", "nr = 1"), sc.geoms[0])
        iso.start()
        iso.step(30)
        gains.append(a.ct_hist()[-5:, 1].mean() / iso.ct_hist()[-5:, 1].mean() - 1.0)
    assert gains[0] > gains[1] > 0.0

"""Prescribed wing kinematics (scope row a18) on the host, bit for bit
against the oracle, on the CPU: the initial pitch and the motion of every
step (translation, shaft rotation, collective and cyclic pitch, slow start)
applied to the geometry of rotor_init, through vlm_wing_kinematics."""
import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C
from volcanor_gb300 import lib


def _cases(tmp):
    out = {}
    h = C.rotor_2blade_hover(nt=10, n_nwake=4, truncate_nt=8)
    out["hover"] = (h.config, h.geom, "", 10)
    f = C.rotor_4blade_forward(nt=8, n_nwake=4)
    d = tmp / "fwd"
    f.write(d)
    geo = f.geom.replace("thetaC = 0.0", "thetaC = 2.0").replace("thetaS = 0.0", "thetaS = -1.5")
    (d / "geom01.nml").write_text(geo)
    out["forward_cyclic"] = (f.config, geo, str(d), 8)
    w = C.wing_ar4(nt=6)
    out["wing"] = (w.config, w.geom, "", 6)
    for ss in (1, 2, 3):
        cfg = C.config_text(nt=8, dt=0.0, density=1.2, fdScheme=3, slowStart=ss, slowStartNt=5)
        geo = C.geom_text(nb=3, nc=2, ns=5, nNwake=4, span=1.5, rootcut=0.15, chord=0.1, Omega=80.0,
                          shaftAxis=(0.0, 0.0, 1.0), theta0=6.0, velBody=(-2.0, 0.0, -0.5), preconeAngle=2.0,
                          pivotLE=0.3, phiThetaPsi=(1.0, -3.0, 5.0))
        out[f"slowstart{ss}"] = (cfg, geo, "", 8)
    return out


@pytest.mark.parametrize("name", ["hover", "forward_cyclic", "wing", "slowstart1", "slowstart2", "slowstart3"])
def test_host_kinematics_match_oracle(name, tmp_path):
    cfg, geo, base, nt = _cases(tmp_path)[name]
    nb = int(O.Sim(cfg, geo, base).geti("nb"))
    its = sorted({0, 1, nt // 2, nt})
    for it in its:
        r = O.Sim(cfg, geo, base)
        r.start()
        if it:
            r.step(it)
        for b in range(1, nb + 1):
            for arr in ("PC", "CP", "nCap", "secCP"):
                np.testing.assert_array_equal(lib.wing_kinematics(cfg, geo, it, arr, b, base), r.get(arr, b),
                                              err_msg=f"{name} iter {it} blade {b} {arr}")
            for arr in ("vr_rvc", "secArea", "secChord"):
                np.testing.assert_array_equal(lib.wing_kinematics(cfg, geo, it, arr, b, base), r.get(arr, b),
                                              err_msg=f"{name} iter {it} blade {b} {arr}")
            ring = lib.wing_kinematics(cfg, geo, it, "vr", b, base).reshape(-1, 4, 3)
            np.testing.assert_array_equal(ring, r.get("vr", b).reshape(-1, 4, 2, 3)[:, :, 0],
                                          err_msg=f"{name} iter {it} blade {b} vr")


def test_kinematics_errors():
    h = C.rotor_2blade_hover(nt=4, n_nwake=2, truncate_nt=3)
    with pytest.raises(lib.VlmError):
        lib.wing_kinematics(h.config, h.geom, 5, "CP")      # beyond nt
    with pytest.raises(lib.VlmError):
        lib.wing_kinematics(h.config, h.geom, 1, "CP", 3)   # no blade 3
    with pytest.raises(lib.VlmError):
        lib.wing_kinematics(h.config, h.geom, 1, "nope")


@pytest.mark.parametrize("tutorial", ["caradonna", "simplewing", "tr1208"])
def test_host_kinematics_match_oracle_on_reference_tutorials(golden_dir, tutorial):
    """The reference's tutorial cases (Caradonna-Tung rotor, simple wing,
    TR1208 wing from PLOT3D), as shipped: geometry and motion of the first
    steps bit for bit."""
    d = golden_dir / f"tutorial-{tutorial}"
    cfg, geo = (d / "config.nml").read_text(), (d / "geom01.nml").read_text()
    nb = int(O.Sim(cfg, geo, str(d)).geti("nb"))
    for it in (0, 1, 4):
        r = O.Sim(cfg, geo, str(d))
        r.start()
        if it:
            r.step(it)
        for b in range(1, nb + 1):
            for arr in ("PC", "CP", "nCap", "secCP", "vr_rvc", "secArea", "secChord"):
                np.testing.assert_array_equal(lib.wing_kinematics(cfg, geo, it, arr, b, d), r.get(arr, b),
                                              err_msg=f"{tutorial} iter {it} blade {b} {arr}")

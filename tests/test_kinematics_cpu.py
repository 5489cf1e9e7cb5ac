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


def _trajectory_text(nt, seed, split_every=0):
    """trajectory01.in: nt records of u v w p q r; every split_every-th record
    runs over two lines and uses Fortran d exponents."""
    rng = np.random.default_rng(seed)
    lines = []
    for i in range(nt):
        u, v, w = -10.0 + 0.5 * np.sin(0.3 * i), 0.2 * rng.normal(), 0.3 * np.cos(0.2 * i)
        p, q, r = 0.05 * rng.normal(), 0.1 * np.sin(0.1 * i), 0.02 * rng.normal()
        if split_every and i % split_every == 0:
            lines.append(f"{u:.10e}, {v:.10e}, {w:.10e}".replace("e", "d"))
            lines.append(f"{p:.10e} {q:.10e} {r:.10e} 99.0")
        else:
            lines.append(f"{u:.12e} {v:.12e} {w:.12e} {p:.12e} {q:.12e} {r:.12e}")
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("kind", ["wing", "rotor"])
def test_custom_trajectory_kinematics_match_oracle(tmp_path, kind):
    """customTrajectorySwitch = 1: the body velocity and rates of every step
    come from trajectory01.in (src/classdef.f90:3065-3081, src/main.f90:111-116,419-424)."""
    nt = 9
    if kind == "wing":
        cfg = C.config_text(nt=nt, dt=0.025, density=1.0, fdScheme=3)
        geo = C.geom_text(nb=1, nc=3, ns=4, nNwake=4, span=2.0, chord=0.5, theta0=5.0, velBody=(-10.0, 0.0, 0.0),
                          customTrajectorySwitch=1, cgCoords=(0.1, 0.0, 0.0))
    else:
        cfg = C.config_text(nt=nt, dt=0.0, density=1.2, fdScheme=3)
        geo = C.geom_text(nb=2, nc=1, ns=5, nNwake=4, span=1.0, rootcut=0.2, chord=0.08, Omega=100.0,
                          shaftAxis=(0.0, 0.0, 1.0), theta0=8.0, velBody=(-5.0, 0.0, 0.0), customTrajectorySwitch=1)
    (tmp_path / "trajectory01.in").write_text(_trajectory_text(nt, 5, split_every=3))
    base = str(tmp_path)
    nb = int(O.Sim(cfg, geo, base).geti("nb"))
    for it in (0, 1, 4, nt):
        r = O.Sim(cfg, geo, base)
        r.start()
        if it:
            r.step(it)
        for b in range(1, nb + 1):
            for arr in ("PC", "CP", "nCap", "secCP"):
                np.testing.assert_array_equal(lib.wing_kinematics(cfg, geo, it, arr, b, base), r.get(arr, b),
                                              err_msg=f"{kind} iter {it} blade {b} {arr}")
    # the motion differs from the namelist's constant velocity
    steady = lib.wing_kinematics(cfg, geo.replace("customTrajectorySwitch = 1", "customTrajectorySwitch = 0"),
                                 nt, "CP", 1, base)
    assert not np.array_equal(steady, lib.wing_kinematics(cfg, geo, nt, "CP", 1, base))
    # rXXParams.json echoes the namelist velocity (params2file runs before any step)
    import json
    assert json.loads(lib.params_json(cfg, geo, base))["u"] == pytest.approx(-10.0 if kind == "wing" else -5.0)


def test_custom_trajectory_missing_or_short_file(tmp_path):
    cfg = C.config_text(nt=5, dt=0.025, density=1.0, fdScheme=3)
    geo = C.geom_text(nb=1, nc=2, ns=3, nNwake=3, span=2.0, chord=0.5, theta0=5.0, velBody=(-10.0, 0.0, 0.0),
                      customTrajectorySwitch=1)
    with pytest.raises(lib.VlmError):
        lib.wing_kinematics(cfg, geo, 1, "CP", 1, tmp_path)
    (tmp_path / "trajectory01.in").write_text(_trajectory_text(3, 0))
    with pytest.raises(lib.VlmError):
        lib.wing_kinematics(cfg, geo, 1, "CP", 1, tmp_path)


def _camber_case(tmp, omega, theta0=4.0, limits=(0.5, 1.0), files=("naca.dat", "tab.dat")):
    xs = np.linspace(0.0, 1.0, 11)
    (tmp / "naca.dat").write_text(f"{len(xs)}\n" + "\n".join(f"{x * 2.0:.12f} {0.08 * x * (1 - x) * 2.0:.12f}"
                                                              for x in xs) + "\n")
    tab = [(0.0, 0.0), (0.1, 0.012), (0.3, 0.03), (0.55, 0.028), (0.8, 0.015), (1.0, 0.0)]
    (tmp / "tab.dat").write_text(f"{len(tab)}\n" + "\n".join(f"{a}d0, {b}D0" for a, b in tab) + "\n")
    nf = len(files)
    geo = C.geom_text(nb=2 if omega else 1, nc=4, ns=6, nNwake=3, span=1.5, rootcut=0.2 if omega else 0.0,
                      chord=0.3, Omega=omega, shaftAxis=(0.0, 0.0, 1.0), theta0=theta0,
                      velBody=(0.0, 0.0, 0.0) if omega else (-10.0, 0.0, 0.0), chordSpacing=2, spanSpacing=2,
                      nCamberFiles=nf)
    sect = ("&CAMBERSECTIONS\ncamberSectionLimit = " + ", ".join(str(v) for v in limits[:nf]) +
            "\ncamberFile = " + ", ".join(f"'{f}'" for f in files) + "\n/\n")
    geo = geo.replace("&ORIENT", sect + "&ORIENT", 1)
    cfg = C.config_text(nt=4, dt=0.0 if omega else 0.025, density=1.0, fdScheme=3)
    return cfg, geo


@pytest.mark.parametrize("omega", [0.0, 60.0, -60.0])
def test_camber_sections_match_oracle(tmp_path, omega):
    """nCamberFiles > 0 (rotor_getCamber, src/classdef.f90:4060-4112, with
    libMath interp1d of order 2): cambered panels, bit for bit against the oracle."""
    cfg, geo = _camber_case(tmp_path, omega)
    assert "&CAMBERSECTIONS" in geo
    base = str(tmp_path)
    nb = int(O.Sim(cfg, geo, base).geti("nb"))
    for it in (0, 3):
        r = O.Sim(cfg, geo, base)
        r.start()
        if it:
            r.step(it)
        for b in range(1, nb + 1):
            for arr in ("PC", "CP", "nCap", "secCP"):
                np.testing.assert_array_equal(lib.wing_kinematics(cfg, geo, it, arr, b, base), r.get(arr, b),
                                              err_msg=f"omega {omega} iter {it} blade {b} {arr}")


def test_camber_reproduces_a_parabola(tmp_path):
    """A parabolic camber line is reproduced exactly by the quadratic
    Lagrange interpolation (no pitch, so the panel corners keep the camber)."""
    cfg, geo = _camber_case(tmp_path, 0.0, theta0=0.0, limits=(1.0,), files=("naca.dat",))
    pc = lib.wing_kinematics(cfg, geo, 0, "PC", 1, tmp_path).reshape(6, 4, 4, 3)  # [j][i][corner]
    x, z = pc[..., 0], pc[..., 2]
    xi = (x - -0.3) / 0.3  # chord from -c (leading edge) to 0
    np.testing.assert_allclose(z, 0.3 * 0.08 * xi * (1 - xi), rtol=0, atol=1e-14)
    assert np.max(z) > 0.005

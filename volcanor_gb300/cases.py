"""Case-file generation: the reference's ``config.nml`` / ``geomXX.nml`` formats.

VOLCANOR reads a case from namelist files (``readConfig``,
src/libCommon.f90:51-108, format version 0.5; ``rotor_readGeom``,
src/classdef.f90:2541-2767, format version 0.15).  This module writes those
files from Python keyword arguments, with every key present, so a case built
here runs unchanged in the reference and in this package.

It also defines the benchmark workloads as concrete case files:

* :func:`wing_ar4` -- flat rectangular wing, chord 1 m, aspect ratio 4,
  4 x 13 rings (cosine spanwise), alpha 5 deg, 10 m/s, dt = c/(4V), 200 steps.
* :func:`rotor_2blade_hover` -- 2-blade hovering rotor, R = 1 m, root cut 0.2R,
  chord 0.08 m, collective 8 deg, Omega = 100 rad/s, 1 x 24 rings per blade,
  dt = 5 deg, 1440 steps, wake truncated after 6 revs (432 steps), viscous
  core growth on.
* :func:`rotor_4blade_forward` -- 4-blade rotor in forward flight (R = 2 m,
  c = 0.12 m, -8 deg linear twist via a PLOT3D blade, collective 10 deg,
  advance ratio 0.1, shaft tilt -4 deg, 1 x 32 rings per blade, dt = 5 deg).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from pathlib import Path
from typing import Dict, Optional

CONFIG_DEFAULTS: Dict[str, Dict[str, object]] = {
    "VERSION": {"fileFormatVersion": "0.5"},
    "PARAMS": {"nt": -10, "dt": 0.0, "nr": 1, "density": 1.0, "velSound": 330.0, "kinematicVisc": 0.000018},
    "OPTIONS": {
        "restartWriteNt": 0, "restartFromNt": 0, "ntSub": 0, "ntSubInit": 0,
        "wakePlot": 0, "wakeTipPlot": 0, "rotorForcePlot": 1, "gridPlot": 0,
        "wakeDissipation": 0, "wakeStrain": 0, "wakeBurst": 0, "wakeSuppress": 0,
        "slowStart": 0, "slowStartNt": 0, "fdScheme": 3, "initWakeVelNt": 0, "probe": 0,
    },
}

GEOM_DEFAULTS: Dict[str, Dict[str, object]] = {
    "VERSION": {"fileFormatVersion": "0.15"},
    "SURFACE": {"surfaceType": 0, "imagePlane": 3, "imageRotorNum": 1},
    "PANELS": {"nb": 1, "propConvention": 0, "spanSpacing": 2, "chordSpacing": 1,
               "geometryFile": "0", "nCamberFiles": 0, "nc": 4, "ns": 13, "nNwake": 160},
    "CAMBERSECTIONS": {"camberSectionLimit": 1.0, "camberFile": "0"},
    "ORIENT": {"hubCoords": (0.0, 0.0, 0.0), "cgCoords": (0.0, 0.0, 0.0),
               "fromCoords": (0.0, 0.0, 0.0), "phiThetaPsi": (0.0, 0.0, 0.0)},
    "GEOMPARAMS": {
        "span": 4.0, "rootcut": 0.0, "chord": 1.0, "preconeAngle": 0.0, "Omega": 0.0,
        "shaftAxis": (0.0, 0.0, 1.0), "theta0": 5.0, "thetaC": 0.0, "thetaS": 0.0, "thetaTwist": 0.0,
        "ductSwitch": 0, "axisymmetrySwitch": 0, "pivotLE": 0.0, "flapHinge": 0.0,
        "spanwiseLiftSwitch": 0, "symmetricTau": 1, "customTrajectorySwitch": 0,
        "velBody": (-10.0, 0.0, 0.0), "omegaBody": (0.0, 0.0, 0.0), "forceCalcSwitch": 0, "nAirfoils": 0,
    },
    "WAKEPARAMS": {
        "apparentViscCoeff": 1.0, "decayCoeff": 0.0, "wakeTruncateNt": 0, "prescWakeAfterTruncNt": 0,
        "prescWakeGenNt": 0, "spanwiseCore": 0.04, "streamwiseCoreVec": 0.04, "rollupStartRadius": 0.75,
        "rollupEndRadius": 1.0, "initWakeVel": 0.0, "psiStart": 0.0, "skewLimit": 0.5,
    },
    "DYNAMICS": {
        "bladeDynamicsSwitch": 0, "flapInitial": 0.0, "dflapInitial": 0.0, "Iflap": 0.0, "cflap": 0.0,
        "kflap": 0.0, "MflapConstant": 0.0, "pitchDynamicsSwitch": 0, "dpitch": 0.0,
        "bodyDynamicsSwitch": 0, "bodyDynamicsIOVars": 0,
    },
    "WINDFRAME": {"dragUnitVec": (0.0, 0.0, 0.0), "sideUnitVec": (0.0, 0.0, 0.0), "liftUnitVec": (0.0, 0.0, 0.0)},
    "PLOTS": {"inflowPlotSwitch": 0, "gammaPlotSwitch": 0, "skewPlotSwitch": 0},
    "AIRFOILS": {"airfoilSectionLimit": 1.0, "alpha0": 0.0, "airfoilFile": "0"},
}


def _fmt(v: object) -> str:
    if isinstance(v, (tuple, list)):
        return ", ".join(_fmt(x) for x in v)
    if isinstance(v, bool):
        return "1" if v else "0"
    if isinstance(v, int):
        return str(v)
    if isinstance(v, float):
        return repr(v)
    return str(v)


def _render(defaults: Dict[str, Dict[str, object]], overrides: Dict[str, object]) -> str:
    groups = {g: dict(kv) for g, kv in defaults.items()}
    keymap = {k.lower(): (g, k) for g, kv in defaults.items() for k in kv}
    for k, v in overrides.items():
        if k.lower() not in keymap:
            raise KeyError(f"unknown namelist key {k!r}")
        g, kk = keymap[k.lower()]
        groups[g][kk] = v
    out = []
    for g, kv in groups.items():
        out.append(f"&{g}")
        for k, v in kv.items():
            out.append(f"{k} = {_fmt(v)}")
        out.append("/")
        out.append("")
    return "\n".join(out)


def config_text(**overrides: object) -> str:
    """config.nml text (version 0.5) with every key present."""
    return _render(CONFIG_DEFAULTS, overrides)


def geom_text(**overrides: object) -> str:
    """geomXX.nml text (version 0.15) with every key present."""
    return _render(GEOM_DEFAULTS, overrides)


@dataclass
class Case:
    """A case directory's contents: config.nml, geom01.nml and extra files."""

    name: str
    config: str
    geom: str
    files: Dict[str, str] = field(default_factory=dict)

    def write(self, directory: str | Path) -> Path:
        d = Path(directory)
        d.mkdir(parents=True, exist_ok=True)
        (d / "config.nml").write_text(self.config)
        (d / "geom01.nml").write_text(self.geom)
        for fname, text in self.files.items():
            (d / fname).write_text(text)
        return d


def c81_text(name: str, mach, alpha, cl, cd, cm) -> str:
    """An airfoil table in the C81 layout the reference reads and writes
    (libC81.f90:60-188): a 30-column name and six 2-digit counts (Mach
    numbers and angles for lift, drag, moment), then per coefficient a line of
    Mach numbers (7 blank columns, 7-column fields, 3 decimals) and per angle
    a line of the angle (7 columns, 2 decimals) and the values (7 columns, 3
    decimals); more than 9 Mach numbers continue on a second line.  cl, cd,
    cm: arrays [angle][Mach]."""
    import numpy as np
    mach, alpha = np.asarray(mach, float), np.asarray(alpha, float)
    M, N = len(mach), len(alpha)
    if not (1 <= M <= 18):
        raise ValueError("1 to 18 Mach numbers")
    out = [f"{name[:30]:<30s}" + "".join(f"{v:02d}" for v in (M, N, M, N, M, N))]
    f73 = lambda v: f"{v:7.3f}"
    for tab in (cl, cd, cm):
        tab = np.asarray(tab, float).reshape(N, M)
        out.append(" " * 7 + "".join(f73(v) for v in mach[:9]))
        if M > 9:
            out.append(" " * 7 + "".join(f73(v) for v in mach[9:]))
        for i in range(N):
            out.append(f"{alpha[i]:7.2f}" + "".join(f73(v) for v in tab[i, :9]))
            if M > 9:
                out.append(" " * 7 + "".join(f73(v) for v in tab[i, 9:]))
    return "\n".join(out) + "\n"


def synthetic_airfoil(name: str, cl_slope: float = 6.0, alpha0_deg: float = 0.0, cd0: float = 0.008,
                      nmach: int = 6) -> str:
    """A smooth synthetic table: angles -20..20 deg (2 deg), Mach 0..0.75,
    CL = slope sin(alpha - alpha0) / sqrt(1 - M^2) (Prandtl-Glauert), CD =
    cd0 + 0.5 sin^2(alpha), CM = -0.02 - 0.05 sin(alpha)."""
    import numpy as np
    mach = np.linspace(0.0, 0.75, nmach)
    alpha = np.arange(-20.0, 20.0 + 1e-9, 2.0)
    a = np.radians(alpha)[:, None]
    pg = 1.0 / np.sqrt(1.0 - mach[None, :] ** 2)
    cl = cl_slope * np.sin(a - np.radians(alpha0_deg)) * pg
    cd = cd0 + 0.5 * np.sin(a) ** 2 + 0 * pg
    cm = -0.02 - 0.05 * np.sin(a) + 0 * pg
    return c81_text(name, mach, alpha, cl, cd, cm)


@dataclass
class SystemCase:
    """Coupled rotors (nr > 1): one config.nml, geom01.nml .. geomNN.nml."""

    name: str
    config: str
    geoms: list

    def write(self, directory: str | Path) -> Path:
        d = Path(directory)
        d.mkdir(parents=True, exist_ok=True)
        (d / "config.nml").write_text(self.config)
        for i, g in enumerate(self.geoms):
            (d / f"geom{i + 1:02d}.nml").write_text(g)
        return d


def rotor_pair(nt: int = 60, ns: int = 8, n_nwake: int = 24, truncate_nt: int = 30, hub2=(0.0, 0.0, -0.3),
               omega2: float = -100.0, hub1=(0.0, 0.0, 0.0), fd_scheme: int = 3, dissipation: int = 1,
               **geom_overrides) -> SystemCase:
    """Two coupled 2-blade hover rotors (R = 1 m, c = 0.08 m, collective 8
    deg, dt = 5 deg): by default coaxial and counter-rotating, the second
    0.3 R below the first."""
    cfg = config_text(nt=nt, dt=0.0, nr=2, density=1.2, kinematicVisc=1.5e-5, fdScheme=fd_scheme,
                      wakeDissipation=dissipation)
    base = dict(nb=2, nc=1, ns=ns, nNwake=n_nwake, span=1.0, rootcut=0.2, chord=0.08, shaftAxis=(0.0, 0.0, 1.0),
                theta0=8.0, velBody=(0.0, 0.0, 0.0), spanSpacing=1, chordSpacing=1, spanwiseCore=0.05,
                streamwiseCoreVec=0.05, apparentViscCoeff=5.0, wakeTruncateNt=truncate_nt, symmetricTau=0,
                pivotLE=0.25)
    base.update(geom_overrides)
    g1 = geom_text(**{**base, "Omega": 100.0, "hubCoords": tuple(hub1), "cgCoords": tuple(hub1)})
    g2 = geom_text(**{**base, "Omega": omega2, "hubCoords": tuple(hub2), "cgCoords": tuple(hub2)})
    return SystemCase("rotor_pair", cfg, [g1, g2])


def rotor_ground_effect(height: float = 0.6, nt: int = 60, ns: int = 8, n_nwake: int = 24, truncate_nt: int = 30,
                        fd_scheme: int = 3) -> SystemCase:
    """A 2-blade hover rotor (as rotor_pair's) with its hub `height` above the
    ground plane z = 0, and its image below it: rotor 2 is surfaceType -1,
    imagePlane 3, mirroring rotor 1 (the reference's ground-effect setup)."""
    sc = rotor_pair(nt=nt, ns=ns, n_nwake=n_nwake, truncate_nt=truncate_nt, hub1=(0.0, 0.0, height),
                    hub2=(0.0, 0.0, -height), omega2=100.0, fd_scheme=fd_scheme)
    img = geom_text(surfaceType=-1, imagePlane=3, imageRotorNum=1, nb=2, nc=1, ns=ns, nNwake=n_nwake)
    return SystemCase("rotor_ground_effect", sc.config, [sc.geoms[0], img])


def wing_ar4(nt: int = 200, fd_scheme: int = 1, n_nwake: Optional[int] = None) -> Case:
    """Flat wing, c = 1 m, AR 4, 4 x 13 rings, alpha 5 deg, V = 10 m/s, dt = c/(4V)."""
    cfg = config_text(nt=nt, dt=0.025, density=1.0, fdScheme=fd_scheme, wakeDissipation=0)
    geo = geom_text(nb=1, nc=4, ns=13, nNwake=nt if n_nwake is None else n_nwake, span=4.0, rootcut=0.0,
                    chord=1.0, Omega=0.0, theta0=5.0, velBody=(-10.0, 0.0, 0.0), spanSpacing=2,
                    chordSpacing=1, spanwiseCore=0.03, streamwiseCoreVec=0.03, apparentViscCoeff=5.0,
                    symmetricTau=1)
    return Case("wing_ar4", cfg, geo)


def rotor_2blade_hover(nt: int = 1440, n_nwake: int = 260, truncate_nt: int = 432, fd_scheme: int = 3) -> Case:
    """2-blade hover rotor, R = 1 m, 1 x 24 rings/blade, dt = 5 deg, truncation at 6 revs."""
    cfg = config_text(nt=nt, dt=0.0, density=1.2, kinematicVisc=1.5e-5, fdScheme=fd_scheme, wakeDissipation=1)
    geo = geom_text(nb=2, nc=1, ns=24, nNwake=n_nwake, span=1.0, rootcut=0.2, chord=0.08, Omega=100.0,
                    shaftAxis=(0.0, 0.0, 1.0), theta0=8.0, velBody=(0.0, 0.0, 0.0), spanSpacing=1,
                    chordSpacing=1, spanwiseCore=0.05, streamwiseCoreVec=0.05, apparentViscCoeff=5.0,
                    wakeTruncateNt=truncate_nt, symmetricTau=0, pivotLE=0.25)
    return Case("rotor_2blade_hover", cfg, geo)


def plot3d_twisted_blade(nc: int, ns: int, radius: float, chord: float, root_cut: float,
                         twist_deg: float, pivot: float = 0.25) -> str:
    """PLOT3D (nx = nc+1, ny = ns+1, nz = 1) flat blade with linear twist.

    ``thetaTwist`` is read by the reference but never applied to the geometry
    (src/classdef.f90:3129), so twist enters through ``geometryFile``
    (``rotor_plot3dtoblade``, src/classdef.f90:3957-4020).  x runs from the
    leading edge (-chord) to the trailing edge (0); the section is twisted
    about the quarter chord by twist_deg * (r - r0)/(R - r0).
    """
    nx, ny = nc + 1, ns + 1
    r0 = root_cut * radius
    xs, ys, zs = [], [], []
    for j in range(ny):
        r = r0 + (radius - r0) * j / ns
        th = math.radians(twist_deg) * (r - r0) / (radius - r0)
        for i in range(nx):
            xc = -chord + chord * i / nc  # LE -> TE
            xp = -chord + pivot * chord
            dx = xc - xp
            # nose-up twist rotates the LE up (+z) for positive theta
            xs.append(xp + dx * math.cos(th))
            ys.append(r)
            zs.append(-dx * math.sin(th))
    def block(vals):
        return "\n".join(" ".join(f"{v:.15e}" for v in vals[k:k + 6]) for k in range(0, len(vals), 6))
    return f"{nx} {ny} 1\n{block(xs)}\n{block(ys)}\n{block(zs)}\n"


def rotor_4blade_forward(nt: int = 2880, n_nwake: int = 72, omega: float = 100.0, mu: float = 0.1,
                         fd_scheme: int = 3, truncate_nt: int = 0) -> Case:
    """4-blade rotor, R = 2 m, c = 0.12 m, -8 deg twist, theta0 = 10 deg, mu = 0.1, shaft tilt -4 deg."""
    radius, chord, nc, ns = 2.0, 0.12, 1, 32
    cfg = config_text(nt=nt, dt=0.0, density=1.2, kinematicVisc=1.5e-5, fdScheme=fd_scheme, wakeDissipation=1)
    geo = geom_text(nb=4, nc=nc, ns=ns, nNwake=n_nwake, span=radius, rootcut=0.2, chord=chord, Omega=omega,
                    shaftAxis=(0.0, 0.0, 1.0), theta0=10.0, velBody=(-mu * omega * radius, 0.0, 0.0),
                    phiThetaPsi=(0.0, -4.0, 0.0), geometryFile="blade.xyz", spanSpacing=1, chordSpacing=1,
                    spanwiseCore=0.05, streamwiseCoreVec=0.05, apparentViscCoeff=5.0,
                    wakeTruncateNt=truncate_nt, symmetricTau=0, pivotLE=0.25)
    return Case("rotor_4blade_forward", cfg, geo,
                files={"blade.xyz": plot3d_twisted_blade(nc, ns, radius, chord, 0.2, -8.0)})


def batch_sweep(n: int = 256, seed: int = 0, nt: Optional[int] = None) -> list:
    """Independent uneven rotor cases for the batched launch: per case (seeded)
    2-4 blades with 24-400 rings in all (1 chordwise row), R = 1-2 m,
    c = 0.08 R, collective U(2, 12) deg, advance ratio U(0, 0.3), Omega =
    100 rad/s, dt = 5 deg, one revolution of near-wake sheet and a far wake
    truncated after 1-8 revolutions (uneven filament counts of about 5k to
    120k), viscous core growth on.  Returns [Case, ...]; nt defaults to
    8 revolutions plus 36 steps (every case then in its steady state)."""
    import random

    rng = random.Random(seed)
    nt = nt if nt is not None else 8 * 72 + 36
    out = []
    for i in range(n):
        nb = rng.choice((2, 3, 4))
        rings = rng.randint(24, 400)
        ns = max(8, min(100, round(rings / nb)))
        radius = rng.uniform(1.0, 2.0)
        revs = rng.randint(1, 8)
        theta0 = rng.uniform(2.0, 12.0)
        mu = rng.uniform(0.0, 0.3)
        omega = 100.0
        cfg = config_text(nt=nt, dt=0.0, density=1.2, kinematicVisc=1.5e-5, fdScheme=3, wakeDissipation=1)
        geo = geom_text(nb=nb, nc=1, ns=ns, nNwake=72, span=radius, rootcut=0.2, chord=0.08 * radius,
                        Omega=omega, shaftAxis=(0.0, 0.0, 1.0), theta0=theta0,
                        velBody=(-mu * omega * radius, 0.0, 0.0), spanSpacing=1, chordSpacing=1,
                        spanwiseCore=0.05, streamwiseCoreVec=0.05, apparentViscCoeff=5.0,
                        wakeTruncateNt=72 * revs + (72 if revs == 1 else 0), symmetricTau=0, pivotLE=0.25)
        out.append(Case(f"sweep_{i:03d}", cfg, geo))
    return out

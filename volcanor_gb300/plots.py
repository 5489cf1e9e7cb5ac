"""The reference's plot files: wake geometry, wake tip, skew, inflow, bound
circulation and probe velocities (src/libPostprocess.f90).

Each writer takes the state the reference writes it from; the runner
(volcanor_gb300/run.py) calls them at the reference's iterations and at its
point inside the iteration:

* ``rXXwingNwakeNNNNN.tec`` (geom2file, src/libPostprocess.f90:143-331) and
  ``rXXtipNNNNN.tec`` / ``rXXtipXYZNNNNN.csv`` (tip2file, :617-784): every
  ``wakePlot`` / ``wakeTipPlot`` iterations, after the wake's shedding,
  ageing, dissipation and burst and before the circulation solve
  (src/main.f90:507-520): the wing of iteration k with the previous
  iteration's circulation, and the wake as it stands between the solve and
  the wake update (the solve does not move or change the wake);
* ``rXXbYYskewNNNNN.csv`` (skew2file, :786-812) every ``skewPlotSwitch``
  iterations at the same point (src/main.f90:497-503);
* ``rXXbYYinflowDistNNNNN.curve`` (inflow2file, :900-946) and
  ``rXXbYYgammaDistNNNNN.curve`` (gamma2file, :948-974) every
  ``inflowPlotSwitch`` / ``gammaPlotSwitch`` iterations after the loads
  (src/main.f90:764-781);
* ``probesNNNNN.csv`` (probes2file, :333-361) every ``probe`` iterations after
  the loads (src/main.f90:792-797), at the probes of ``probes.in``.

Numbers written with Fortran list-directed output use the layout the
reference's golden files show (``ld_real``: 15 significant digits in 24
columns), three to a line (list-directed records wrap at 80 columns).
Formatted records (``E15.7``, ``F15.7``) are exact.  The ``ageAzimuthal``
column of the tip file is the element's age times the current rotor speed
(the reference integrates the speed over the element's life; equal for a
constant speed).  The ``skew`` column of the near-wake zone is the current
skew when ``skewPlotSwitch`` is on (the reference writes the values of its
last skew evaluation), else 0 as the reference.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from . import lib
from .results import fortran_e

RAD2DEG = 180.0 / math.pi
EPS = np.finfo(np.float64).eps


def ld_real(x: float) -> str:
    """One REAL(8) item of list-directed output (24 columns): F-form with 15
    significant digits and 5 trailing blanks for 0.1 <= |x| < 1e15, else a
    16-digit mantissa with a signed three-digit exponent."""
    x = float(x)
    if x != 0.0 and math.isfinite(x):
        e10 = int(f"{abs(x):.14e}".split("e")[1])
        if -1 <= e10 <= 14:
            return f"{x:.{14 - e10}f}".rjust(19) + " " * 5
    if not math.isfinite(x):
        return ("NaN" if x != x else ("Infinity" if x > 0 else "-Infinity")).rjust(24)
    if x == 0.0:
        return ("0.000000000000000E+000").rjust(24)
    m, e = f"{x:.15e}".split("e")
    e = int(e)
    return f"{m}E{'-' if e < 0 else '+'}{abs(e):03d}".rjust(24)


def ld_lines(values) -> str:
    """A list-directed record of reals: a leading blank, three items a line."""
    v = [ld_real(x) for x in np.ravel(values)]
    if not v:
        return " \n"
    return "".join(" " + "".join(v[i:i + 3]) + "\n" for i in range(0, len(v), 3))


def ld_text(s: str) -> str:
    return " " + s + "\n"


def _i5(n: int) -> str:
    return f"{n:5d}".strip()


class CaseView:
    """The arrays the writers read, from a case (its getters) and the case
    files (the panel corners of iteration k, host kinematics)."""

    def __init__(self, case, config: str, geom: str, base_dir=""):
        self.case = case
        self.config, self.geom, self.base = config, geom, str(base_dir)
        g = case.geti
        self.nb, self.nc, self.ns = g("nb"), g("nc"), g("ns")
        self.NW, self.NF = g("nNwake"), g("nFwake")

    def panel_corners(self, k: int, b: int) -> np.ndarray:
        """(nc*ns, 4, 3) panel corners PC of blade b at iteration k, panel i + nc j."""
        return lib.wing_kinematics(self.config, self.geom, k, "PC", b, self.base).reshape(-1, 4, 3)

    def vind_points(self, P) -> np.ndarray:
        """Induced velocity of every wing and wake at the points P (M x 3)."""
        return self.case.vind_points(P)

    def vind_filaments(self, fc, rvc, gam, P) -> np.ndarray:
        """Induced velocity of the filaments fc (N x 2 x 3) at the points P."""
        return lib.biot_savart_filaments(fc, rvc, gam, P, lib.PREC_FP64)

    def wake_skew(self, b: int) -> np.ndarray:
        """(ns, nNwake) skew of blade b's near-wake rings (rotor_calc_skew,
        src/classdef.f90:4919-4936): blades past the convected ones of an
        axisymmetric rotor take blade 1's values."""
        c, ns, NW = self.case, self.ns, self.NW
        src = 1 if b > c.geti("nbConvect") else b
        wn = c.get("waN", src).reshape(ns, NW, 4, 3)
        wg = c.get("waN_gam", src).reshape(ns, NW)
        return ring_skew(wn.reshape(-1, 4, 3), wg.ravel()).reshape(ns, NW)


def _wing_mesh(pc: np.ndarray, nc: int, ns: int) -> np.ndarray:
    """(nc+1, ns+1, 3) mesh of panel corners (geom2file's wingMesh)."""
    P = pc.reshape(ns, nc, 4, 3)  # [j][i]
    m = np.zeros((nc + 1, ns + 1, 3))
    m[:nc, :ns] = P[:, :, 0].transpose(1, 0, 2)
    m[:nc, ns] = P[ns - 1, :, 3]
    m[nc, :ns] = P[:, nc - 1, 1]
    m[nc, ns] = P[ns - 1, nc - 1, 2]
    return m


def _zone_xyz(mesh) -> str:
    """X, Y, Z blocks of a mesh (i fastest)."""
    return "".join(ld_lines(mesh[..., a].T.ravel()) for a in range(3))


def ring_skew(corners: np.ndarray, gam: np.ndarray) -> np.ndarray:
    """vr_getBimedianCos (src/classdef.f90:704-720) of rings with |gam| > eps,
    else 0 (calc_skew, :737-747); corners (n, 4, 3)."""
    p1, p2, p3, p4 = (corners[:, k] for k in range(4))
    x1 = p3 + p4 - p1 - p2
    x2 = p4 + p1 - p2 - p3
    with np.errstate(invalid="ignore", divide="ignore"):  # rings not yet shed: all corners at 0
        c = np.abs(np.sum(x1 * x2, 1) / np.sqrt(np.sum(x1 * x1, 1) * np.sum(x2 * x2, 1)))
    return np.where(np.abs(gam) > EPS, c, 0.0)


def geom2file(path, view: CaseView, k: int, wing_gam_prev, skew_on: bool) -> Path:
    """rXXwingNwakeNNNNN.tec: per blade the wing mesh, the near wake and the
    far wake (and prescribed far wake) as Tecplot BLOCK zones."""
    c, nc, ns, NW, NF = view.case, view.nc, view.ns, view.NW, view.NF
    rowNear, rowFar = c.geti("rowNear"), c.geti("rowFar")
    o = [ld_text('Title = "Wing and Wake"'), ld_text('VARIABLES = "X" "Y" "Z" "GAM" "skew"')]
    for b in range(1, view.nb + 1):
        mesh = _wing_mesh(view.panel_corners(k, b), nc, ns)
        gam = wing_gam_prev[b - 1].reshape(ns, nc)  # [j][i]
        o.append(ld_text(f'Zone I={_i5(nc + 1)} J={_i5(ns + 1)} K=1  T="Blade {b:02d}"'))
        o.append(ld_text("DATAPACKING=BLOCK"))
        o.append(ld_text("VARLOCATION=([4]=CELLCENTERED,[5]=CELLCENTERED)"))
        o.append(_zone_xyz(mesh))
        o.append(ld_lines(-1.0 * gam.ravel()))
        o.append(ld_lines(gam.ravel() * 0.0))
        if c.geti("wakeSuppress") != 0 or NW == 0:
            continue
        wn = c.get("waN", b).reshape(ns, NW, 4, 3)
        wg = c.get("waN_gam", b).reshape(ns, NW)
        rows = NW - (rowNear - 1)
        m = np.zeros((rows + 1, ns + 1, 3))
        r0 = rowNear - 1
        m[:rows, :ns] = wn[:, r0:, 0].transpose(1, 0, 2)
        m[:rows, ns] = wn[ns - 1, r0:, 3]
        m[rows, :ns] = wn[:, NW - 1, 1]
        m[rows, ns] = wn[ns - 1, NW - 1, 2]
        skew = view.wake_skew(b) if skew_on else np.zeros((ns, NW))
        o.append(ld_text(f'Zone I={_i5(rows + 1)} J={_i5(ns + 1)} K=1  T="NearWake"'))
        o.append(ld_text("DATAPACKING=BLOCK"))
        o.append(ld_text("VARLOCATION=([4]=CELLCENTERED, [5]=CELLCENTERED)"))
        o.append(_zone_xyz(m))
        o.append(ld_lines(-1.0 * wg[:, r0:].ravel()))
        o.append(ld_lines(skew[:, r0:].ravel()))
        last = wn[ns - 1, NW - 1, 2]
        if NF > 0 and rowFar <= NF:
            wf = c.get("waF", b).reshape(NF, 2, 3)
            tip = np.concatenate([wf[rowFar - 1:, 1], wf[NF - 1:, 0]])
            o.append(ld_text(f'Zone I={_i5(NF - (rowFar - 1) + 1)} J=1   K=1   T="FarWake"'))
            o.append(ld_text("DATAPACKING=BLOCK"))
            o.append(ld_text("VARLOCATION=([4]=CELLCENTERED ,[5]=CELLCENTERED)"))
            o.append("".join(ld_lines(tip[:, a]) for a in range(3)))
            o.append(ld_lines(-1.0 * c.get("waF_gam", b)[rowFar - 1:]))
            o.append(ld_lines(c.get("waF_rvc", b)[rowFar - 1:] * 0.0))
        else:
            o += _point_zone("FarWake", last, ", [5]")
        try:
            wp = c.get("waP", b).reshape(-1, 2, 3)
            present = c.get("waP_gam", b)[0] != 0.0 or np.any(wp != 0.0)
        except KeyError:
            present = False
        if present:
            tip = np.concatenate([wp[:, 1], wp[-1:, 0]])
            o.append(ld_text(f'Zone I={_i5(len(wp) + 1)} J=1   K=1   T="PrescFarWake"'))
            o.append(ld_text("DATAPACKING=BLOCK"))
            o.append(ld_text("VARLOCATION=([4]=CELLCENTERED ,[5]=CELLCENTERED)"))
            o.append("".join(ld_lines(tip[:, a]) for a in range(3)))
            o.append(ld_lines(np.full(len(wp), -1.0 * c.get("waP_gam", b)[0])))
            o.append(ld_lines(np.full(len(wp), c.get("waP_rvc", b)[0])))
        else:
            o += _point_zone("PrescFarWake", last, ", [5]")
    p = Path(path)
    with open(p, "a") as f:  # the reference appends
        f.write("".join(o))
    return p


def _point_zone(title: str, pt, varloc: str) -> list:
    """A zone of one redundant point (no far wake present)."""
    return [ld_text(f'Zone I={_i5(2)} J=1   K=1   T="{title}"'), ld_text("DATAPACKING=BLOCK"),
            ld_text(f"VARLOCATION=([4]=CELLCENTERED{varloc}=CELLCENTERED)"),
            ld_lines([pt[0], pt[0]]), ld_lines([pt[1], pt[1]]), ld_lines([pt[2], pt[2]]),
            ld_lines([0.0]), ld_lines([0.0])]


def tip2file(tec_path, csv_path, view: CaseView, k: int, wing_gam_prev, omega: float, theta0: float):
    """rXXtipNNNNN.tec and rXXtipXYZNNNNN.csv: the wing and the rolled-up tip
    of the near wake (circulation-weighted centroid of the roll-up stations)
    and the far wake."""
    c, nc, ns, NW, NF = view.case, view.nc, view.ns, view.NW, view.NF
    rowNear, rowFar = c.geti("rowNear"), c.geti("rowFar")
    rs, re = c.geti("rollupStart"), c.geti("rollupEnd")
    speed = omega  # ageAzimuthal = age x rotor speed (signed)
    o = [ld_text('Title = "Wing and Tip"'), ld_text('VARIABLES = "X" "Y" "Z" "GAM" "ageAzimuthal"')]
    xyz = []
    for b in range(1, view.nb + 1):
        mesh = _wing_mesh(view.panel_corners(k, b), nc, ns)
        gam = wing_gam_prev[b - 1].reshape(ns, nc)
        o.append(ld_text(f'Zone I={_i5(nc + 1)} J={_i5(ns + 1)} K=1  T="Blade"'))
        o.append(ld_text("DATAPACKING=BLOCK"))
        o.append(ld_text("VARLOCATION=([4,5]=CELLCENTERED)"))
        o.append(_zone_xyz(mesh))
        o.append(ld_lines(-1.0 * gam.ravel()))
        o.append(ld_lines(np.zeros(nc * ns)))
        wn = c.get("waN", b).reshape(ns, NW, 4, 3)
        wg = c.get("waN_gam", b).reshape(ns, NW)
        age = c.get("waN_age", b).reshape(ns, NW)
        tips, groll = [], []
        sgn = math.copysign(1.0, omega * theta0) > EPS
        for i in range(rowNear - 1, NW):
            g0 = wg[ns - 1, i]
            s = np.zeros(3)
            gs = 0.0
            for j in range(rs - 1, re):
                s = s + wn[j, i, 3] * wg[j, i]
                gs = gs + wg[j, i]
                g0 = min(g0, wg[j, i]) if sgn else max(g0, wg[j, i])
            tips.append(s / gs if abs(gs) > EPS else wn[re - 1, i, 3])
            groll.append(g0)
        s = np.zeros(3)
        gs = 0.0
        for j in range(rs - 1, re):
            s = s + wn[j, NW - 1, 2] * wg[j, NW - 1]
            gs = gs + wg[j, NW - 1]
        tips.append(s / gs if abs(gs) > EPS else wn[re - 1, NW - 1, 2])
        tips = np.array(tips)
        o.append(ld_text(f'Zone I={_i5(NW - (rowNear - 1) + 1)} J=1    K=1  T="NearWake"'))
        o.append(ld_text("DATAPACKING=BLOCK"))
        o.append(ld_text("VARLOCATION=([4,5]=CELLCENTERED)"))
        o.append("".join(ld_lines(tips[:, a]) for a in range(3)))
        o.append(ld_lines(-1.0 * np.array(groll)))
        o.append(ld_lines(age[ns - 1, rowNear - 1:] * speed * RAD2DEG))
        xyz.append(ld_text("X        Y         Z"))
        xyz += [ld_lines(t) for t in tips]
        if NF > 0 and rowFar <= NF:
            wf = c.get("waF", b).reshape(NF, 2, 3)
            tip = np.concatenate([wf[rowFar - 1:, 1], wf[NF - 1:, 0]])
            o.append(ld_text(f'Zone I={_i5(NF - (rowFar - 1) + 1)} J=1   K=1   T="FarWake"'))
            o.append(ld_text("DATAPACKING=BLOCK"))
            o.append(ld_text("VARLOCATION=([4,5]=CELLCENTERED)"))
            o.append("".join(ld_lines(tip[:, a]) for a in range(3)))
            o.append(ld_lines(-1.0 * c.get("waF_gam", b)[rowFar - 1:]))
            o.append(ld_lines(c.get("waF_age", b)[rowFar - 1:] * speed * RAD2DEG))
            xyz += [ld_lines(t) for t in tip]
        else:
            pt = wn[ns - 1, NW - 1, 2]
            o += [ld_text(f'Zone I={_i5(2)} J=1   K=1   T="FarWake"'), ld_text("DATAPACKING=BLOCK"),
                  ld_text("VARLOCATION=([4,5]=CELLCENTERED)"), ld_lines([pt[0], pt[0]]), ld_lines([pt[1], pt[1]]),
                  ld_lines([pt[2], pt[2]]), ld_lines([0.0]), ld_lines([0.0])]
    with open(tec_path, "a") as f:
        f.write("".join(o))
    with open(csv_path, "a") as f:
        f.write("".join(xyz))
    return Path(tec_path), Path(csv_path)


def skew2file(path_of_blade, view: CaseView):
    """rXXbYYskewNNNNN.csv per blade: max and mean skew of every near-wake
    row, oldest first (skew2file, src/libPostprocess.f90:786-812)."""
    c, ns, NW = view.case, view.ns, view.NW
    rowNear = c.geti("rowNear")
    out = []
    for b in range(1, view.nb + 1):
        sk = view.wake_skew(b)
        lines = ["max".rjust(15) + "avg".rjust(15) + "\n"]
        for i in range(NW - 1, rowNear - 2, -1):
            tot = 0.0
            for v in sk[:, i]:
                tot = tot + v
            lines.append(fortran_e(sk[:, i].max()) + fortran_e(tot / ns) + "\n")
        p = Path(path_of_blade(b))
        p.write_text("".join(lines))
        out.append(p)
    return out


def bound_vortex_filaments(case, nb: int, nc: int, ns: int):
    """The wing's bound vortices as filaments (vind_bywing_boundVortices,
    src/classdef.f90:1376-1393): per panel filaments 2 and 4 with its
    circulation, minus filament 2 of the trailing-edge row."""
    fc, gam = [], []
    for b in range(1, nb + 1):
        vr = case.get("vr", b).reshape(ns, nc, 4, 3)
        g = case.get("gam", b).reshape(ns, nc)
        for j in range(ns):
            for i in range(nc):
                fc += [(vr[j, i, 1], vr[j, i, 2]), (vr[j, i, 3], vr[j, i, 0])]
                gam += [g[j, i], g[j, i]]
        for j in range(ns):
            fc.append((vr[j, nc - 1, 1], vr[j, nc - 1, 2]))
            gam.append(-g[j, nc - 1])
    return np.array(fc).reshape(-1, 2, 3), np.array(gam)


def inflow2file(path_of_blade, view: CaseView, direction=(0.0, 0.0, -1.0)):
    """rXXbYYinflowDistNNNNN.curve per blade: the induced velocity along
    `direction` at the section points (wing without its bound vortices,
    plus wake), against the reference's span coordinate
    dot(secCP, hub - yAxis) (inflow2file, src/libPostprocess.f90:900-946)."""
    c, nb, nc, ns = view.case, view.nb, view.nc, view.ns
    d = np.asarray(direction, dtype=float)
    wing_rvc = [c.get("vr_rvc", b).reshape(-1, 4) for b in range(1, nb + 1)]
    fc, gam = bound_vortex_filaments(c, nb, nc, ns)
    rv = []
    for b in range(1, nb + 1):
        r = wing_rvc[b - 1].reshape(ns, nc, 4)
        rv += [r[j, i, k] for j in range(ns) for i in range(nc) for k in (1, 3)]
    for b in range(1, nb + 1):
        r = wing_rvc[b - 1].reshape(ns, nc, 4)
        rv += [r[j, nc - 1, 1] for j in range(ns)]
    hub = c.get("hub")
    out = []
    for b in range(1, nb + 1):
        P = c.get("secCP", b).reshape(ns, 3)
        V = view.vind_points(P) - view.vind_filaments(fc, np.array(rv), gam, P)
        lines = ["secSpan".rjust(15) + "inflowVel".rjust(15) + "\n"]
        ya = c.get("yAxis", b)
        for j in range(ns):
            lines.append(f"{P[j] @ (hub - ya):15.7f}{V[j] @ d:15.7f}\n")
        p = Path(path_of_blade(b))
        with open(p, "a") as f:
            f.write("".join(lines))
        out.append(p)
    return out


def gamma2file(path_of_blade, view: CaseView):
    """rXXbYYgammaDistNNNNN.curve per blade: span coordinate of the first
    chordwise panel's collocation point and minus the section's summed
    circulation (gamma2file, src/libPostprocess.f90:948-974)."""
    c, nc, ns = view.case, view.nc, view.ns
    hub = c.get("hub")
    out = []
    for b in range(1, view.nb + 1):
        cp = c.get("CP", b).reshape(ns, nc, 3)
        g = c.get("gam", b).reshape(ns, nc)
        ya = c.get("yAxis", b)
        lines = [ld_text("# Row01")]
        for j in range(ns):
            d = cp[j, 0] - hub
            span = (d[0] * ya[0] + d[1] * ya[1]) + d[2] * ya[2]
            tot = 0.0
            for v in g[j]:
                tot = tot + v
            lines.append(" " + ld_real(span) + ld_real(-1.0 * tot) + "\n")
        p = Path(path_of_blade(b))
        with open(p, "a") as f:
            f.write("".join(lines))
        out.append(p)
    return out


def read_probes(path) -> tuple:
    """probes.in (src/main.f90:84-92): the probe count, then per probe its
    position and velocity (six numbers)."""
    toks = Path(path).read_text().replace(",", " ").split()
    n = int(toks[0])
    v = np.array([float(t.lower().replace("d", "e")) for t in toks[1:1 + 6 * n]]).reshape(n, 6)
    return v[:, :3], v[:, 3:]


def probes2file(path, view: CaseView, probe, probe_vel, t: float) -> Path:
    """probesNNNNN.csv: velocity (probe velocity + induced velocity of every
    wing and wake) at the probes moved to time t (probes2file,
    src/libPostprocess.f90:333-361)."""
    loc = probe + probe_vel * t
    vel = probe_vel + view.vind_points(loc)
    lines = ["".join(n.rjust(15) for n in ("u", "v", "w", "x", "y", "z")) + "\n"]
    for v, x in zip(vel, loc):
        lines.append("".join(fortran_e(a) for a in (*v, *x)) + "\n")
    p = Path(path)
    p.write_text("".join(lines))
    return p

"""Wake filament files and the Eulerian field of a wake on a Cartesian grid.

``filamentsNNNNN.dat`` is the reference's snapshot of every vortex element
of a run (filaments2file, src/libPostprocess.f90:363-473): Fortran
unformatted sequential records, as gfortran writes them (a 4-byte
little-endian length before and after each record):

    nVrWing | nVrNwake | nVfNwakeTE | nVfFwake         (default integers)
    vrWing(nVrWing), vrNwake(nVrNwake)                 (vr_class, 50 doubles)
    vfNwakeTE(nVfNwakeTE), gamNwakeTE(nVfNwakeTE)      (vf_class, 12 doubles)
    vfFwake(nVfFwake), gamFwake(nVfFwake)

vf_class = fc(3,2) (start xyz, end xyz), l0, lc, rVc0, rVc, age,
ageAzimuthal; vr_class = vf(4), gam, skew (src/classdef.f90:57-104).
:func:`filaments_from_case` takes them from a running case (the engine
keeps fc, rVc and gam of every element, and l0, lc, rVc0 and age of the far
wake; the fields it does not keep are written as zero -- gridgen reads only
fc, rVc and gam).  It reads the state between two steps: after step k's
wake convection.  The reference writes its file of iteration k inside step
k, after the loads and before that convection (src/main.f90:785-790), so a
file written here after step k holds the wake of the reference's file k
convected by one step (same elements and circulations, moved nodes).

``gridgen`` (src/gridgen.f90) reads ``gridconfig.nml`` and the filament
files of a run and writes ``Results/gridNNNNN.tec``: the induced velocity
plus a free stream at the cell centres of a Cartesian grid, evaluated here
by the GPU ring and filament kernels (``vlm_biot_savart_rings`` /
``vlm_biot_savart_filaments``).  The reference's wing loop assigns instead
of accumulating (``velCentre = vrWing(ifil)%vind(...)*gam``,
src/gridgen.f90:120-122), so its field holds only the LAST wing ring's
contribution; that is reproduced unless ``fix_wing_sum=True``.

    python -m volcanor_gb300.gridgen <case dir> [--precision fp64|fp32|fp32near] [--fix-wing-sum]
"""
from __future__ import annotations

import argparse
import re
import struct
import sys
from dataclasses import dataclass
from pathlib import Path

import numpy as np

VF = 12  # doubles per vf_class
VR = 50  # doubles per vr_class


@dataclass
class Filaments:
    vr_wing: np.ndarray    # (nVrWing, 50)
    vr_nwake: np.ndarray   # (nVrNwake, 50)
    vf_te: np.ndarray      # (nVfNwakeTE, 12)
    gam_te: np.ndarray     # (nVfNwakeTE,)
    vf_far: np.ndarray     # (nVfFwake, 12)
    gam_far: np.ndarray    # (nVfFwake,)


# ---- Fortran unformatted sequential records ------------------------------

def _record(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


def write_filaments(path, F: Filaments) -> Path:
    """Writes a filamentsNNNNN.dat file in the reference's record layout."""
    p = Path(path)
    counts = [len(F.vr_wing), len(F.vr_nwake), len(F.vf_te), len(F.vf_far)]
    parts = [_record(struct.pack("<i", c)) for c in counts]
    f64 = lambda *a: b"".join(np.ascontiguousarray(x, dtype="<f8").tobytes() for x in a)
    parts.append(_record(f64(F.vr_wing, F.vr_nwake)))
    parts.append(_record(f64(F.vf_te, F.gam_te)))
    parts.append(_record(f64(F.vf_far, F.gam_far)))
    p.write_bytes(b"".join(parts))
    return p


def read_filaments(path) -> Filaments:
    """Reads a filamentsNNNNN.dat file (the reference's or this module's)."""
    data = Path(path).read_bytes()
    recs, o = [], 0
    while o < len(data):
        (n,) = struct.unpack_from("<i", data, o)
        payload = data[o + 4:o + 4 + n]
        (n2,) = struct.unpack_from("<i", data, o + 4 + n)
        if n2 != n:
            raise ValueError(f"{path}: corrupt record markers at byte {o}")
        recs.append(payload)
        o += 8 + n
    if len(recs) != 7:
        raise ValueError(f"{path}: expected 7 records, found {len(recs)}")
    nW, nN, nT, nF = (struct.unpack("<i", r)[0] for r in recs[:4])
    a = np.frombuffer(recs[4], dtype="<f8")
    b = np.frombuffer(recs[5], dtype="<f8")
    c = np.frombuffer(recs[6], dtype="<f8")
    if a.size != VR * (nW + nN) or b.size != (VF + 1) * nT or c.size != (VF + 1) * nF:
        raise ValueError(f"{path}: record sizes do not match the counts")
    return Filaments(a[:VR * nW].reshape(nW, VR).copy(), a[VR * nW:].reshape(nN, VR).copy(),
                     b[:VF * nT].reshape(nT, VF).copy(), b[VF * nT:].copy(),
                     c[:VF * nF].reshape(nF, VF).copy(), c[VF * nF:].copy())


# ---- from a running case ---------------------------------------------------

def _vr_from_corners(corners, rvc, gam) -> np.ndarray:
    """vr_class rows from ring corners (n, 4, 3), core radii (n, 4) and gam."""
    n = corners.shape[0]
    out = np.zeros((n, VR))
    for k in range(4):
        o = VF * k
        out[:, o:o + 3] = corners[:, k]
        out[:, o + 3:o + 6] = corners[:, (k + 1) % 4]
        out[:, o + 9] = rvc[:, k]
    out[:, 48] = gam
    return out


def filaments_from_case(case) -> Filaments:
    """The elements filaments2file writes, from a case's current state: wing
    rings, all near-wake rings, the trailing filament of the last near-wake
    row (vf(2), circulation negated) and the active far-wake filaments,
    blade by blade in the reference's loop order (src/libPostprocess.f90:399-450)."""
    nb, nc, ns = case.geti("nb"), case.geti("nc"), case.geti("ns")
    NW, NF, rowFar = case.geti("nNwake"), case.geti("nFwake"), case.geti("rowFar")
    if NF == 0 or rowFar > NF:
        raise ValueError("filaments files need a developed far wake (rowFar <= nFwake), as the reference requires")
    wing, nwake, te, gte, far, gfar = [], [], [], [], [], []
    for b in range(1, nb + 1):
        wing.append(_vr_from_corners(case.get("vr", b).reshape(-1, 4, 3), case.get("vr_rvc", b).reshape(-1, 4),
                                     case.get("gam", b)))
        cN = case.get("waN", b).reshape(ns, NW, 4, 3)  # [j][i]: ring (i, j) at index i + NW j
        rN = case.get("waN_rvc", b).reshape(ns, NW, 4)
        gN = case.get("waN_gam", b).reshape(ns, NW)
        vr = _vr_from_corners(cN.reshape(-1, 4, 3), rN.reshape(-1, 4), gN.reshape(-1))
        vr[:, [VF * k + 10 for k in range(4)]] = case.get("waN_age", b)[:, None]
        nwake.append(vr)
        t = np.zeros((ns, VF))
        t[:, 0:3] = cN[:, NW - 1, 1]
        t[:, 3:6] = cN[:, NW - 1, 2]
        t[:, 9] = rN[:, NW - 1, 1]
        te.append(t)
        gte.append(-1.0 * gN[:, NW - 1])
        fC = case.get("waF", b).reshape(NF, 2, 3)[rowFar - 1:]
        f = np.zeros((fC.shape[0], VF))
        f[:, 0:6] = fC.reshape(-1, 6)
        for col, name in ((6, "waF_l0"), (7, "waF_lc"), (8, "waF_rvc0"), (9, "waF_rvc"), (10, "waF_age")):
            f[:, col] = case.get(name, b)[rowFar - 1:]
        far.append(f)
        gfar.append(case.get("waF_gam", b)[rowFar - 1:])
    cat = lambda x, w: np.concatenate(x) if x else np.zeros((0, w))
    return Filaments(cat(wing, VR), cat(nwake, VR), cat(te, VF), np.concatenate(gte), cat(far, VF),
                     np.concatenate(gfar))


# ---- gridconfig.nml and the grid ------------------------------------------

def read_gridconfig(text: str) -> dict:
    """The INPUTS of gridconfig.nml (template version 0.2, src/gridgen.f90:27-44)."""
    body = re.sub(r"!.*", "", text)
    vals = {}
    for key, rhs in re.findall(r"(\w+)\s*=\s*([^=]*?)(?=,?\s*\w+\s*=|/|$)", body, flags=re.S):
        items = [v.strip().strip("'\"") for v in rhs.replace("\n", " ").split(",") if v.strip()]
        vals[key.lower()] = items
    ver = vals.get("fileformatversion", [""])[0]
    if ver != "0.2":
        raise ValueError("gridconfig.nml template version does not match")
    num = lambda s: float(s.lower().replace("d", "e"))
    cfg = {k: int(vals[k][0]) for k in ("nx", "ny", "nz", "filerangestart", "filerangestep", "filerangeend")}
    for k in ("xyzmin", "xyzmax", "vel"):
        cfg[k] = np.array([num(v) for v in vals[k]][:3])
    if np.any(cfg["xyzmin"] > cfg["xyzmax"]):
        raise ValueError("all xyzMin values must not exceed the xyzMax values")
    return cfg


def linspace(a: float, b: float, n: int) -> np.ndarray:
    """libMath linspace (src/libMath.f90:138-157): i*dx + start."""
    dx = (b - a) / (n - 1)
    return np.arange(n, dtype=np.float64) * dx + a


def grid_and_centres(cfg: dict):
    """grid (3, nx, ny, nz) and the cell centres (3, nx-1, ny-1, nz-1), the
    eight corners summed in the reference's order and scaled by 0.125
    (src/gridgen.f90:67-86)."""
    nx, ny, nz = cfg["nx"], cfg["ny"], cfg["nz"]
    xv, yv, zv = (linspace(cfg["xyzmin"][k], cfg["xyzmax"][k], n) for k, n in enumerate((nx, ny, nz)))
    g = np.empty((3, nx, ny, nz))
    g[0] = xv[:, None, None]
    g[1] = yv[None, :, None]
    g[2] = zv[None, None, :]
    c = (g[:, :-1, :-1, :-1] + g[:, 1:, :-1, :-1] + g[:, 1:, 1:, :-1] + g[:, 1:, 1:, 1:] + g[:, :-1, 1:, :-1]
         + g[:, :-1, 1:, 1:] + g[:, :-1, :-1, 1:] + g[:, 1:, :-1, 1:])
    return g, c * 0.125


def _rings(vr: np.ndarray):
    corners = np.stack([vr[:, VF * k:VF * k + 3] for k in range(4)], axis=1)
    rvc = np.stack([vr[:, VF * k + 9] for k in range(4)], axis=1)
    return corners, rvc, vr[:, 48]


def evaluate(F: Filaments, points: np.ndarray, vel, precision: int = 0, fix_wing_sum: bool = False) -> np.ndarray:
    """Velocity at points (M, 3): wing (the last ring only, as the reference,
    unless fix_wing_sum) + near-wake rings + trailing filaments + far-wake
    filaments + the free stream, on the GPU."""
    from . import lib
    P = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    V = np.zeros_like(P)
    wing = F.vr_wing if fix_wing_sum else F.vr_wing[-1:]
    for vr in (wing, F.vr_nwake):
        if len(vr):
            V += lib.biot_savart_rings(*_rings(vr), P, precision)
    for vf, g in ((F.vf_te, F.gam_te), (F.vf_far, F.gam_far)):
        if len(vf):
            V += lib.biot_savart_filaments(vf[:, 0:6].reshape(-1, 2, 3), vf[:, 9], g, P, precision)
    return V + np.asarray(vel, dtype=np.float64)[None, :]


def _values(a: np.ndarray, per_line: int = 5) -> str:
    """Values in Fortran order, written list-directed style (several per line)."""
    flat = np.asarray(a, dtype=np.float64).reshape(-1, order="F")
    lines = [" ".join(f"{v: .15E}" for v in flat[k:k + per_line]) for k in range(0, flat.size, per_line)]
    return "\n".join(" " + ln for ln in lines)


def write_tec(path, grid: np.ndarray, vel_centre: np.ndarray) -> Path:
    """gridNNNNN.tec (src/gridgen.f90:148-163): Tecplot BLOCK data, grid
    nodes and cell-centred U, V, W."""
    _, nx, ny, nz = grid.shape
    head = [' TITLE = "Grid"', ' VARIABLES = "X" "Y" "Z" "U" "V" "W"',
            f' ZONE I={nx} J={ny} K={nz} T="Data"', " DATAPACKING=BLOCK",
            " VARLOCATION=([4]=CELLCENTERED,[5]=CELLCENTERED,[6]=CELLCENTERED)"]
    body = [_values(grid[k]) for k in range(3)] + [_values(vel_centre[k]) for k in range(3)]
    p = Path(path)
    p.write_text("\n".join(head + body) + "\n")
    return p


def run(case_dir, precision: int = 0, fix_wing_sum: bool = False) -> list:
    """gridgen over a case directory: every filament file of the configured
    range -> Results/gridNNNNN.tec.  Returns the written paths."""
    d = Path(case_dir)
    cfg = read_gridconfig((d / "gridconfig.nml").read_text())
    grid, centres = grid_and_centres(cfg)
    pts = np.moveaxis(centres, 0, -1).reshape(-1, 3, order="C")
    out = []
    for it in range(cfg["filerangestart"], cfg["filerangeend"] + 1, cfg["filerangestep"]):
        F = read_filaments(d / "Results" / f"filaments{it:05d}.dat")
        V = evaluate(F, pts, cfg["vel"], precision, fix_wing_sum)
        vc = np.moveaxis(V.reshape(centres.shape[1:] + (3,)), -1, 0)
        dst = d / "Results" / f"grid{it:05d}.tec"
        if dst.exists():
            raise FileExistsError(f"{dst} exists (the reference opens it with status='new')")
        out.append(write_tec(dst, grid, vc))
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("case_dir")
    ap.add_argument("--precision", choices=["fp64", "fp32", "fp32near"], default="fp64")
    ap.add_argument("--fix-wing-sum", action="store_true")
    a = ap.parse_args(argv)
    prec = {"fp64": 0, "fp32": 1, "fp32near": 2}[a.precision]
    for p in run(a.case_dir, prec, a.fix_wing_sum):
        print(p)
    return 0


if __name__ == "__main__":
    sys.exit(main())

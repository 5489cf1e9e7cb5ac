"""Host side of the filament files and gridgen: the reference's record
layout (write -> read round trip, record markers), gridconfig.nml parsing,
the grid and its cell centres, and the oracle's filament sum."""
import struct

import numpy as np
import pytest

from volcanor_gb300 import gridgen as G


def _random_filaments(rng, nW=3, nN=5, nT=2, nF=4):
    return G.Filaments(rng.normal(size=(nW, 50)), rng.normal(size=(nN, 50)), rng.normal(size=(nT, 12)),
                       rng.normal(size=nT), rng.normal(size=(nF, 12)), rng.normal(size=nF))


def test_filament_file_round_trip_and_layout(tmp_path):
    F = _random_filaments(np.random.default_rng(0))
    p = G.write_filaments(tmp_path / "filaments00010.dat", F)
    data = p.read_bytes()
    # four integer records (4-byte marker, int32, marker), then three real ones
    for r in range(4):
        n1, val, n2 = struct.unpack_from("<iii", data, 12 * r)
        assert n1 == n2 == 4
        assert val == [3, 5, 2, 4][r]
    assert struct.unpack_from("<i", data, 48)[0] == 8 * 50 * (3 + 5)
    assert len(data) == 48 + 3 * 8 + 8 * (50 * 8 + 13 * 2 + 13 * 4)
    G2 = G.read_filaments(p)
    for a, b in zip(vars(F).values(), vars(G2).values()):
        np.testing.assert_array_equal(a, b)


def test_filament_file_rejects_corrupt_markers(tmp_path):
    F = _random_filaments(np.random.default_rng(1))
    p = G.write_filaments(tmp_path / "f.dat", F)
    b = bytearray(p.read_bytes())
    b[-1] ^= 0x7F
    p.write_bytes(bytes(b))
    with pytest.raises(ValueError):
        G.read_filaments(p)


GRIDCONFIG = """&VERSION
fileFormatVersion = 0.2
/
! comment line
&INPUTS
nx = 5
ny = 4
nz = 3
xyzMin = -1.0, -2.0, 0.5
xyzMax = 1.0, 2.0, 1.5
vel = 0.0, -6.0, -3.0d0
fileRangeStart = 20
fileRangeStep = 10
fileRangeEnd = 40
/
"""


def test_gridconfig_and_grid_centres():
    cfg = G.read_gridconfig(GRIDCONFIG)
    assert (cfg["nx"], cfg["ny"], cfg["nz"]) == (5, 4, 3)
    assert (cfg["filerangestart"], cfg["filerangestep"], cfg["filerangeend"]) == (20, 10, 40)
    np.testing.assert_array_equal(cfg["vel"], [0.0, -6.0, -3.0])
    g, c = G.grid_and_centres(cfg)
    assert g.shape == (3, 5, 4, 3) and c.shape == (3, 4, 3, 2)
    # libMath linspace: i*dx + start
    dx = (1.0 - -1.0) / 4
    np.testing.assert_array_equal(g[0, :, 0, 0], np.arange(5) * dx + -1.0)
    ref = np.zeros_like(c)
    for a in (0, 1):
        for b in (0, 1):
            for e in (0, 1):
                ref += g[:, a:a + 4, b:b + 3, e:e + 2]
    np.testing.assert_allclose(c, ref * 0.125, rtol=1e-15, atol=1e-15)
    with pytest.raises(ValueError):
        G.read_gridconfig(GRIDCONFIG.replace("0.2", "0.1"))


def test_oracle_filament_sum_is_the_vf_vind_loop():
    from oracle import oracle as O
    rng = np.random.default_rng(2)
    fc = rng.uniform(-1, 1, (7, 2, 3))
    rvc = rng.uniform(0.01, 0.1, 7)
    gam = rng.normal(size=7)
    P = rng.uniform(-1, 1, (5, 3))
    V = O.vind_filaments(fc, rvc, gam, P)
    for m in range(5):
        acc = np.zeros(3)
        for n in range(7):
            acc = acc + O.vf_vind(fc[n, 0], fc[n, 1], rvc[n], P[m]) * gam[n]
        np.testing.assert_array_equal(V[m], acc)

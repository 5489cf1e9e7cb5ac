"""Coupled rotors (nr > 1, vlm_system_*) on the GPU against the oracle's
system of rotors (oracle/vlm_oracle.cpp System: src/main.f90's loop with
every induced-velocity sum over all rotors): FP64 bit for bit with equal
summation blocks, the FP32 forms within the CT tolerance of the solver
tests, a lone rotor as a system equal to the case, and the rotor handles'
stepping calls refused."""
import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu

CHUNK = 16


def oracle_system(sc, steps):
    O.set_threads(8)
    y = O.System(sc.config, sc.geoms)
    y.set_sum_chunk(CHUNK)
    y.start()
    y.step(steps)
    return y


def gpu_system(sc, steps, precision=lib.PREC_FP64, **kw):
    y = lib.System(sc.config, sc.geoms, precision=precision, sum_chunk=CHUNK, **kw)
    y.start()
    rows = y.step(steps)
    return y, rows


def assert_same_state(g, o, nb):
    np.testing.assert_array_equal(g.ct_hist(), o.ct_hist())
    np.testing.assert_array_equal(g.get("gamVec"), o.get("gamVec"))
    for b in range(1, nb + 1):
        # the library stores a ring's 4 corners, the oracle its 4 filaments' ends
        np.testing.assert_array_equal(g.get("waN", b).reshape(-1, 4, 3),
                                      o.get("waN", b).reshape(-1, 4, 2, 3)[:, :, 0])
        for name in ("waN_gam", "waN_rvc", "waF", "waF_gam", "velCP", "velCPTotal"):
            np.testing.assert_array_equal(g.get(name, b), o.get(name, b), err_msg=name)


def test_coaxial_pair_fp64_bitwise():
    """Counter-rotating coaxial rotors through roll-up and truncation."""
    sc = C.rotor_pair(nt=60)
    o = oracle_system(sc, 60)
    g, rows = gpu_system(sc, 60)
    for ir in range(2):
        assert_same_state(g.rotors[ir], o.rotors[ir], 2)
        assert np.array_equal(rows[:, ir, :], o.rotors[ir].ct_hist()[1:])
    # the coupling is not negligible: the lower rotor's CT moves by percents
    iso = O.Sim(sc.config.replace("nr = 2", "nr = 1"), sc.geoms[1])
    iso.set_sum_chunk(CHUNK)
    iso.start()
    iso.step(60)
    assert np.max(np.abs(iso.ct_hist()[-10:, 1] / rows[-10:, 1, 1] - 1)) > 0.02


@pytest.mark.parametrize("fd", [0, 1, 2, 4, 5])
def test_side_by_side_every_scheme_fp64_bitwise(fd):
    """Two co-rotating rotors side by side, every finite-difference scheme."""
    sc = C.rotor_pair(nt=14, n_nwake=8, truncate_nt=10, hub1=(1.3, 0.0, 0.0), hub2=(-1.3, 0.0, 0.0), omega2=100.0,
                      fd_scheme=fd)
    o = oracle_system(sc, 14)
    g, _ = gpu_system(sc, 14)
    for ir in range(2):
        assert_same_state(g.rotors[ir], o.rotors[ir], 2)


def test_symmetric_pair_equal_loads():
    """Rotors at (+-1.3, 0, 0) turning the same way map onto each other by a
    half turn about the shaft: equal CT to rounding (not bitwise: the two sum
    each other's records in different orders)."""
    sc = C.rotor_pair(nt=40, hub1=(1.3, 0.0, 0.0), hub2=(-1.3, 0.0, 0.0), omega2=100.0)
    _, rows = gpu_system(sc, 40)
    a, b = rows[:, 0, 1], rows[:, 1, 1]
    assert np.max(np.abs(a - b) / np.abs(a)) < 1e-12


@pytest.mark.parametrize("prec", [lib.PREC_FP32, lib.PREC_FP32_NEAR64])
def test_fp32_forms_within_ct_tolerance(prec):
    sc = C.rotor_pair(nt=40)
    _, r64 = gpu_system(sc, 40)
    _, r32 = gpu_system(sc, 40, precision=prec)
    rel = np.abs(r32[:, :, 1] - r64[:, :, 1]) / np.abs(r64[:, :, 1])
    assert rel.max() < 1e-4, rel.max()


def test_lone_rotor_system_equals_case():
    c = C.rotor_2blade_hover(nt=30, n_nwake=10, truncate_nt=16)
    y = lib.System(c.config, [c.geom], precision=lib.PREC_FP64, sum_chunk=CHUNK)
    y.start()
    ry = y.step(30)
    k = lib.Case(c.config, c.geom, precision=lib.PREC_FP64, sum_chunk=CHUNK)
    k.start()
    rk = k.step(30)
    assert np.array_equal(ry[:, 0, :], rk)
    assert np.array_equal(y.rotors[0].get("waN", 1), k.get("waN", 1))


def test_case_directory_and_rotor_handles(tmp_path):
    """vlm_system_create_from_dir reads nr from config.nml and geom01..geomNN;
    a rotor's case handle refuses the single-case stepping calls."""
    sc = C.rotor_pair(nt=6, n_nwake=4, truncate_nt=0)
    d = sc.write(tmp_path / "pair")
    L = lib.load()
    h = lib._vp()
    opt = lib.options(lib.PREC_FP64, CHUNK, use_graph=False)
    lib._err(L.vlm_system_create_from_dir(str(d).encode(), lib.ctypes.byref(opt), lib.ctypes.byref(h)))
    try:
        assert L.vlm_system_rotor_count(h) == 2
        r0 = lib._vp()
        lib._err(L.vlm_system_rotor(h, 0, lib.ctypes.byref(r0)))
        assert L.vlm_case_start(r0) == STATE
        assert L.vlm_case_step(r0, 1, None) == STATE
        lib._err(L.vlm_system_start(h))
        rows = np.zeros((6, 2, 10))
        lib._err(L.vlm_system_step(h, 6, lib._ptr(rows)))
        _, ref = gpu_system(sc, 6)
        assert np.array_equal(rows, ref)
    finally:
        L.vlm_system_destroy(h)


STATE = 7  # VLM_ERR_STATE (include/vlm.h)


@pytest.mark.parametrize("fd,nt", [(3, 40), (1, 16), (0, 16)])
def test_ground_effect_image_rotor_fp64_bitwise(fd, nt):
    """A hover rotor 0.6 R above the ground and its image (surfaceType -1,
    imagePlane 3): the image's circulation, velCP and wake mirror the
    rotor's; every rotor's state and loads are the oracle's bit for bit."""
    sc = C.rotor_ground_effect(height=0.6, nt=nt, fd_scheme=fd)
    o = oracle_system(sc, nt)
    g, rows = gpu_system(sc, nt)
    for ir in range(2):
        assert_same_state(g.rotors[ir], o.rotors[ir], 2)
    np.testing.assert_array_equal(g.rotors[1].get("gamVec"), -g.rotors[0].get("gamVec"))
    wa, wb = g.rotors[0].get("waN", 1).reshape(-1, 3), g.rotors[1].get("waN", 1).reshape(-1, 3)
    np.testing.assert_array_equal(wb[:, :2], wa[:, :2])
    np.testing.assert_array_equal(wb[:, 2], -wa[:, 2])


def test_ground_effect_fp32_within_ct_tolerance():
    sc = C.rotor_ground_effect(height=0.6, nt=40)
    _, r64 = gpu_system(sc, 40)
    _, r32 = gpu_system(sc, 40, precision=lib.PREC_FP32_NEAR64)
    rel = np.abs(r32[:, 0, 1] - r64[:, 0, 1]) / np.abs(r64[:, 0, 1])
    assert rel.max() < 1e-4, rel.max()

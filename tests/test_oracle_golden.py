"""Pin the oracle to the reference's own golden vectors.

Every expected value below is transcribed from the reference's tests
(tests/*_test.f90, tolerance ``tol = 1.E-6`` from src/classdef.f90:10) or
read from its full-case reference results (tests/*.case/referenceResults,
printed with 7 significant digits by src/libPostprocess.f90:822-838).
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C

TOL = 1e-6  # src/classdef.f90:10


def _wing(nc, ns, chord, theta0, vel):
    # tests/wing1x2_test.f90:16-70 and tests/wing1x3_test.f90:16-75
    cfg = C.config_text(nt=1, dt=0.00625, density=1.2, fdScheme=3)
    geo = C.geom_text(nb=1, nc=nc, ns=ns, nNwake=2, surfaceType=1, span=2.0, rootcut=0.0, chord=chord,
                      Omega=0.0, shaftAxis=(0.0, 0.0, 0.0), theta0=theta0, velBody=(vel, 0.0, 0.0), pivotLE=0.25,
                      symmetricTau=1, apparentViscCoeff=5.0, spanwiseCore=0.04, streamwiseCoreVec=0.04,
                      spanSpacing=2, chordSpacing=1)
    return O.Sim(cfg, geo)


def _rotor(omega, theta0):
    # tests/rotor1x2_test.f90:13-80 (dt is the single precision literal -0.014)
    cfg = C.config_text(nt=1, dt=float(np.float32(-0.014)), density=1.2, fdScheme=3, wakeDissipation=1)
    geo = C.geom_text(nb=1, nc=1, ns=2, nNwake=2, surfaceType=1, span=2.0, rootcut=0.5, chord=1.0, Omega=omega,
                      shaftAxis=(0.0, 0.0, 1.0), theta0=theta0, velBody=(0.0, 0.0, 0.0), pivotLE=0.25,
                      symmetricTau=0, apparentViscCoeff=1.0, spanwiseCore=0.04, streamwiseCoreVec=0.04,
                      spanSpacing=2, chordSpacing=1)
    s = O.Sim(cfg, geo)
    th = s.gettheta(0.0, 1)
    s.set_blade_theta(1, th)
    s.rot_pitch(1, math.copysign(1.0, omega) * th)
    return s


def test_wing1x2_coords_aic_force():
    s = _wing(1, 2, 1.0, 5.0, -10.0)
    pc = s.get("PC").reshape(2, 4, 3)
    # tests/wing1x2_test.f90:79-101
    np.testing.assert_allclose(pc[0], [[-1, 0, 0], [0, 0, 0], [0, 1, 0], [-1, 1, 0]], atol=TOL)
    np.testing.assert_allclose(pc[1], [[-1, 1, 0], [0, 1, 0], [0, 2, 0], [-1, 2, 0]], atol=TOL)
    vr = s.get("vr").reshape(2, 4, 2, 3)[:, :, 0]
    # tests/wing1x2_test.f90:103-149
    np.testing.assert_allclose(vr[0], [[-0.75, 0, 0], [0.01875, 0, 0], [0.01875, 1, 0], [-0.75, 1, 0]], atol=TOL)
    np.testing.assert_allclose(vr[1], [[-0.75, 1, 0], [0.01875, 1, 0], [0.01875, 2, 0], [-0.75, 2, 0]], atol=TOL)
    # tests/wing1x2_test.f90:151-157
    np.testing.assert_allclose(s.get("CP").reshape(2, 3), [[-0.25, 0.5, 0], [-0.25, 1.5, 0]], atol=TOL)
    # tests/wing1x2_test.f90:159-171
    s.calc_aic()
    np.testing.assert_allclose(s.get("AIC").reshape(2, 2, order="F"),
                               [[1.1223476, -9.2667149e-2], [-9.2667149e-2, 1.1223476]], atol=TOL)
    # tests/wing1x2_test.f90:173-275
    s.rot_pitch(1, s.gettheta(0.0, 1))
    d = math.radians(5.0)
    np.testing.assert_allclose(s.get("nCap").reshape(2, 3), [[math.sin(d), 0, math.cos(d)]] * 2, atol=TOL)
    s.test_freestream(False)
    s.dir_lift_drag()
    np.testing.assert_allclose(s.get("secLiftDir").reshape(2, 3), [[0, 0, 1]] * 2, atol=TOL)
    np.testing.assert_allclose(s.get("secDragDir").reshape(2, 3), [[1, 0, 0]] * 2, atol=TOL)
    s.calc_sec_alpha()
    np.testing.assert_allclose(s.get("secTheta"), [d, d], atol=TOL)
    np.testing.assert_allclose(s.get("secAlpha"), [d, d], atol=TOL)
    s.calc_force()
    np.testing.assert_allclose(s.get("delP"), [91.3763089754279] * 2, atol=TOL)
    nf = [7.96397007829292, 0.0, 91.0285945325144]
    np.testing.assert_allclose(s.get("normalForce").reshape(2, 3), [nf, nf], atol=TOL)
    np.testing.assert_allclose(s.get("secForceInertial").reshape(2, 3), [nf, nf], atol=TOL)
    np.testing.assert_allclose(s.get("secLift").reshape(2, 3), [[0, 0, nf[2]]] * 2, atol=TOL)
    np.testing.assert_allclose(s.get("secLiftOutPlane").reshape(2, 3), [[0, 0, nf[2]]] * 2, atol=TOL)
    np.testing.assert_allclose(s.get("secLiftInPlane").reshape(2, 3), [[0, 0, 0]] * 2, atol=TOL)
    np.testing.assert_allclose(s.get("secCL"), [1.51714324220857] * 2, atol=TOL)
    np.testing.assert_allclose(s.get("forceInertial"), [15.9279401565858, 0, 182.057189065029], atol=TOL)
    np.testing.assert_allclose(s.get("lift"), [0, 0, 182.057189065029], atol=TOL)


@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_wing1x3_and_negpitch(sign):
    # tests/wing1x3_test.f90:74-198 and tests/wing1x3NegPitch_test.f90
    s = _wing(1, 3, 0.3, 7.0 * sign, -6.0)
    s.calc_aic()
    aic = [[3.18902463326559, -0.135541879282409, -0.002934863377599825],
           [-0.02762714554230721, 2.97991717943654, -0.02762714554230732],
           [-0.002934863377599823, -0.135541879282409, 3.18902463326559]]
    np.testing.assert_allclose(s.get("AIC").reshape(3, 3, order="F"), aic, atol=TOL)
    s.rot_pitch(1, s.gettheta(0.0, 1))
    ct, st = math.cos(math.radians(7.0)), math.sin(math.radians(7.0))
    np.testing.assert_allclose(s.get("nCap").reshape(3, 3), [[sign * st, 0, ct]] * 3, atol=TOL)
    s.test_freestream(False)
    np.testing.assert_allclose(s.get("gamVec"), sign * np.array([-0.240131, -0.249833, -0.240131]), atol=TOL)
    s.dir_lift_drag()
    np.testing.assert_allclose(s.get("secLiftDir").reshape(3, 3), [[0, 0, 1]] * 3, atol=TOL)
    np.testing.assert_allclose(s.get("secDragDir").reshape(3, 3), [[1, 0, 0]] * 3, atol=TOL)
    s.calc_force()
    np.testing.assert_allclose(s.get("delP"), sign * np.array([28.7727659410054, 29.9353746086400, 28.7727659410054]),
                               atol=TOL)
    nf = np.array([[0.525977713977048, 0.0, 4.28374471602321], [1.09446133444262, 0.0, 8.91367225972409],
                   [0.525977713977048, 0.0, 4.28374471602321]])
    nf[:, 2] *= sign
    tol_nf = TOL if sign > 0 else 1e-6 + 5e-7  # NegPitch vectors carry 7 digits
    np.testing.assert_allclose(s.get("normalForce").reshape(3, 3), nf, atol=tol_nf)
    np.testing.assert_allclose(s.get("secForceInertial").reshape(3, 3), nf, atol=tol_nf)
    np.testing.assert_allclose(s.get("secLift").reshape(3, 3), np.c_[np.zeros((3, 2)), nf[:, 2]], atol=tol_nf)
    np.testing.assert_allclose(s.get("secCL"), sign * np.array([1.32214343087136, 1.37556670674755, 1.32214343087136]),
                               atol=tol_nf)
    np.testing.assert_allclose(s.get("forceInertial"), [2.14641676239672, 0, sign * 17.4811616917705], atol=tol_nf)
    np.testing.assert_allclose(s.get("lift"), [0, 0, sign * 17.4811616917705], atol=tol_nf)


@pytest.mark.parametrize("variant", ["rotor1x2", "rotor1x2Rev", "rotor1x2NegPitch"])
def test_rotor1x2_family(variant):
    # tests/rotor1x2_test.f90, rotor1x2Rev_test.f90, rotor1x2NegPitch_test.f90
    omega = -100.0 if variant == "rotor1x2Rev" else 100.0
    pitch = -5.0 if variant == "rotor1x2NegPitch" else 5.0
    s = _rotor(omega, pitch)
    np.testing.assert_allclose(s.get("dt"), [8.7964597e-4], atol=TOL)
    th = math.radians(pitch)
    ct, st = math.cos(th), math.sin(th)
    xs = 1.0 if variant == "rotor1x2Rev" else -1.0
    pc = s.get("PC").reshape(2, 4, 3)
    exp1 = [[xs * (0.75 + 0.25 * ct), 1.0, 0.25 * st], [xs * (0.75 - 0.75 * ct), 1.0, -0.75 * st],
            [xs * (0.75 - 0.75 * ct), 1.5, -0.75 * st], [xs * (0.75 + 0.25 * ct), 1.5, 0.25 * st]]
    np.testing.assert_allclose(pc[0], exp1, atol=TOL)
    vr = s.get("vr").reshape(2, 4, 2, 3)[:, :, 0]
    zs = 6.59418e-2 if variant == "rotor1x2NegPitch" else -6.59418e-2
    np.testing.assert_allclose(vr[0], [[xs * 0.75, 1.0, 0.0], [-xs * 3.71826e-3, 1.0, zs],
                                       [-xs * 3.71826e-3, 1.5, zs], [xs * 0.75, 1.5, 0.0]], atol=TOL)
    nx = -st if variant == "rotor1x2Rev" else st
    np.testing.assert_allclose(s.get("nCap").reshape(2, 3), [[nx, 0.0, ct]] * 2, atol=TOL)
    s.calc_aic()
    a, b = 1.600113, -0.281091
    if variant == "rotor1x2Rev":
        a, b = -a, -b
    np.testing.assert_allclose(s.get("AIC").reshape(2, 2, order="F"), [[a, b], [b, a]], atol=TOL)
    s.test_freestream(True)
    g = np.array([-8.753162, -11.069649]) * (-1.0 if variant != "rotor1x2" else 1.0)
    np.testing.assert_allclose(s.get("gamVec"), g, atol=TOL)
    s.dir_lift_drag()
    np.testing.assert_allclose(s.get("secLiftDir").reshape(2, 3), [[0, 0, 1]] * 2, atol=TOL)
    dd = -1.0 if variant == "rotor1x2Rev" else 1.0
    np.testing.assert_allclose(s.get("secDragDir").reshape(2, 3), [[dd, 0, 0]] * 2, atol=TOL)
    s.calc_sec_alpha()
    np.testing.assert_allclose(s.get("secTheta"), [th, th], atol=TOL)
    np.testing.assert_allclose(s.get("secAlpha"), [th, th], atol=TOL)
    s.calc_force()
    sd = -1.0 if variant == "rotor1x2NegPitch" else 1.0
    np.testing.assert_allclose(s.get("delP"), sd * np.array([7278.445742, 9866.306155]), atol=TOL)
    sx = -1.0 if variant == "rotor1x2Rev" else 1.0
    nf = np.array([[sx * 317.179172, 0.0, sd * 3625.374529], [sx * 429.952620, 0.0, sd * 4914.380941]])
    np.testing.assert_allclose(s.get("normalForce").reshape(2, 3), nf, atol=TOL)
    np.testing.assert_allclose(s.get("secForceInertial").reshape(2, 3), nf, atol=TOL)
    np.testing.assert_allclose(s.get("secLift").reshape(2, 3), np.c_[np.zeros((2, 2)), nf[:, 2]], atol=TOL)
    np.testing.assert_allclose(s.get("secCL"), sd * np.array([0.773413, 0.534898]), atol=TOL)
    np.testing.assert_allclose(s.get("forceInertial"), nf.sum(0), atol=TOL)
    np.testing.assert_allclose(s.get("lift"), [0, 0, nf[:, 2].sum()], atol=TOL)


def test_libmath_inverse_and_matvec():
    # tests/libMath_test.f90:64-95
    mat = np.array([[1.0, -1.0, 2.0], [4.0, 0.0, 6.0], [0.0, 1.0, -1.0]])
    truth = np.array([[3.0, -0.5, 3.0], [-2.0, 0.5, -1.0], [-2.0, 0.5, -2.0]])
    np.testing.assert_allclose(O.inv2(mat), truth, atol=1e-6)
    np.testing.assert_allclose(O.matvec(mat, [1.0, 2.0, 3.0]), [5.0, 22.0, -1.0], atol=1e-6)


def test_inverse_matches_lapack():
    """The restated DGETRF+DGETRI inverse agrees with LAPACK on a random AIC-like matrix."""
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(3)
    a = rng.normal(size=(40, 40)) + 40 * np.eye(40)
    lu, piv, info = scipy_linalg.lapack.dgetrf(a)
    inv, info2 = scipy_linalg.lapack.dgetri(lu, piv)
    assert info == 0 and info2 == 0
    np.testing.assert_allclose(O.inv2(a), inv, rtol=0, atol=1e-14)


def _ct_check(case_dir, nsteps, rel_tol=5.1e-7):
    s = O.Sim.from_case_dir(case_dir)
    s.start()
    s.step(nsteps)
    ct = s.ct_hist()
    ref = np.loadtxt(case_dir / "r01ForceNonDim.csv.ref", skiprows=1)[: nsteps + 1]
    assert ct.shape[0] == nsteps + 1
    np.testing.assert_array_equal(ct[:, 0], ref[:, 0])
    # E15.7 output: 7 significant digits -> relative rounding <= 5e-7
    rel = np.abs(ct[:, 1] - ref[:, 1]) / np.abs(ref[:, 1])
    assert rel.max() <= rel_tol, (rel.max(), int(rel.argmax()))
    # remaining columns (CLu, CFx..CFz): printed precision of each value, plus
    # a floor of 2e-7 x |CL/CT| because CLu and the small force components are
    # differences of nearly equal terms (gamTrapz - gamPrev, projections)
    for col in (3, 7, 8, 9):
        bound = 5.1e-7 * np.abs(ref[:, col]) + 2e-7 * np.abs(ref[:, 1])
        assert np.all(np.abs(ct[:, col] - ref[:, col]) <= bound), (col, np.abs(ct[:, col] - ref[:, col]).max())
    return s, ct, ref


def test_katz_plotkin_ar4_first_steps(golden_dir):
    """tests/katzNplotkin-AR04.case: fixed wing, AM2 convection, CT history rows 0..40."""
    _ct_check(golden_dir / "katzNplotkin-AR04", 40)


def test_elevate_rotor_first_steps(golden_dir):
    """tests/elevateTest.case: 5-blade PLOT3D rotor (axisymmetry, dissipation), rows 0..40 (past rollup)."""
    s, _, _ = _ct_check(golden_dir / "elevateTest", 40)
    assert s.geti("wakeTruncateNt") == 75  # r01Params.json.ref
    np.testing.assert_allclose(s.get("dt"), [2.793147502635958e-3], rtol=1e-15)
    np.testing.assert_allclose(s.get("nonDimDenom"), [15897245.0107259], rtol=1e-14)


@pytest.mark.slow
def test_katz_plotkin_ar4_full(golden_dir):
    """All 161 CT rows plus the sectional distribution at step 160 (tests/test_katzNplotkinAR04.py)."""
    s, ct, ref = _ct_check(golden_dir / "katzNplotkin-AR04", 160)
    # testCT: last value and mean of the last ten, places=6
    assert abs(ct[-1, 1] - ref[-1, 1]) < 5e-7
    assert abs(ct[-10:, 1].mean() - ref[-10:, 1].mean()) < 5e-7
    # testSect: secSpan, secCL, secArea, secVel, secAlpha (places=6)
    dist = s.get("forceDist").reshape(-1, 16)
    refd = np.loadtxt(golden_dir / "katzNplotkin-AR04" / "r01b01ForceDist00160.csv.ref", skiprows=1)
    for col in (0, 1, 8, 9, 12):
        np.testing.assert_allclose(dist[:, col], refd[:, col], rtol=5.1e-7, atol=5e-7)


@pytest.mark.slow
def test_elevate_rotor_full(golden_dir):
    """All 151 CT rows (through rollup at step 30 and truncation at step 75) plus sections at step 150."""
    s, ct, ref = _ct_check(golden_dir / "elevateTest", 150)
    dist = s.get("forceDist").reshape(-1, 16)
    refd = np.loadtxt(golden_dir / "elevateTest" / "r01b01ForceDist00150.csv.ref", skiprows=1)
    for col in (0, 1, 8, 9, 12):
        np.testing.assert_allclose(dist[:, col], refd[:, col], rtol=5.1e-7, atol=5e-7)

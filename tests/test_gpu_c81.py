"""Loads from airfoil tables (forceCalcSwitch 1: rotor_calc_force_alpha with
C81 files, src/classdef.f90:2091-2195, 4734-4747) on the GPU against the
oracle: two tables split at r/R 0.6, the hover rotor through roll-up and
truncation.  The flow does not depend on the loads, so the wake stays bit
for bit the oracle's; the CT rows agree to 1e-12 (the sectional angle of
attack is an atan2, evaluated by the device and the host libm)."""
import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu


def c81_case(d, nt):
    c = C.rotor_2blade_hover(nt=nt, n_nwake=10, truncate_nt=16)
    (d / "inboard.C81").write_text(C.synthetic_airfoil("inboard", cl_slope=5.6, alpha0_deg=-1.0, cd0=0.01))
    (d / "outboard.C81").write_text(C.synthetic_airfoil("outboard", cl_slope=6.1, cd0=0.007, nmach=11))
    geo = (c.geom.replace("forceCalcSwitch = 0", "forceCalcSwitch = 1").replace("nAirfoils = 0", "nAirfoils = 2")
           .replace("airfoilSectionLimit = 1.0", "airfoilSectionLimit = 0.6, 1.0")
           .replace("alpha0 = 0.0", "alpha0 = -1.0, 0.0")
           .replace("airfoilFile = 0", "airfoilFile = inboard.C81, outboard.C81"))
    assert "forceCalcSwitch = 1" in geo and "outboard.C81" in geo
    return c.config, geo


@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_FP32_NEAR64])
def test_airfoil_table_loads_match_the_oracle(tmp_path, prec):
    nt = 30
    cfg, geo = c81_case(tmp_path, nt)
    g = lib.Case(cfg, geo, tmp_path, precision=prec, sum_chunk=16)
    g.start()
    rows = g.step(nt)
    if prec != lib.PREC_FP64:
        # the FP32 form: within the solver's CT tolerance of the FP64 form
        f = lib.Case(cfg, geo, tmp_path, precision=lib.PREC_FP64, sum_chunk=16)
        f.start()
        r64 = f.step(nt)
        assert np.max(np.abs(rows[:, 1] - r64[:, 1]) / np.abs(r64[:, 1])) < 1e-4
        return
    O.set_threads(8)
    o = O.Sim(cfg, geo, tmp_path)
    o.set_sum_chunk(16)
    o.start()
    o.step(nt)
    ref = o.ct_hist()
    got = g.ct_hist()
    assert got.shape == ref.shape
    np.testing.assert_array_equal(got[:, 0], ref[:, 0])
    # relative to the largest load (the in-plane force columns are rounding
    # noise of zero, ~1e-20)
    scale = np.max(np.abs(ref[:, 1:]))
    assert np.max(np.abs(got[:, 1:] - ref[:, 1:])) < 1e-12 * scale
    # the loads feed nothing back: the wake is the oracle's bit for bit
    for b in (1, 2):
        np.testing.assert_array_equal(g.get("waN", b).reshape(-1, 4, 3), o.get("waN", b).reshape(-1, 4, 2, 3)[:, :, 0])
        np.testing.assert_array_equal(g.get("gam", b), o.get("gam", b))
    # the tables are in use: CT differs from the pressure-integrated loads
    plain = lib.Case(cfg, geo.replace("forceCalcSwitch = 1", "forceCalcSwitch = 0"), tmp_path,
                     precision=prec, sum_chunk=16)
    plain.start()
    assert np.max(np.abs(plain.step(nt)[:, 1] - rows[:, 1]) / np.abs(rows[:, 1])) > 1e-3


def test_missing_table_and_axisymmetry_are_refused(tmp_path):
    cfg, geo = c81_case(tmp_path, 10)
    with pytest.raises(lib.VlmError):
        lib.Case(cfg, geo.replace("inboard.C81", "missing.C81"), tmp_path)
    with pytest.raises(lib.VlmError):
        lib.Case(cfg, geo.replace("axisymmetrySwitch = 0", "axisymmetrySwitch = 1"), tmp_path)

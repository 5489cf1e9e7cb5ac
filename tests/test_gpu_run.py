"""The case-directory runner (volcanor_gb300.run): a reference case run end
to end writes the Results/ files the reference's post-processing reads."""
import json

import numpy as np
import pytest

from volcanor_gb300 import cases as C
from volcanor_gb300 import gridgen as G
from volcanor_gb300 import lib
from volcanor_gb300 import run as RUN

pytestmark = pytest.mark.gpu


def test_run_reference_case_directory(golden_dir, tmp_path):
    d = golden_dir / "katzNplotkin-AR04"
    s = RUN.run_case(d, lib.PREC_FP64, results_dir=tmp_path)
    assert s["steps"] == 160 and s["filament_files"] == []
    hist = np.loadtxt(tmp_path / "r01ForceNonDim.csv", skiprows=1)
    ref = np.loadtxt(d / "r01ForceNonDim.csv.ref", skiprows=1)
    assert hist.shape == ref.shape
    assert abs(hist[-1, 1] - ref[-1, 1]) < 5e-7
    assert json.loads((tmp_path / "r01Params.json").read_text())["nt"] == 160
    assert len(list(tmp_path.glob("r01b01ForceDist*.csv"))) == 161


def test_run_writes_filament_files(tmp_path):
    cfg = C.config_text(nt=14, dt=0.025, density=1.0, fdScheme=3, gridPlot=7)
    geo = C.geom_text(nb=1, nc=2, ns=4, nNwake=4, span=2.0, chord=0.5, theta0=6.0, velBody=(-10.0, 0.0, 0.0),
                      wakeTruncateNt=9)
    case = tmp_path / "case"
    case.mkdir()
    (case / "config.nml").write_text(cfg)
    (case / "geom01.nml").write_text(geo)
    s = RUN.run_case(case, lib.PREC_FP32_NEAR64)
    names = [p.name for p in s["filament_files"]]
    assert names == ["filaments00007.dat", "filaments00014.dat"]
    F = G.read_filaments(s["filament_files"][-1])
    assert F.vr_wing.shape == (8, 50) and F.vr_nwake.shape == (16, 50) and F.vf_te.shape == (4, 12)
    assert np.all(np.isfinite(F.vf_far)) and len(F.gam_far) > 0
    assert (case / "Results" / "r01ForceNonDim.csv").exists()


def test_run_coupled_rotor_directory(tmp_path):
    """A case directory with nr = 2 (a rotor and its ground image) writes
    r01 and r02 force files; their CT rows are the system's."""
    sc = C.rotor_ground_effect(height=0.8, nt=12, n_nwake=6, truncate_nt=9)
    d = sc.write(tmp_path / "ge")
    s = RUN.run_case(d, lib.PREC_FP64, results_dir=tmp_path / "out")
    assert s["rotors"] == 2 and s["steps"] == 12
    y = lib.System(sc.config, sc.geoms, d)
    y.start()
    rows = y.step(12)
    for ir in (1, 2):
        hist = np.loadtxt(tmp_path / "out" / f"r{ir:02d}ForceNonDim.csv", skiprows=1)
        assert hist.shape == (13, 10)
        np.testing.assert_allclose(hist[1:, 1], rows[:, ir - 1, 1], rtol=1e-6)  # E15.7 text
        assert (tmp_path / "out" / f"r{ir:02d}Params.json").exists()
        assert (tmp_path / "out" / f"r{ir:02d}b01ForceDist00012.csv").exists()

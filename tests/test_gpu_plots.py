"""Plot files of a GPU run against the same files written from the oracle's
state: a two-blade rotor whose near wake fills and spills into the far wake,
every plot switch on.  The wing/wake geometry, tip, skew and bound
circulation files are identical text (FP64, equal summation blocks); the
inflow and probe files hold velocities that the two sides sum in different
orders, so their numbers agree to a unit in the last written digit."""
import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C
from volcanor_gb300 import lib
from volcanor_gb300 import plots as PL
from volcanor_gb300 import run as RUN

pytestmark = pytest.mark.gpu

CHUNK = 16
NT = 9


def _case(tmp_path):
    cfg = C.config_text(nt=NT, dt=0.0, density=1.2, kinematicVisc=1.5e-5, fdScheme=3, wakeDissipation=1,
                        wakePlot=3, wakeTipPlot=3, probe=1)
    geo = C.geom_text(nb=2, nc=2, ns=6, nNwake=4, span=1.0, rootcut=0.2, chord=0.08, Omega=100.0,
                      shaftAxis=(0.0, 0.0, 1.0), theta0=8.0, velBody=(0.0, 0.0, 0.0), spanwiseCore=0.05,
                      streamwiseCoreVec=0.05, symmetricTau=0, pivotLE=0.25, skewPlotSwitch=3, inflowPlotSwitch=3,
                      gammaPlotSwitch=2)
    d = C.Case("plots", cfg, geo, {"probes.in": "2\n0.3 0.1 -0.05 0.0 0.0 -1.0\n-0.2 0.6 0.02 0.5 0.0 0.0\n"})
    return d.write(tmp_path / "case"), cfg, geo


class _OracleCase:
    """The oracle's state behind the getters the writers read (ring corners
    instead of its filament layout)."""

    def __init__(self, sim):
        self.s = sim

    def geti(self, n):
        return self.s.geti(n)

    def get(self, n, b=1):
        v = self.s.get(n, b)
        return v.reshape(-1, 4, 2, 3)[:, :, 0].ravel() if n in ("waN", "vr") else v

    def vind_points(self, P):
        return self.s.vind_points(np.asarray(P, dtype=float))


class _OracleView(PL.CaseView):
    def panel_corners(self, k, b):
        assert self.case.geti("iter") == k  # inside iteration k
        return self.case.get("PC", b).reshape(-1, 4, 3)

    def vind_filaments(self, fc, rvc, gam, P):
        return O.vind_filaments(fc, rvc, gam, P)


def _oracle_files(out, d, cfg, geo, omega, theta0, dt):
    r = O.Sim(cfg, geo, d)
    r.set_sum_chunk(CHUNK)
    r.start()
    oc = _OracleCase(r)
    view = _OracleView(oc, cfg, geo, d)
    probe, probe_vel = PL.read_probes(d / "probes.in")
    t = 0.0
    for k in range(1, NT + 1):
        t = t + dt
        due = RUN._due({"wakePlot": 3, "wakeTipPlot": 3, "gridPlot": 0, "probe": 1, "skewPlotSwitch": 3,
                        "inflowPlotSwitch": 3, "gammaPlotSwitch": 2, "wakeSuppress": 0, "nNwake": 4}, k)
        gam_prev = [oc.get("gam", b) for b in (1, 2)]
        r.step_open()
        ts = f"{k:05d}"
        if due["skew"]:
            PL.skew2file(lambda b: out / f"r01b{b:02d}skew{ts}.csv", view)
        if due["geom"]:
            PL.geom2file(out / f"r01wingNwake{ts}.tec", view, k, gam_prev, True)
        if due["tip"]:
            PL.tip2file(out / f"r01tip{ts}.tec", out / f"r01tipXYZ{ts}.csv", view, k, gam_prev, omega, theta0)
        if due["inflow"]:
            PL.inflow2file(lambda b: out / f"r01b{b:02d}inflowDist{ts}.curve", view)
        if due["gamma"]:
            PL.gamma2file(lambda b: out / f"r01b{b:02d}gammaDist{ts}.curve", view)
        PL.probes2file(out / f"probes{ts}.csv", view, probe, probe_vel, t)
        r.step_close()
    return r


def _numbers(text):
    return np.array([float(x) for l in text.splitlines()[1:] for x in l.split()])


def test_plot_files_match_oracle(tmp_path):
    d, cfg, geo = _case(tmp_path)
    s = RUN.run_case(d, lib.PREC_FP64, results_dir=tmp_path / "gpu", sum_chunk=CHUNK)
    g = lib.Case(cfg, geo, d)
    omega, theta0, dt = g.get("Omega")[0], g.get("theta0")[0], g.get("dt")[0]
    (tmp_path / "ora").mkdir()
    r = _oracle_files(tmp_path / "ora", d, cfg, geo, omega, theta0, dt)
    np.testing.assert_array_equal(s["last_row"], r.ct_hist()[-1])
    names = sorted(p.name for p in (tmp_path / "ora").iterdir())
    got = sorted(p.name for p in s["files"])
    assert got == names
    assert {n[:9] for n in names} >= {"r01wingNw", "r01tip000", "r01tipXYZ", "r01b01ske", "r01b02inf", "r01b01gam",
                                      "probes000"}
    assert "r01wingNwake00009.tec" in names and "r01b02gammaDist00008.curve" in names
    # the far wake exists by iteration 9: its zone has more than the placeholder point
    assert 'T="FarWake"' in (tmp_path / "gpu" / "r01wingNwake00009.tec").read_text()
    assert "Zone I=2 J=1   K=1   T=\"FarWake\"" not in (tmp_path / "gpu" / "r01wingNwake00009.tec").read_text()
    for n in names:
        a, b = (tmp_path / "gpu" / n).read_text(), (tmp_path / "ora" / n).read_text()
        if "inflow" in n or n.startswith("probes"):
            assert a.splitlines()[0] == b.splitlines()[0]
            x, y = _numbers(a), _numbers(b)
            assert x.shape == y.shape and x.size > 0
            tol = 1.01e-7 if "inflow" in n else 1.01e-6 * np.abs(y) + 1e-300
            assert np.all(np.abs(x - y) <= tol), n
        else:
            assert a == b, n

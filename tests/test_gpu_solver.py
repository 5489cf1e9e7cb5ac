"""GPU free-wake solver against the oracle (same summation blocks -> same bits)
and against the reference's full-case golden CT histories."""
import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu


def run_both(cfg, geo, nsteps, base="", chunk=256, precision=lib.PREC_FP64):
    g = lib.Case(cfg, geo, base, precision=precision, sum_chunk=chunk)
    g.start()
    g.step(nsteps)
    r = O.Sim(cfg, geo, base)
    r.set_sum_chunk(chunk)
    r.start()
    r.step(nsteps)
    return g, r


def small_wing(fd, nt=14, nnw=6, trunc=10, **kw):
    cfg = C.config_text(nt=nt, dt=0.025, density=1.0, fdScheme=fd, **kw)
    geo = C.geom_text(nb=1, nc=3, ns=5, nNwake=nnw, span=2.0, chord=0.5, theta0=6.0, velBody=(-10.0, 0.0, 0.0),
                      wakeTruncateNt=trunc, spanwiseCore=0.04, streamwiseCoreVec=0.04)
    return cfg, geo


def assert_same_state(g, r, nb=1):
    np.testing.assert_array_equal(g.ct_hist(), r.ct_hist())
    np.testing.assert_array_equal(g.get("gamVec"), r.get("gamVec"))
    for b in range(1, nb + 1):
        gw = g.get("waN", b).reshape(-1, 4, 3)
        rw = r.get("waN", b).reshape(-1, 4, 2, 3)[:, :, 0]
        np.testing.assert_array_equal(gw, rw)
        np.testing.assert_array_equal(g.get("waN_gam", b), r.get("waN_gam", b))
        np.testing.assert_array_equal(g.get("waN_rvc", b), r.get("waN_rvc", b))
        np.testing.assert_array_equal(g.get("waF", b), r.get("waF", b))
        np.testing.assert_array_equal(g.get("waF_gam", b), r.get("waF_gam", b))


@pytest.mark.parametrize("fd", [0, 1, 2, 3, 4, 5])
def test_fd_schemes_bitwise(fd):
    cfg, geo = small_wing(fd)
    g, r = run_both(cfg, geo, 14, chunk=16)
    assert_same_state(g, r)


def test_dissipation_strain_initwake_bitwise():
    cfg, geo = small_wing(3, wakeDissipation=1, wakeStrain=1, initWakeVelNt=5)
    geo = geo.replace("initWakeVel = 0.0", "initWakeVel = 1.5")
    g, r = run_both(cfg, geo, 14, chunk=16)
    assert_same_state(g, r)


def test_reference_sequential_order_bitwise():
    """sum_chunk = 0: the reference's own summation order."""
    cfg, geo = small_wing(3)
    g, r = run_both(cfg, geo, 12, chunk=0)
    assert_same_state(g, r)


def test_rotor_two_blades_truncation_bitwise():
    c = C.rotor_2blade_hover(nt=40, n_nwake=12, truncate_nt=20)
    g, r = run_both(c.config, c.geom, 40, chunk=64)
    assert_same_state(g, r, nb=2)
    assert g.geti("rowFar") == 1 and g.geti("rowNear") == 1


def test_elevate_axisymmetric_plot3d_bitwise(golden_dir):
    """tests/elevateTest.case (5 blades, axisymmetry, PLOT3D, dissipation, truncation), 90 steps."""
    d = golden_dir / "elevateTest"
    cfg, geo = (d / "config.nml").read_text(), (d / "geom01.nml").read_text()
    g, r = run_both(cfg, geo, 90, base=d, chunk=256)
    assert_same_state(g, r, nb=5)


def test_katz_plotkin_full_case_vs_reference_golden(golden_dir):
    """All 161 CT rows of tests/katzNplotkin-AR04.case to the reference's printed 7 digits."""
    d = golden_dir / "katzNplotkin-AR04"
    g = lib.Case.from_case_dir(d, precision=lib.PREC_FP64, sum_chunk=256)
    g.start()
    g.step(160)
    ct = g.ct_hist()
    ref = np.loadtxt(d / "r01ForceNonDim.csv.ref", skiprows=1)
    rel = np.abs(ct[:, 1] - ref[:, 1]) / np.abs(ref[:, 1])
    assert rel.max() <= 5.1e-7, rel.max()


def test_elevate_full_case_vs_reference_golden(golden_dir):
    d = golden_dir / "elevateTest"
    g = lib.Case.from_case_dir(d, precision=lib.PREC_FP64, sum_chunk=256)
    g.start()
    g.step(150)
    ct = g.ct_hist()
    ref = np.loadtxt(d / "r01ForceNonDim.csv.ref", skiprows=1)
    rel = np.abs(ct[:, 1] - ref[:, 1]) / np.abs(ref[:, 1])
    assert rel.max() <= 5.1e-7, rel.max()


@pytest.mark.parametrize("prec", [lib.PREC_FP32, lib.PREC_FP32_NEAR64])
def test_fp32_solver_ct_error(prec):
    c = C.rotor_2blade_hover(nt=60, n_nwake=20, truncate_nt=40)
    g64 = lib.Case(c.config, c.geom, precision=lib.PREC_FP64)
    g64.start()
    a = g64.step(60)[:, 1]
    g32 = lib.Case(c.config, c.geom, precision=prec)
    g32.start()
    b = g32.step(60)[:, 1]
    assert np.max(np.abs(b - a) / np.abs(a)) < 1e-4


def test_fp32_lu_refinement_matches_fp64_inverse():
    """FP32 LU + FP64 iterative refinement: the refined circulations equal the
    FP64-inverse solve to ~1e-14, so the CT history agrees to 1e-10 over a
    free-wake run, and the reported residual is at round-off level."""
    c = C.rotor_2blade_hover(nt=40, n_nwake=20, truncate_nt=30)
    runs = {}
    for mode in (0, 1):
        g = lib.Case(c.config, c.geom, precision=lib.PREC_FP64, solve_mode=mode)
        g.start()
        runs[mode] = (g.step(40)[:, 1], g.get("gamVec"), g.get("lu_residual")[0])
    a, b = runs[0][0], runs[1][0]
    assert np.max(np.abs(b - a) / np.abs(a)) < 1e-10
    ga, gb = runs[0][1], runs[1][1]
    assert np.max(np.abs(gb - ga)) <= 1e-12 * np.max(np.abs(ga))
    assert runs[0][2] == 0.0
    assert 0.0 <= runs[1][2] < 1e-12


@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_FP32_NEAR64])
def test_graph_replay_is_bit_identical(prec):
    """Steady-state steps replayed from a captured CUDA graph give the same
    bits as the same steps launched one by one."""
    c = C.rotor_2blade_hover(nt=70, n_nwake=20, truncate_nt=30)
    out = []
    for graph in (False, True):
        g = lib.Case(c.config, c.geom, precision=prec, use_graph=graph)
        g.start()
        rows = np.concatenate([g.step(20), g.step(1), g.step(49)])
        out.append((rows, g.get("waN", 1), g.get("waF", 2)))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_errors_and_state_checks():
    cfg, geo = small_wing(3)
    g = lib.Case(cfg, geo)
    with pytest.raises(lib.VlmError):
        g.step(1)  # before start
    g.start()
    with pytest.raises(lib.VlmError):
        g.step(100)  # past nt
    with pytest.raises(lib.VlmError):
        lib.Case(cfg.replace("fdScheme = 3", "fdScheme = 9"), geo)


@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_FP32_NEAR64])
def test_checkpoint_resume_is_bit_identical(prec, tmp_path):
    """Save after 25 steps, continue 30; a fresh case loaded from the file
    continues the same 30 steps bit for bit (the reference's restart files)."""
    c = C.rotor_2blade_hover(nt=60, n_nwake=20, truncate_nt=30)
    a = lib.Case(c.config, c.geom, precision=prec)
    a.start()
    a.step(25)
    ck = tmp_path / "ck.bin"
    a.checkpoint_save(ck)
    ra = a.step(30)
    b = lib.Case(c.config, c.geom, precision=prec)
    b.checkpoint_load(ck)
    assert b.geti("iter") == 25
    rb = b.step(30)
    assert np.array_equal(ra, rb)
    assert np.array_equal(a.get("waN", 2), b.get("waN", 2))
    # a checkpoint of another case is refused
    other = C.rotor_2blade_hover(nt=60, n_nwake=21, truncate_nt=30)
    o = lib.Case(other.config, other.geom, precision=prec)
    with pytest.raises(lib.VlmError):
        o.checkpoint_load(ck)


def test_checkpoint_loads_across_precisions(tmp_path):
    """The saved state is FP64 in every precision: an FP32 + near-field case
    continues from an FP64 state (factoring the restored AIC in FP32 for its
    refined solve) within the FP32 tolerance of the FP64 continuation, and an
    FP64 case continues from the FP32 case's state exactly as a second FP64
    case loaded from the same file."""
    c = C.rotor_2blade_hover(nt=60, n_nwake=20, truncate_nt=30)
    a = lib.Case(c.config, c.geom, precision=lib.PREC_FP64)
    a.start()
    a.step(30)
    ck64 = tmp_path / "ck64.bin"
    a.checkpoint_save(ck64)
    r64 = a.step(10)[:, 1]
    b = lib.Case(c.config, c.geom, precision=lib.PREC_FP32_NEAR64)
    b.checkpoint_load(ck64)
    assert b.geti("iter") == 30
    r32 = b.step(10)[:, 1]
    assert np.max(np.abs(r32 - r64) / np.abs(r64)) < 1e-4
    assert 0.0 <= b.get("lu_residual")[0] < 1e-12
    ck32 = tmp_path / "ck32.bin"
    b.checkpoint_save(ck32)
    x = lib.Case(c.config, c.geom, precision=lib.PREC_FP64)
    x.checkpoint_load(ck32)
    y = lib.Case(c.config, c.geom, precision=lib.PREC_FP64)
    y.checkpoint_load(ck32)
    assert x.geti("iter") == 40
    assert np.array_equal(x.step(5), y.step(5))


def _lattice_cases():
    h = C.rotor_2blade_hover(nt=48, n_nwake=24, truncate_nt=36)
    f = C.rotor_4blade_forward(nt=40, n_nwake=16, truncate_nt=30)
    # core radius varying by station: streamwise filaments of neighbouring
    # rings differ in core, so those edges stay separate in lattice form
    ns = 8
    cfg = C.config_text(nt=30, dt=0.025, density=1.0, fdScheme=3, wakeDissipation=1, kinematicVisc=1.5e-5)
    geo = C.geom_text(nb=1, nc=2, ns=ns, nNwake=20, span=2.0, chord=0.5, theta0=6.0, velBody=(-10.0, 0.0, 0.0),
                      spanwiseCore=0.04, streamwiseCoreVec=tuple(0.03 + 0.004 * k for k in range(ns + 1)),
                      wakeTruncateNt=25)
    return {"hover": (h.config, h.geom, h.files, 48), "forward": (f.config, f.geom, f.files, 40),
            "wing_station_cores": (cfg, geo, {}, 30)}


@pytest.mark.parametrize("name", ["hover", "forward", "wing_station_cores"])
@pytest.mark.parametrize("prec", [lib.PREC_FP32, lib.PREC_FP32_NEAR64])
def test_lattice_form_matches_ring_form(name, prec, tmp_path):
    """FP32 paths: evaluating each near-wake lattice edge once with the
    circulation difference of its two rings gives the ring-by-ring sum up to
    FP32 rounding; both stay within 1e-4 of FP64 in CT."""
    cfg, geo, files, n = _lattice_cases()[name]
    for fn, text in files.items():
        (tmp_path / fn).write_text(text)
    runs = {}
    for key, kw in {"lat": dict(precision=prec, lattice=True), "ring": dict(precision=prec, lattice=False),
                    "fp64": dict(precision=lib.PREC_FP64)}.items():
        g = lib.Case(cfg, geo, tmp_path, **kw)
        g.start()
        runs[key] = (g.step(n)[:, 1], g.get("velN", 1), g.get("waN", 1))
    ct_lat, ct_ring, ct64 = runs["lat"][0], runs["ring"][0], runs["fp64"][0]
    assert np.max(np.abs(ct_lat - ct_ring) / np.abs(ct_ring)) < 2e-5
    assert np.max(np.abs(ct_lat - ct64) / np.abs(ct64)) < 1e-4
    vl, vr = runs["lat"][1], runs["ring"][1]
    assert np.max(np.abs(vl - vr)) <= 1e-4 * np.max(np.abs(vr))


def test_custom_trajectory_bitwise(tmp_path):
    """customTrajectorySwitch = 1 (trajectory01.in: body velocity and rates
    per step): the motion enters through the host-computed frames only, so
    the FP64 run stays bit-identical to the oracle."""
    nt = 12
    cfg = C.config_text(nt=nt, dt=0.025, density=1.0, fdScheme=3, wakeDissipation=1, kinematicVisc=1.5e-5)
    geo = C.geom_text(nb=1, nc=3, ns=5, nNwake=6, span=2.0, chord=0.5, theta0=6.0, velBody=(-10.0, 0.0, 0.0),
                      wakeTruncateNt=10, customTrajectorySwitch=1, cgCoords=(0.1, 0.0, 0.0))
    rng = np.random.default_rng(7)
    rows = []
    for i in range(nt):
        rows.append(f"{-10.0 + 0.5 * np.sin(0.3 * i):.12e} {0.2 * rng.normal():.12e} {0.3 * np.cos(0.2 * i):.12e} "
                    f"{0.05 * rng.normal():.12e} {0.1 * np.sin(0.1 * i):.12e} {0.02 * rng.normal():.12e}")
    (tmp_path / "trajectory01.in").write_text("\n".join(rows) + "\n")
    g, r = run_both(cfg, geo, nt, base=tmp_path, chunk=16)
    assert_same_state(g, r)


def test_cambered_wing_bitwise(tmp_path):
    """Camber sections (nCamberFiles > 0): the cambered geometry enters
    through the host geometry only, so the FP64 run stays bit-identical to
    the oracle."""
    xs = np.linspace(0.0, 1.0, 9)
    (tmp_path / "camber.dat").write_text(f"{len(xs)}\n" + "\n".join(f"{x:.12f} {0.06 * x * (1 - x):.12f}" for x in xs))
    cfg = C.config_text(nt=10, dt=0.025, density=1.0, fdScheme=3)
    geo = C.geom_text(nb=1, nc=3, ns=5, nNwake=5, span=2.0, chord=0.5, theta0=3.0, velBody=(-10.0, 0.0, 0.0),
                      wakeTruncateNt=8, chordSpacing=2, nCamberFiles=2)
    geo = geo.replace("&ORIENT", "&CAMBERSECTIONS\ncamberSectionLimit = 0.5, 1.0\n"
                      "camberFile = 'camber.dat', '0'\n/\n&ORIENT", 1)
    g, r = run_both(cfg, geo, 10, base=tmp_path, chunk=16)
    assert_same_state(g, r)

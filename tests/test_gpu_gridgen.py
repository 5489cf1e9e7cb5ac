"""Point-field evaluation of a wake (gridgen) on the GPU: the filament
kernel against the oracle, the filament file of a GPU run against the
oracle's state, and a whole gridgen run against the oracle's sums."""
import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C
from volcanor_gb300 import gridgen as G
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu


def test_filament_kernel_matches_oracle():
    rng = np.random.default_rng(3)
    N, M = 700, 300
    a = rng.uniform(-1, 1, (N, 3))
    fc = np.stack([a, a + rng.uniform(-0.2, 0.2, (N, 3))], axis=1)
    rvc = rng.uniform(0.005, 0.05, N)
    gam = rng.normal(size=N)
    P = rng.uniform(-1, 1, (M, 3))
    P[:5] = fc[:5, 0]                          # targets on filament ends
    P[5:10] = 0.5 * (fc[5:10, 0] + fc[5:10, 1])  # and on filament lines
    chunk = lib.rings_sum_chunk(N, M, lib.PREC_FP64)
    V64 = lib.biot_savart_filaments(fc, rvc, gam, P, lib.PREC_FP64)
    np.testing.assert_array_equal(V64, O.vind_filaments(fc, rvc, gam, P, chunk=chunk))
    scale = np.max(np.abs(V64))
    for prec in (lib.PREC_FP32, lib.PREC_FP32_NEAR64):
        V = lib.biot_savart_filaments(fc, rvc, gam, P, prec)
        assert np.max(np.abs(V - V64)) <= 2e-5 * scale
    assert lib.biot_savart_filaments(fc[:0], rvc[:0], gam[:0], P).max() == 0.0


def _case():
    cfg = C.config_text(nt=14, dt=0.025, density=1.0, fdScheme=3, wakeDissipation=1, kinematicVisc=1.5e-5)
    geo = C.geom_text(nb=1, nc=3, ns=5, nNwake=6, span=2.0, chord=0.5, theta0=6.0, velBody=(-10.0, 0.0, 0.0),
                      wakeTruncateNt=10, spanwiseCore=0.04, streamwiseCoreVec=0.04)
    return cfg, geo


def _oracle_filaments(r):
    """The reference's filaments2file arrays built from the oracle's state."""
    nb, nc, ns = r.geti("nb"), r.geti("nc"), r.geti("ns")
    NW, NF, rowFar = r.geti("nNwake"), r.geti("nFwake"), r.geti("rowFar")
    wing, nwake, te, gte, far, gfar = [], [], [], [], [], []

    def vr(fil, rvc, gam):  # fil: (n, 4, 2, 3)
        out = np.zeros((fil.shape[0], 50))
        for k in range(4):
            out[:, 12 * k:12 * k + 6] = fil[:, k].reshape(-1, 6)
            out[:, 12 * k + 9] = rvc[:, k]
        out[:, 48] = gam
        return out

    for b in range(1, nb + 1):
        wing.append(vr(r.get("vr", b).reshape(-1, 4, 2, 3), r.get("vr_rvc", b).reshape(-1, 4), r.get("gam", b)))
        fil = r.get("waN", b).reshape(-1, 4, 2, 3)
        rvc = r.get("waN_rvc", b).reshape(-1, 4)
        gam = r.get("waN_gam", b)
        nwake.append(vr(fil, rvc, gam))
        last = [NW - 1 + NW * j for j in range(ns)]
        t = np.zeros((ns, 12))
        t[:, 0:6] = fil[last, 1].reshape(-1, 6)
        t[:, 9] = rvc[last, 1]
        te.append(t)
        gte.append(-1.0 * gam[last])
        f = np.zeros((NF - rowFar + 1, 12))
        f[:, 0:6] = r.get("waF", b).reshape(NF, 6)[rowFar - 1:]
        f[:, 9] = r.get("waF_rvc", b)[rowFar - 1:]
        far.append(f)
        gfar.append(r.get("waF_gam", b)[rowFar - 1:])
    return G.Filaments(np.concatenate(wing), np.concatenate(nwake), np.concatenate(te), np.concatenate(gte),
                       np.concatenate(far), np.concatenate(gfar))


FC_RVC_GAM_VR = [c for k in range(4) for c in range(12 * k, 12 * k + 6)] + [12 * k + 9 for k in range(4)] + [48]
FC_RVC_VF = list(range(6)) + [9]


def test_filament_file_of_a_gpu_run_matches_oracle_state(tmp_path):
    cfg, geo = _case()
    g = lib.Case(cfg, geo, precision=lib.PREC_FP64, sum_chunk=16)
    r = O.Sim(cfg, geo)
    r.set_sum_chunk(16)
    g.start()
    r.start()
    g.step(14)
    r.step(14)
    assert g.geti("rowFar") <= g.geti("nFwake")
    F = G.read_filaments(G.write_filaments(tmp_path / "filaments00014.dat", G.filaments_from_case(g)))
    R = _oracle_filaments(r)
    np.testing.assert_array_equal(F.vr_wing[:, FC_RVC_GAM_VR], R.vr_wing[:, FC_RVC_GAM_VR])
    np.testing.assert_array_equal(F.vr_nwake[:, FC_RVC_GAM_VR], R.vr_nwake[:, FC_RVC_GAM_VR])
    np.testing.assert_array_equal(F.vf_te[:, FC_RVC_VF], R.vf_te[:, FC_RVC_VF])
    np.testing.assert_array_equal(F.gam_te, R.gam_te)
    np.testing.assert_array_equal(F.vf_far[:, FC_RVC_VF], R.vf_far[:, FC_RVC_VF])
    np.testing.assert_array_equal(F.gam_far, R.gam_far)


@pytest.mark.parametrize("fix", [False, True])
def test_gridgen_run_matches_oracle_sums(tmp_path, fix):
    cfg, geo = _case()
    g = lib.Case(cfg, geo, precision=lib.PREC_FP64)
    g.start()
    g.step(14)
    (tmp_path / "Results").mkdir()
    F = G.filaments_from_case(g)
    G.write_filaments(tmp_path / "Results" / "filaments00014.dat", F)
    (tmp_path / "gridconfig.nml").write_text(
        "&VERSION\nfileFormatVersion = 0.2\n/\n&INPUTS\nnx = 6\nny = 5\nnz = 4\n"
        "xyzMin = -0.5, -1.2, -0.3\nxyzMax = 1.5, 1.2, 0.3\nvel = 10.0, 0.0, 0.0\n"
        "fileRangeStart = 14\nfileRangeStep = 1\nfileRangeEnd = 14\n/\n")
    (out,) = G.run(tmp_path, fix_wing_sum=fix)
    text = out.read_text().splitlines()
    assert text[2].strip() == 'ZONE I=6 J=5 K=4 T="Data"'
    vals = np.array(" ".join(text[5:]).split(), dtype=float)
    n_nodes, n_cells = 6 * 5 * 4, 5 * 4 * 3
    assert vals.size == 3 * n_nodes + 3 * n_cells
    U = vals[3 * n_nodes:].reshape(3, n_cells)
    cfgd = G.read_gridconfig((tmp_path / "gridconfig.nml").read_text())
    _, centres = G.grid_and_centres(cfgd)
    P = centres.reshape(3, -1, order="F").T  # Fortran order of the cells, as written
    wing = F.vr_wing if fix else F.vr_wing[-1:]
    ref = np.zeros_like(P)
    for vr in (wing, F.vr_nwake):
        corners = np.stack([vr[:, 12 * k:12 * k + 3] for k in range(4)], axis=1)
        rvc = np.stack([vr[:, 12 * k + 9] for k in range(4)], axis=1)
        ref += O.vind_rings(corners, rvc, vr[:, 48], P)
    for vf, gam in ((F.vf_te, F.gam_te), (F.vf_far, F.gam_far)):
        ref += O.vind_filaments(vf[:, 0:6].reshape(-1, 2, 3), vf[:, 9], gam, P)
    ref += np.array([10.0, 0.0, 0.0])
    # the file holds 16 significant digits; the GPU sums in blocks
    np.testing.assert_allclose(U.T, ref, rtol=0, atol=1e-12 * np.max(np.abs(ref)))


def test_filament_file_taken_mid_step_matches_oracle_mid_step(tmp_path):
    """The reference writes filamentsNNNNN.dat inside iteration NNNNN, after the
    loads and before the wake update (src/main.f90:788): the step's separate
    calls reach that state, and it equals the oracle's state at the same point."""
    cfg, geo = _case()
    g = lib.Case(cfg, geo, precision=lib.PREC_FP64, sum_chunk=16)
    r = O.Sim(cfg, geo)
    r.set_sum_chunk(16)
    g.start()
    r.start()
    g.step(13)
    r.step(13)
    g.solve_circulation()
    g.loads()
    r.step_open()
    assert g.geti("iter") == 13 and g.geti("rowFar") == r.geti("rowFar")
    F = G.read_filaments(G.write_filaments(tmp_path / "filaments00014.dat", G.filaments_from_case(g)))
    R = _oracle_filaments(r)
    np.testing.assert_array_equal(F.vr_wing[:, FC_RVC_GAM_VR], R.vr_wing[:, FC_RVC_GAM_VR])
    np.testing.assert_array_equal(F.vr_nwake[:, FC_RVC_GAM_VR], R.vr_nwake[:, FC_RVC_GAM_VR])
    np.testing.assert_array_equal(F.vf_te[:, FC_RVC_VF], R.vf_te[:, FC_RVC_VF])
    np.testing.assert_array_equal(F.vf_far[:, FC_RVC_VF], R.vf_far[:, FC_RVC_VF])
    np.testing.assert_array_equal(F.gam_far, R.gam_far)
    g.wake_step()
    r.step_close()
    np.testing.assert_array_equal(g.ct_hist(), r.ct_hist())

"""The time step as separate calls (vlm_case_solve_circulation,
vlm_case_loads, vlm_case_wake_step): the same bits as vlm_case_step, a
caller-supplied kinematic velocity, the mid-step state, and the call order
rules."""
import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu


def phased(g, nsteps, plot=1):
    rows = []
    for _ in range(nsteps):
        k = g.geti("iter") + 1
        g.solve_circulation()
        if k % plot == 0:
            rows.append(g.loads())
        g.wake_step()
    return np.array(rows)


@pytest.mark.parametrize("prec", [lib.PREC_FP64, lib.PREC_FP32_NEAR64])
@pytest.mark.parametrize("fd", [1, 3])
def test_phases_equal_whole_steps(prec, fd):
    c = C.rotor_2blade_hover(nt=40, n_nwake=12, truncate_nt=24, fd_scheme=fd)
    a = lib.Case(c.config, c.geom, precision=prec)
    a.start()
    ra = a.step(30)
    b = lib.Case(c.config, c.geom, precision=prec)
    b.aic_factor()
    b.start()
    rb = phased(b, 30)
    np.testing.assert_array_equal(ra, rb)
    for bl in (1, 2):
        for name in ("waN", "waN_gam", "waF", "waF_rvc", "velN", "gam"):
            np.testing.assert_array_equal(a.get(name, bl), b.get(name, bl), err_msg=name)
    # and back to whole steps
    np.testing.assert_array_equal(a.step(5), b.step(5))


def test_loads_every_other_step_as_rotor_force_plot():
    """rotorForcePlot = 2: vlm_case_step computes loads on even iterations;
    phases with loads on the same iterations give the same bits."""
    c = C.rotor_2blade_hover(nt=30, n_nwake=10, truncate_nt=20)
    cfg = c.config.replace("rotorForcePlot = 1", "rotorForcePlot = 2")
    a = lib.Case(cfg, c.geom)
    a.start()
    a.step(20, with_ct=False)
    b = lib.Case(cfg, c.geom)
    b.start()
    rb = phased(b, 20, plot=2)
    np.testing.assert_array_equal(a.ct_hist()[2::2], rb)
    np.testing.assert_array_equal(a.get("waN", 1), b.get("waN", 1))


def test_caller_kinematic_velocity():
    """The host's own kinematic velocity: passing the library's values gives
    the same circulations; a changed value changes them."""
    c = C.rotor_2blade_hover(nt=20, n_nwake=8, truncate_nt=12)
    a = lib.Case(c.config, c.geom)
    a.start()
    a.step(6)
    ga = a.solve_circulation()
    kv = np.concatenate([a.get("velKin", bl).reshape(-1, 3) for bl in (1, 2)])
    b = lib.Case(c.config, c.geom)
    b.start()
    b.step(6)
    gb = b.solve_circulation(kv)
    np.testing.assert_array_equal(ga, gb)
    x = lib.Case(c.config, c.geom)
    x.start()
    x.step(6)
    gx = x.solve_circulation(kv + np.array([0.0, 0.0, -1.0]))
    assert np.max(np.abs(gx - ga)) > 1e-3 * np.max(np.abs(ga))
    for g in (a, b, x):
        g.wake_step()


def test_mid_step_state_is_the_references_file_state():
    """Between the loads and the wake update the wake is the one the
    reference writes filaments2file from (src/main.f90:788), which equals
    the oracle's wake after its loads: the oracle's next wake update has not
    moved it yet, so the GPU mid-step wake equals the oracle's end-of-step
    wake of the previous iteration plus this step's shedding."""
    c = C.rotor_2blade_hover(nt=20, n_nwake=8, truncate_nt=12)
    g = lib.Case(c.config, c.geom, sum_chunk=16)
    g.start()
    g.step(9)
    g.solve_circulation()
    g.loads()
    waN, wg, waF, fg = g.get_wake(1)
    r = O.Sim(c.config, c.geom)
    r.set_sum_chunk(16)
    r.start()
    r.step(9)
    # the oracle at the end of step 9 then step 10's leading-edge shedding and
    # ageing/dissipation happen before the solve: compare the rows the solve
    # phase does not touch (every row but the newest)
    rw = r.get("waN", 1).reshape(-1, 4, 2, 3)[:, :, 0]
    NW, ns = g.geti("nNwake"), g.geti("ns")
    old_rows = [i + NW * j for j in range(ns) for i in range(1, NW)]
    np.testing.assert_array_equal(waN[old_rows], rw[old_rows])
    np.testing.assert_array_equal(waF, r.get("waF", 1).reshape(-1, 2, 3))
    g.wake_step()
    assert g.geti("iter") == 10


def test_call_order_errors():
    c = C.rotor_2blade_hover(nt=10, n_nwake=6, truncate_nt=8)
    g = lib.Case(c.config, c.geom)
    g.start()
    with pytest.raises(lib.VlmError):
        g.loads()          # no open step
    with pytest.raises(lib.VlmError):
        g.wake_step()      # no open step
    g.solve_circulation()
    with pytest.raises(lib.VlmError):
        g.step(1)          # step open
    with pytest.raises(lib.VlmError):
        g.solve_circulation()
    g.wake_step()
    g.step(1)
    assert g.geti("iter") == 2

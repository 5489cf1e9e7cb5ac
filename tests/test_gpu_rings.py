"""GPU ring kernel (vlm_biot_savart_rings) against the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu


def random_rings(rng, N, core=0.002):
    """Seeded rings as in the isolated-kernel workload: corner 1 ~ U[0,1]^3,
    closed quads from edge vectors of length U(0.005, 0.05)."""
    c0 = rng.uniform(0, 1, size=(N, 3))
    def edge():
        v = rng.normal(size=(N, 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        return v * rng.uniform(0.005, 0.05, size=(N, 1))
    e1, e2 = edge(), edge()
    corners = np.stack([c0, c0 + e1, c0 + e1 + e2, c0 + e2], axis=1)
    return corners, np.full((N, 4), core), rng.normal(size=N)


def test_fp64_matches_oracle_bit_for_bit():
    rng = np.random.default_rng(1)
    corners, rvc, gam = random_rings(rng, 700)
    P = rng.uniform(0, 1, size=(333, 3))
    P[:20] = corners[:20, 0]          # targets on ring corners (filament end points)
    P[20:40] = 0.5 * (corners[20:40, 0] + corners[20:40, 1])  # on a filament
    V = lib.biot_savart_rings(corners, rvc, gam, P, lib.PREC_FP64)
    C = lib.rings_sum_chunk(700, 333, lib.PREC_FP64)
    W = O.vind_rings(corners, rvc, gam, P, chunk=C if C < 700 else 0)
    np.testing.assert_array_equal(V, W)


def test_fp64_single_block_is_the_reference_order():
    rng = np.random.default_rng(2)
    corners, rvc, gam = random_rings(rng, 40)
    P = rng.uniform(0, 1, size=(50000, 3))  # many targets -> one summation block
    assert lib.rings_sum_chunk(40, 50000) == 40
    np.testing.assert_array_equal(lib.biot_savart_rings(corners, rvc, gam, P), O.vind_rings(corners, rvc, gam, P))


# FP32 coordinates carry ~6e-8 absolute rounding at |x| ~ 1; at a few core
# radii (0.008) from a filament that is a ~1e-5 relative velocity error, so the
# worst target sits near 1e-4 of the mean speed in FP32; the FP64 near-field
# path removes the pairs inside near_factor core radii.
@pytest.mark.parametrize("prec,tol,tol_rms", [(lib.PREC_FP32, 2e-3, 5e-5), (lib.PREC_FP32_NEAR64, 2e-4, 2e-5)])
def test_fp32_variants_error_vs_fp64(prec, tol, tol_rms):
    rng = np.random.default_rng(3)
    corners, rvc, gam = random_rings(rng, 4096)
    P = rng.uniform(0, 1, size=(2048, 3))
    V64 = O.vind_rings(corners, rvc, gam, P)
    V = lib.biot_savart_rings(corners, rvc, gam, P, prec)
    err = np.linalg.norm(V - V64, axis=1)
    scale = np.linalg.norm(V64, axis=1).mean()
    assert err.max() / scale < tol, (err.max() / scale)
    assert np.sqrt(np.mean(err ** 2)) / scale < tol_rms


def _near_targets(rng, corners, n, lo=1.0, hi=3.0, core=0.002):
    """Targets lo..hi core radii from points 20-80 % along random filaments."""
    i = rng.integers(0, corners.shape[0], n)
    k = rng.integers(0, 4, n)
    a, b = corners[i, k], corners[i, (k + 1) % 4]
    e = b - a
    u = np.cross(e, rng.normal(size=(n, 3)))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    return a + rng.uniform(0.2, 0.8, (n, 1)) * e + u * (rng.uniform(lo, hi, (n, 1)) * core)


def test_near_field_pairs_are_fp64():
    """Targets 1-3 core radii from filaments.  The FP32 kernel's own position
    rounding (6e-8 absolute at |x| ~ 1) is a ~1e-5 relative error at a few
    core radii; the FP64 near-field correction recomputes those pairs from
    FP64 positions.  What remains is the FP32 rounding of the other pairs and
    of the tile sums that held the near terms (~1e-7 of the near term,
    visible only where the target's total velocity cancels far below it).
    (a) one ring: the near terms dominate the velocity; the error left is the
        FP32 position rounding of the ring's other filaments (~1e-6 of the
        total), several times below FP32's;
    (b) 4096 random rings: typical errors well below FP32's, all below 1e-4."""
    rng = np.random.default_rng(11)
    corners, rvc, gam = random_rings(rng, 1)
    corners = corners * 0 + np.array([[0.3, 0.4, 0.5], [0.33, 0.4, 0.5], [0.33, 0.43, 0.5], [0.3, 0.43, 0.5]])
    P = _near_targets(rng, corners, 400)
    V64 = O.vind_rings(corners, rvc, gam, P)
    scale = np.linalg.norm(V64, axis=1)
    err32 = np.linalg.norm(lib.biot_savart_rings(corners, rvc, gam, P, lib.PREC_FP32) - V64, axis=1) / scale
    errn = np.linalg.norm(lib.biot_savart_rings(corners, rvc, gam, P, lib.PREC_FP32_NEAR64) - V64, axis=1) / scale
    assert errn.max() < 5e-6, errn.max()
    assert err32.max() > 5 * errn.max(), (err32.max(), errn.max())

    corners, rvc, gam = random_rings(rng, 4096)
    P = _near_targets(rng, corners, 600)
    V64 = O.vind_rings(corners, rvc, gam, P)
    scale = np.linalg.norm(V64, axis=1)
    err32 = np.linalg.norm(lib.biot_savart_rings(corners, rvc, gam, P, lib.PREC_FP32) - V64, axis=1) / scale
    errn = np.linalg.norm(lib.biot_savart_rings(corners, rvc, gam, P, lib.PREC_FP32_NEAR64) - V64, axis=1) / scale
    assert errn.max() < 1e-4, errn.max()
    assert np.median(errn) < 0.5 * np.median(err32), (np.median(errn), np.median(err32))


def test_edge_cases():
    rng = np.random.default_rng(4)
    corners, rvc, gam = random_rings(rng, 5)
    P = rng.uniform(0, 1, size=(7, 3))
    # no rings -> zero velocity; no targets -> nothing to do
    np.testing.assert_array_equal(lib.biot_savart_rings(corners[:0], rvc[:0], gam[:0], P), np.zeros((7, 3)))
    assert lib.biot_savart_rings(corners, rvc, gam, P[:0]).shape == (0, 3)
    # degenerate ring (all corners equal) and zero circulation contribute nothing
    deg = np.repeat(corners[:1, :1], 4, axis=1)
    V = lib.biot_savart_rings(np.concatenate([corners, deg]), np.concatenate([rvc, rvc[:1]]),
                              np.concatenate([gam, [3.0]]), P)
    np.testing.assert_array_equal(V, lib.biot_savart_rings(corners, rvc, gam, P))
    with pytest.raises(lib.VlmError):
        lib.biot_savart_rings(corners, rvc, gam, P, precision=7)


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_context_stays_usable():
    """A pipeline wait that nothing releases gives up after its poll limit and
    reports (no hang, no fault); the GPU keeps working afterwards."""
    assert lib.selftest_bounded_wait(4096)
    c = np.array([[[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]]], float)
    V = lib.biot_savart_rings(c, np.full((1, 4), 0.01), np.array([1.0]), np.array([[0.5, 0.5, 0.3]]),
                              lib.PREC_FP32)
    assert np.all(np.isfinite(V)) and abs(V[0, 2]) > 0

"""The allocation-free ring kernel entry point (vlm_biot_savart_rings_noalloc).

It exists for callers that cannot allocate device memory when they need a
Biot-Savart sum (a solver that reserves its device memory once at start-up, a
process under a hard memory cap, a caller that must not trigger the device
synchronisation an allocation can cause).  This file is collected last so a
run that stops at the first failure has run every other test first; it must
pass on its own in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rings(rng, N, core=0.002):
    c0 = rng.uniform(0, 1, size=(N, 3))

    def edge():
        v = rng.normal(size=(N, 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        return v * rng.uniform(0.005, 0.05, size=(N, 1))
    e1, e2 = edge(), edge()
    return np.stack([c0, c0 + e1, c0 + e1 + e2, c0 + e2], axis=1), np.full((N, 4), core), rng.normal(size=N)


def call_noalloc(corners, rvc, gam, P, precision):
    dev = torch.device("cuda")
    tc, tr, tg, tp = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (corners, rvc, gam, P))
    tv = torch.full_like(tp, float("nan"))  # every output element must be written
    stream = torch.cuda.current_stream().cuda_stream
    lib.biot_savart_rings_noalloc(tc.data_ptr(), tr.data_ptr(), tg.data_ptr(), corners.shape[0], tp.data_ptr(),
                                  P.shape[0], tv.data_ptr(), precision, stream)
    torch.cuda.synchronize()
    return tv.cpu().numpy()


# FP64: same arithmetic, possibly different summation blocks -> rounding-level
# differences; FP32 variants: different block partial sums in FP32.
TOL = {lib.PREC_FP64: 1e-12, lib.PREC_FP32: 2e-5, lib.PREC_FP32_NEAR64: 2e-5}


@pytest.mark.parametrize("precision", [lib.PREC_FP64, lib.PREC_FP32, lib.PREC_FP32_NEAR64])
def test_noalloc_matches_allocating_entry_point_over_calls(precision):
    rng = np.random.default_rng(20 + precision)
    # the later calls reuse the scratch left by the first; M = 64 splits the
    # FP32 sums into the most chunks, M = 65536 leaves room for one
    for N, M in ((3000, 5000), (16384, 1111), (16384, 64), (2000, 65536)):
        corners, rvc, gam = rings(rng, N)
        P = rng.uniform(0, 1, size=(M, 3))
        P[:10] = corners[:10, 2]  # targets on ring corners
        ref = lib.biot_savart_rings(corners, rvc, gam, P, precision)
        got = call_noalloc(corners, rvc, gam, P, precision)
        assert np.all(np.isfinite(got))
        scale = np.abs(ref).max()
        np.testing.assert_allclose(got, ref, rtol=0, atol=TOL[precision] * scale)


@pytest.mark.parametrize("precision", [lib.PREC_FP64, lib.PREC_FP32_NEAR64])
def test_noalloc_without_rings_writes_zeros(precision):
    rng = np.random.default_rng(7)
    P = rng.uniform(0, 1, size=(300, 3))
    got = call_noalloc(np.zeros((0, 4, 3)), np.zeros((0, 4)), np.zeros(0), P, precision)
    assert np.array_equal(got, np.zeros_like(P))


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L = lib.load()
    rc = L.vlm_biot_savart_rings_noalloc(None, None, None, 16385, None, 10, None, lib.PREC_FP64, None)
    assert rc == 1
    buf = ctypes.create_string_buffer(512)
    L.vlm_last_error(buf, 512)
    assert b"16384" in buf.value
    rc = L.vlm_biot_savart_rings_noalloc(None, None, None, 10, None, 65537, None, lib.PREC_FP32, None)
    assert rc == 1


def test_noalloc_refuses_a_capturing_stream():
    """The call waits for its stream, which a capturing stream cannot do: it
    returns VLM_ERR_INVALID before it launches anything, and the capture
    stays valid."""
    L = lib.load()
    rng = np.random.default_rng(3)
    corners, rvc, gam = rings(rng, 10)
    dev = torch.device("cuda")
    tc, tr, tg = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (corners, rvc, gam))
    tp = torch.rand(10, 3, dtype=torch.float64, device=dev)
    tv = torch.zeros_like(tp)
    x = torch.zeros(4, device=dev)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        x += 1.0
        rc = L.vlm_biot_savart_rings_noalloc(tc.data_ptr(), tr.data_ptr(), tg.data_ptr(), 10, tp.data_ptr(), 10,
                                             tv.data_ptr(), lib.PREC_FP64, ctypes.c_void_p(s.cuda_stream))
    assert rc == 1
    buf = ctypes.create_string_buffer(512)
    L.vlm_last_error(buf, 512)
    assert b"capturing" in buf.value
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(x.cpu(), torch.ones(4))

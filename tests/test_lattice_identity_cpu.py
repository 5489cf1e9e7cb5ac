"""The lattice form's identity on the oracle (FP64, CPU): a near-wake
lattice summed ring by ring equals its edges summed once with the
circulation differences of the rings that share them, the border edges and
the edges whose neighbours differ in core radius kept with their own ring's
circulation.  The edge weights follow the device gather's rule
(lattice_weights in volcanor_gb300/csrc/solver.cu)."""
import numpy as np

from oracle import oracle as O


def lattice(rows=6, cols=5, seed=0):
    rng = np.random.default_rng(seed)
    # nodes (rows+1) x (cols+1) of a wavy sheet; ring (i, j) has corners
    # c0 = node(i, j), c1 = node(i+1, j), c2 = node(i+1, j+1), c3 = node(i, j+1)
    x, y = np.meshgrid(np.linspace(0, 1.2, rows + 1), np.linspace(0, 1.0, cols + 1), indexing="ij")
    z = 0.05 * np.sin(3 * x) * np.cos(2 * y) + rng.uniform(-0.01, 0.01, x.shape)
    node = np.stack([x, y, z], -1)
    corners = np.zeros((rows, cols, 4, 3))
    corners[:, :, 0] = node[:-1, :-1]
    corners[:, :, 1] = node[1:, :-1]
    corners[:, :, 2] = node[1:, 1:]
    corners[:, :, 3] = node[:-1, 1:]
    rvc = np.full((rows, cols, 4), 0.02)
    rvc[0, :, 1] = 0.03  # the newest row's trailing edge core has grown, its neighbour's not
    rvc[:, :, 2] = rvc[:, :, 0]  # edge 2 copies edge 0 (as the dissipation does)
    rvc[1:, :, 3] = rvc[:-1, :, 1]
    rvc[1, :, 3] = 0.02
    gam = rng.normal(size=(rows, cols))
    gam[2, 3] = 0.0  # a skipped ring
    return corners, rvc, gam


def edge_weights(corners, rvc, gam):
    rows, cols = gam.shape
    W = np.zeros((rows, cols, 4))

    def merge_s(i, j):  # ring (i, j-1) edge 2 == ring (i, j) edge 0 reversed
        a, c = (i, j - 1), (i, j)
        return (np.array_equal(corners[a][3], corners[c][0]) and np.array_equal(corners[a][2], corners[c][1])
                and rvc[a][2] == rvc[c][0])

    def merge_c(i, j):  # ring (i, j) edge 1 == ring (i+1, j) edge 3 reversed
        a, c = (i, j), (i + 1, j)
        return (np.array_equal(corners[c][0], corners[a][1]) and np.array_equal(corners[c][3], corners[a][2])
                and rvc[c][3] == rvc[a][1])

    for i in range(rows):
        for j in range(cols):
            G = gam[i, j]
            W[i, j, 0] = G - gam[i, j - 1] if j > 0 and merge_s(i, j) else G
            W[i, j, 1] = G - gam[i + 1, j] if i + 1 < rows and merge_c(i, j) else G
            W[i, j, 2] = 0.0 if j + 1 < cols and merge_s(i, j + 1) else G
            W[i, j, 3] = 0.0 if i > 0 and merge_c(i - 1, j) else G
    return W


def test_lattice_edges_sum_to_the_ring_sum():
    corners, rvc, gam = lattice()
    rng = np.random.default_rng(1)
    P = np.concatenate([rng.uniform([-0.2, -0.2, -0.3], [1.4, 1.2, 0.3], (200, 3)),
                        corners[1:3, 1:3, 0].reshape(-1, 3)])  # and some lattice nodes
    V_rings = O.vind_rings(corners.reshape(-1, 4, 3), rvc.reshape(-1, 4), gam.reshape(-1), P)
    W = edge_weights(corners, rvc, gam)
    fc, rv, gw = [], [], []
    for k in range(4):
        act = W[:, :, k] != 0.0
        fc.append(np.stack([corners[:, :, k][act], corners[:, :, (k + 1) % 4][act]], 1))
        rv.append(rvc[:, :, k][act])
        gw.append(W[:, :, k][act])
    V_edges = O.vind_filaments(np.concatenate(fc), np.concatenate(rv), np.concatenate(gw), P)
    np.testing.assert_allclose(V_edges, V_rings, rtol=0, atol=1e-12 * np.max(np.abs(V_rings)))
    # interior rings carry two edges; the border, the mismatched rows and
    # the skipped ring's neighbours keep the rest
    n_edges = sum(len(g) for g in gw)
    assert n_edges < 0.7 * 4 * gam.size
    assert np.all(W[-1, :, 1] == gam[-1])       # last row: nothing below
    assert np.all(W[:, -1, 2] == gam[:, -1])    # last station
    assert np.all(W[0, :, 1] == gam[0])         # newest row: cores differ
    assert np.all(W[1, :, 3] == gam[1])

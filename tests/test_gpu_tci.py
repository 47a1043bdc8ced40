"""Tensor cross interpolation into device networks
(ext/ITensorNumericalAnalysisTCIExt/tci_util.jl:21-55)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_interpolate_1d(ina):
    s = ina.continuous_siteinds(ina.named_path_graph(20))
    f = lambda X: np.exp(-X[:, 0]) * np.sin(20 * X[:, 0]) + X[:, 0] ** 2
    g = ina.interpolate(f, s, tol=1e-12, maxbonddim=32)
    # compare on grid points: the network holds f on the 2^20 digit grid
    X = np.floor(np.random.default_rng(0).random((4000, 1)) * 2**20) / 2**20
    assert np.max(np.abs(g.evaluate_batch(X) - f(X))) < 1e-9
    assert g.maxlinkdim() <= 12


def test_interpolate_2d_comb(ina):
    L = 10
    s = ina.continuous_siteinds(ina.named_comb_tree((2, L)),
                                [[(1, j) for j in range(L, 0, -1)], [(2, j) for j in range(1, L + 1)]])
    f = lambda X: np.cos(3 * X[:, 0] + 2 * X[:, 1])
    g = ina.interpolate(f, s, tol=1e-12, maxbonddim=16)
    X = np.floor(np.random.default_rng(1).random((4000, 2)) * 2**L) / 2**L
    assert np.max(np.abs(g.evaluate_batch(X, [1, 2]) - f(X))) < 1e-9


def test_interpolate_a_network(ina):
    """A device network as the black box: the interpolant reproduces it with
    the same bond dimension (exp + sin has QTT rank 3)."""
    s = ina.continuous_siteinds(ina.named_path_graph(16))
    h = ina.exp_itn(s, k=-1.0) + ina.sin_itn(s, k=2 * np.pi)
    g = ina.interpolate(h, s, tol=1e-13)
    X = np.random.default_rng(2).random((2000, 1))
    assert np.max(np.abs(g.evaluate_batch(X) - h.evaluate_batch(X))) < 1e-10
    assert g.maxlinkdim() <= 3


def test_interpolate_binary_tree_3d(ina):
    """A 3-variable function on a 45-vertex binary tree (15 digits per
    variable) through the tree form of TCI; checked on grid points."""
    s = ina.continuous_siteinds(ina.named_binary_tree(45), map_dimension=3)
    f = lambda X: np.cos(X[:, 0] + 2 * X[:, 1]) * np.exp(-X[:, 2]) + X[:, 0] * X[:, 2] ** 2
    g = ina.interpolate(f, s, tol=1e-12, maxbonddim=32)
    X = np.floor(np.random.default_rng(3).random((4000, 3)) * 2**15) / 2**15
    assert np.max(np.abs(g.evaluate_batch(X, [1, 2, 3]) - f(X))) < 1e-9
    assert g.maxlinkdim() <= 16


@pytest.mark.parametrize("shape,rank", [((30, 40), 3), ((64, 64), 64), ((128, 96), 20), ((200, 150), 7)])
def test_device_cross_matches_oracle(ina, shape, rank):
    """tnfa_cross (one CTA on the device, residual in shared memory or, for
    the largest block, in global memory) against the oracle's cross: the same
    pivots in the same order and the same residual, on low-rank, full-rank and
    rank-capped blocks."""
    from itensornumericalanalysis.tci import _aca_full

    import oracle as O

    rng = np.random.default_rng(95 + rank)
    m, n = shape
    M = rng.standard_normal((m, rank)) @ rng.standard_normal((rank, n))
    for tol, cap in ((1e-12, 64), (1e-3, 64), (1e-12, 5), (0.0, 0)):
        got = _aca_full(M, tol, cap)
        ref = O.aca_full(M, tol, cap)
        assert got[0] == ref[0] and got[1] == ref[1], (tol, cap)
        assert got[2] == ref[2] and got[3] == ref[3], (got[2:], ref[2:])
    # ties: a block of equal magnitudes takes the first in row-major order
    T = np.ones((5, 7))
    T[2, 3] = -1.0
    assert _aca_full(T, 0.0, 3)[:2] == O.aca_full(T, 0.0, 3)[:2]

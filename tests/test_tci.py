"""Tensor cross interpolation: the sweep logic on CPU, with the oracle's
cross (numpy) standing in for the device's tnfa_cross (compared with each
other in tests/test_gpu_tci.py)."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "itensornumericalanalysis.jl_gb300"))
sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import oracle as O  # noqa: E402
from itensornumericalanalysis import tci as _tci  # noqa: E402
from itensornumericalanalysis.tci import tci_path  # noqa: E402

_aca_full = O.aca_full


@pytest.fixture(autouse=True)
def _oracle_cross(monkeypatch):
    monkeypatch.setattr(_tci, "_aca_full", O.aca_full)


def _mps_values(cores, idx):
    out = np.ones((idx.shape[0], 1))
    for l, A in enumerate(cores):
        out = np.einsum("pa,pab->pb", out, A[:, idx[:, l], :].transpose(1, 0, 2))
    return out[:, 0]


def _bits_to_x(idx):
    L = idx.shape[1]
    return idx @ (2.0 ** -np.arange(1, L + 1))


def test_aca_recovers_low_rank():
    rng = np.random.default_rng(1)
    M = rng.standard_normal((30, 3)) @ rng.standard_normal((3, 40))
    rows, cols, err, scale = _aca_full(M, 1e-12, 10)
    assert len(rows) == 3 and err <= 1e-10 * scale
    # the cross reproduces M
    C, R, P = M[:, cols], M[rows, :], M[np.ix_(rows, cols)]
    assert np.allclose(C @ np.linalg.solve(P, R), M, atol=1e-10)


def test_tci_1d_smooth_function():
    L = 24
    f = lambda x: np.exp(-x) * np.sin(20 * x) + x**2
    sample = lambda idx: f(_bits_to_x(idx))
    cores, info = tci_path(sample, [2] * L, tol=1e-12, maxbonddim=32)
    rng = np.random.default_rng(2)
    idx = rng.integers(0, 2, (2000, L))
    err = np.max(np.abs(_mps_values(cores, idx) - sample(idx)))
    assert err < 1e-9, (err, info)
    assert max(info["ranks"]) <= 12, info["ranks"]


def test_tci_exact_low_rank_2d():
    """exp(x y) on interleaved digits is not low rank exactly, but
    cos(x + y) = cos x cos y - sin x sin y has rank 2 across the split."""
    L = 10
    f = lambda x, y: np.cos(3 * x + 2 * y)
    def sample(idx):
        return f(_bits_to_x(idx[:, :L]), _bits_to_x(idx[:, L:][:, ::-1]))
    cores, info = tci_path(sample, [2] * (2 * L), tol=1e-12, maxbonddim=16)
    idx = np.random.default_rng(3).integers(0, 2, (1000, 2 * L))
    assert np.max(np.abs(_mps_values(cores, idx) - sample(idx))) < 1e-10
    assert info["ranks"][L - 1] == 2


def test_interpolate_layout_through_the_oracle(monkeypatch):
    """interpolate() hands the device layout [site, parent, children] to the
    library; intercept it and contract those tensors with the oracle."""
    import itensornumericalanalysis as ina
    from itensornumericalanalysis.network import ITensorNetworkFunction

    captured = {}

    def fake_from_tensors(cls, s, ts, ctx=None, legs=None, dtype=None):
        captured["s"], captured["ts"] = s, ts

        class Dummy:
            pass
        return Dummy()

    monkeypatch.setattr(ITensorNetworkFunction, "from_tensors", classmethod(fake_from_tensors))
    L = 6
    g = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g, [[(1, j) for j in range(L, 0, -1)], [(2, j) for j in range(1, L + 1)]])
    f = lambda X: np.exp(X[:, 0] - 2 * X[:, 1]) + X[:, 0] * X[:, 1]
    ina.interpolate(f, s, tol=1e-13)
    ts = captured["ts"]
    lay = s.layout
    X = np.random.default_rng(4).random((50, 2))
    X = np.floor(X * 2**L) / 2**L  # grid points: the interpolant is exact there

    def value(x):
        iv = s.calculate_ind_values([x[0], x[1]], [1, 2])

        def up(i):  # vector over vertex i's parent bond
            v = lay.order[i]
            T = ts[v][iv[s.legs[v][0]]]  # [parent, children...]
            for c in reversed(lay.children[i]):
                T = T @ up(c)
            return T
        return float(up(0)[0])

    got = np.array([value(x) for x in X])
    assert np.max(np.abs(got - f(X))) < 1e-11


def _heap_tree(n):
    nbrs = [[] for _ in range(n)]
    for v in range(1, n):
        p = (v - 1) // 2
        nbrs[p].append(v)
        nbrs[v].append(p)
    return nbrs


def test_tci_tree_on_a_binary_tree():
    """tci_tree on a 31-vertex binary tree, 3 variables with round-robin
    digits: the assembled cross form matches f at random digit strings."""
    from itensornumericalanalysis.tci import _tree_values, tci_tree

    n = 31
    nbrs = _heap_tree(n)
    var = [v % 3 for v in range(n)]
    dig = [v // 3 + 1 for v in range(n)]

    def sample(idx):
        X = np.zeros((idx.shape[0], 3))
        for v in range(n):
            X[:, var[v]] += idx[:, v] * 2.0 ** (-dig[v])
        return np.cos(X[:, 0] + 2 * X[:, 1]) * np.exp(-X[:, 2]) + X[:, 0] * X[:, 2] ** 2

    cores, info = tci_tree(sample, nbrs, [2] * n, tol=1e-12, maxbonddim=32)
    idx = np.random.default_rng(5).integers(0, 2, (4000, n))
    err = np.max(np.abs(_tree_values(cores, nbrs, 0, idx) - sample(idx)))
    assert err < 1e-10, (err, info)
    assert max(info["ranks"]) <= 12, info


def test_tci_tree_agrees_with_path_version():
    """On a path both formulations interpolate to the tolerance."""
    from itensornumericalanalysis.tci import _tree_values, tci_tree

    L = 20
    nbrs = [[j for j in (i - 1, i + 1) if 0 <= j < L] for i in range(L)]
    f = lambda x: np.exp(-x) * np.sin(20 * x) + x**2
    sample = lambda idx: f(_bits_to_x(idx))
    cores, info = tci_tree(sample, nbrs, [2] * L, tol=1e-12, maxbonddim=32)
    pcores, pinfo = tci_path(sample, [2] * L, tol=1e-12, maxbonddim=32)
    idx = np.random.default_rng(6).integers(0, 2, (2000, L))
    assert np.max(np.abs(_tree_values(cores, nbrs, 0, idx) - sample(idx))) < 1e-9
    assert np.max(np.abs(_mps_values(pcores, idx) - sample(idx))) < 1e-9
    assert max(info["ranks"]) <= max(pinfo["ranks"]) + 2


def test_interpolate_tree_layout_through_the_oracle(monkeypatch):
    """interpolate() on a non-path tree (a comb with three teeth): the layout
    tensors [site, parent, children] handed to the library contract to f on
    grid points."""
    import itensornumericalanalysis as ina
    from itensornumericalanalysis.network import ITensorNetworkFunction

    captured = {}

    def fake_from_tensors(cls, s, ts, ctx=None, legs=None, dtype=None):
        captured["ts"] = ts

        class Dummy:
            pass
        return Dummy()

    monkeypatch.setattr(ITensorNetworkFunction, "from_tensors", classmethod(fake_from_tensors))
    L = 5
    g = ina.named_comb_tree((3, L))
    s = ina.continuous_siteinds(g, [[(i, j) for j in range(1, L + 1)] for i in range(1, 4)])
    f = lambda X: np.exp(X[:, 0] - X[:, 1]) * np.cos(2 * X[:, 2]) + X[:, 1] * X[:, 2]
    ina.interpolate(f, s, tol=1e-13)
    ts = captured["ts"]
    lay = s.layout
    X = np.floor(np.random.default_rng(7).random((60, 3)) * 2**L) / 2**L

    def value(x):
        iv = s.calculate_ind_values(list(x), [1, 2, 3])

        def up(i):
            v = lay.order[i]
            T = ts[v][iv[s.legs[v][0]]]
            for c in reversed(lay.children[i]):
                T = T @ up(c)
            return T
        return float(up(0)[0])

    got = np.array([value(x) for x in X])
    assert np.max(np.abs(got - f(X))) < 1e-11


def test_tci_tree_on_random_trees():
    """Prüfer-random trees (vertices of degree up to 5) with one digit per
    vertex: the cross form reproduces f at random digit strings."""
    from itensornumericalanalysis.tci import _tree_values, tci_tree

    for seed, n in ((11, 18), (12, 25)):
        rng = np.random.default_rng(seed)
        prufer = rng.integers(0, n, n - 2)
        degree = np.ones(n, dtype=int)
        for x in prufer:
            degree[x] += 1
        nbrs = [[] for _ in range(n)]
        for x in prufer:
            leaf = int(np.flatnonzero(degree == 1)[0])
            nbrs[leaf].append(int(x))
            nbrs[int(x)].append(leaf)
            degree[leaf] -= 1
            degree[x] -= 1
        u, w = (int(i) for i in np.flatnonzero(degree == 1))
        nbrs[u].append(w)
        nbrs[w].append(u)
        var = [v % 2 for v in range(n)]
        dig = [v // 2 + 1 for v in range(n)]

        def sample(idx):
            X = np.zeros((idx.shape[0], 2))
            for v in range(n):
                X[:, var[v]] += idx[:, v] * 2.0 ** (-dig[v])
            return np.exp(-X[:, 0]) * np.cos(3 * X[:, 1]) + X[:, 0] * X[:, 1]

        cores, info = tci_tree(sample, nbrs, [2] * n, tol=1e-12, maxbonddim=32)
        idx = rng.integers(0, 2, (3000, n))
        err = np.max(np.abs(_tree_values(cores, nbrs, 0, idx) - sample(idx)))
        assert err < 1e-10, (seed, err, info)
        assert max(len(x) for x in nbrs) >= 3

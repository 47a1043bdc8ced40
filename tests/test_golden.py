"""The oracle reproduces the committed golden fixtures (tests/golden/), and the
fixtures satisfy the analytic facts they encode."""
from pathlib import Path

import numpy as np
import pytest

import oracle as O

G = Path(__file__).resolve().parent / "golden"


def test_config1_fixture_is_oracle_output():
    d = np.load(G / "config1_path12.npz")
    L = 12
    so = O.siteinds(O.path_graph(L))
    f = O.net_add(O.exp_itn(so, k=-1.0), O.sin_itn(so, k=2 * np.pi))
    F, _ = O.dense_grid_1d(f)
    assert np.allclose(F.real, d["f_grid"], rtol=0, atol=1e-13)
    x = np.arange(2**L) / 2**L
    assert np.allclose(d["f_grid"], np.exp(-x) + np.sin(2 * np.pi * x), atol=1e-12)
    # interior second difference ~ f'' to O(delta^2)
    fpp = np.exp(-x) - (2 * np.pi) ** 2 * np.sin(2 * np.pi * x)
    assert np.max(np.abs(d["d2f_grid"][1:-1] - fpp[1:-1])) < 1e-3


def test_shift_fixture_identities():
    d = np.load(G / "shifts_comb2x3_poly.npz")
    F = d["f"]
    assert np.allclose(d["fwd_Dirichlet_0"][:-1], F[1:]) and d["fwd_Dirichlet_0"][-1] == 0
    assert np.allclose(d["bwd_Periodic_1"][2:], F[:-2]) and np.allclose(d["bwd_Periodic_1"][:2], F[-2:])
    assert np.allclose(d["fwd_Neumann_0"][-1], F[-1])


def test_random_tree_fixture_reproduces():
    d = np.load(G / "random_binary15_chi4.npz")
    import sys
    sys.path.insert(0, str(G))
    from make_golden import canonical_random, to_oracle
    from itensornumericalanalysis.graphs import named_binary_tree

    s, flat, shapes = canonical_random(named_binary_tree(15), 3, 4, seed=101)
    assert np.array_equal(np.concatenate(flat), d["tensors"])
    net = to_oracle(s, flat, shapes, O.binary_tree_graph(15))
    vals = np.array([O.evaluate(net, list(x), [1, 2, 3]) for x in d["X"][:16]])
    assert np.allclose(vals, d["values"][:16], rtol=1e-13, atol=0)


def test_complex_fixture_matches_analytic():
    d = np.load(G / "complex_cosh_comb2x3.npz")
    k, a, c = complex(d["k"]), complex(d["a"]), complex(d["c"])
    Z = d["Z"]
    # the digit map truncates each part to 3 binary digits
    zq = np.floor(Z.real * 8) / 8 + 1j * np.floor(Z.imag * 8) / 8
    assert np.allclose(d["values"], c * np.cosh(k * zq + a), rtol=1e-12)


def _fixture_tensors(d, s):
    flat, ts, off = d["tensors"], {}, 0
    for v, sh in zip(s.layout.order, d["shapes"]):
        sh = tuple(int(x) for x in sh if x > 0)
        n = int(np.prod(sh))
        ts[v] = flat[off:off + n].reshape(sh)
        off += n
    return ts


def test_partial_fixture_is_oracle_output():
    import sys
    sys.path.insert(0, str(G))
    from make_golden import to_oracle
    from itensornumericalanalysis.graphs import named_comb_tree
    from itensornumericalanalysis.indexmap import continuous_siteinds
    d = np.load(G / "partial_comb3x3_chi3.npz")
    s = continuous_siteinds(named_comb_tree((3, 3)), map_dimension=3)
    ts = _fixture_tensors(d, s)
    shapes = [ts[v].shape for v in s.layout.order]
    net = to_oracle(s, [ts[v].ravel() for v in s.layout.order], shapes, O.comb_tree_graph((3, 3)))
    so = net.s
    order = sorted((i for v in so.verts for i in so.site[v]), key=lambda i: so.info[i][:2])
    F = O.dense(net, order).reshape(8, 8, 8)
    assert np.allclose(F.mean(axis=1), d["p2"], atol=1e-14)
    # the fixtures are consistent with each other
    assert np.allclose(d["p2"].mean(axis=1), d["p23"], atol=1e-14)
    assert np.allclose(d["p1_sum"] / 8, F.mean(axis=0), atol=1e-14)


def test_linsolve_fixture_solves_the_stencil():
    d = np.load(G / "linsolve_path9.npz")
    L = 9
    N = 2**L
    x = d["x_grid"]
    # (x[i+1] - 2 x[i] + x[i-1]) 4^L = b[i], Dirichlet zeros outside the grid
    xp = np.concatenate([[0.0], x, [0.0]])
    lap = (xp[2:] - 2 * xp[1:-1] + xp[:-2]) * 4.0**L
    assert np.max(np.abs(lap - d["b_grid"])) <= 1e-9 * np.max(np.abs(d["b_grid"]))

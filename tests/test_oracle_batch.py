"""The oracle's batched evaluate (message passing over many points) against
its per-point evaluate, which restates itensornetworkfunction.jl:96-106
directly: trees, forests, complex maps and a graph with a cycle (per-point
fallback)."""
import numpy as np
import pytest

import oracle as O


@pytest.mark.parametrize("gname,md", [("binary9", 3), ("comb3x4", 2), ("path6", 1)])
def test_batch_equals_per_point(gname, md):
    graph = {"binary9": O.binary_tree_graph(9), "comb3x4": O.comb_tree_graph((3, 4)),
             "path6": O.path_graph(6)}[gname]
    rng = np.random.default_rng(81)
    s = O.siteinds(graph, map_dimension=md)
    net = O.random_net(s, 3, rng)
    X = rng.random((37, md))
    dims = list(range(1, md + 1))
    got = O.evaluate_batch(net, X, dims)
    ref = np.array([O.evaluate(net, list(x), dims) for x in X])
    assert np.max(np.abs(got - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))


def test_batch_leaf_root_and_single_vertex():
    rng = np.random.default_rng(82)
    for graph in (O.path_graph(1), O.path_graph(2)):
        s = O.siteinds(graph)
        net = O.random_net(s, 2, rng)
        X = rng.random((11, 1))
        got = O.evaluate_batch(net, X)
        ref = np.array([O.evaluate(net, list(x)) for x in X])
        assert np.allclose(got, ref, rtol=1e-13, atol=1e-14)


def test_batch_with_cycle_falls_back():
    rng = np.random.default_rng(83)
    s = O.siteinds(O.grid_graph((2, 3)), map_dimension=2)
    net = O.random_net(s, 2, rng)
    X = rng.random((9, 2))
    got = O.evaluate_batch(net, X, [1, 2])
    ref = np.array([O.evaluate(net, list(x), [1, 2]) for x in X])
    assert np.allclose(got, ref, rtol=1e-13, atol=1e-14)


def test_batch_complex_map():
    rng = np.random.default_rng(84)
    s = O.complex_siteinds(O.comb_tree_graph((2, 3)))
    net = O.random_net(s, 2, rng)
    X = rng.random(13) + 1j * rng.random(13)
    got = O.evaluate_batch(net, X)
    ref = np.array([O.evaluate(net, [x]) for x in X])
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-13)

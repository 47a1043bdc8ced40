"""Maps on graphs with cycles (the reference evaluates functions on
named_grid graphs, test/test_realitensorfunction.jl:39-57,147-160): the tree
image of vertex groups and the exact merge of a network onto it, checked on
the CPU against the oracle's contraction of the network with its cycles."""
import numpy as np
import pytest

import oracle as O
from _helpers import oracle_to_graph_tensors, product_map


def _dense_of_image(img, ts):
    """The full function tensor of tensors on a tree map, over its legs in
    layout order (numpy contraction)."""
    lay = img.layout
    ops, nsym, out = [], 0, []
    bond = {}
    for i, v in enumerate(lay.order):
        t = ts[v]
        nl = len(img.legs[v])
        sub = list(range(nsym, nsym + nl))
        nsym += nl
        out += sub
        for j in [lay.parent[i]] if lay.parent[i] >= 0 else [None]:
            key = (min(i, j), max(i, j)) if j is not None else ("root", i)
            bond.setdefault(key, 30 + len(bond))
            sub.append(bond[key])
        for c in lay.children[i]:
            key = (min(i, c), max(i, c))
            bond.setdefault(key, 30 + len(bond))
            sub.append(bond[key])
        ops += [t, sub]
    return np.einsum(*ops, out, optimize=True)


@pytest.mark.parametrize("dims,chi,nd", [((3, 3), 2, 1), ((3, 2), 3, 2), ((2, 2, 2), 2, 3)])
def test_merge_onto_tree_image_is_exact(dims, chi, nd):
    import itensornumericalanalysis as ina

    graph = O.grid_graph(dims)
    rng = np.random.default_rng(sum(dims) + chi)
    s_or = O.siteinds(graph, map_dimension=nd)
    net = O.random_net(s_or, chi, rng)
    s = product_map(ina, graph, s_or)
    assert not s.graph.is_forest()
    img = s.tree_image
    assert img.graph.is_tree() and img.tree_image is img
    merged = ina.merge_to_tree_image(s, oracle_to_graph_tensors(net, s))
    got = _dense_of_image(img, merged)
    legs = [l for v in img.layout.order for l in img.legs[v]]
    order = [s_or.ind(l.dim, l.digit) for l in legs]
    ref = O.dense(net, order)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_tree_groups_of_grids():
    import itensornumericalanalysis as ina

    for dims, ngroups in (((3, 3), 3), ((3, 2), 3), ((4, 4), 4)):
        s = ina.continuous_siteinds(ina.named_grid(dims))
        img = s.tree_image
        assert len(img.groups) == ngroups and img.graph.is_tree()
        assert sorted(v for gr in img.groups.values() for v in gr) == sorted(s.vertices())
        assert [l for v in img.layout.order for l in img.legs[v]] != []
    path = ina.continuous_siteinds(ina.named_grid((5, 1)))
    assert path.tree_image is path

"""Helpers shared by the tests: move networks between the oracle's labelled
tensors and the product's canonical device layout."""
from __future__ import annotations

import numpy as np

import oracle as O


def product_map(ina, graph, s_or: O.SiteMap):
    """The product IndsNetworkMap with the same graph and legs as an oracle SiteMap."""
    verts, edges = graph
    g = ina.NamedGraph(verts, edges)
    legs = {}
    for v in verts:
        legs[v] = [
            ina.SiteLeg(v, s_or.info[i][0], s_or.info[i][1], i.dim, "real" if s_or.info[i][2] else "imag")
            for i in s_or.site[v]
        ]
    return ina.IndsNetworkMap(g, legs, s_or.is_complex)


def oracle_to_tensors(net: O.Net, s_prod) -> dict:
    """Per-vertex arrays in the product layout [site..., parent, children...]."""
    lay = s_prod.layout
    out = {}
    for i, v in enumerate(lay.order):
        nb = lay.neighbours_in_layout_order(i)
        links = [net.link[frozenset((v, lay.order[j]))] for j in nb]
        t = net.T[v].permute(net.s.site[v] + links).arr
        if lay.parent[i] < 0:
            t = t.reshape(t.shape[: len(net.s.site[v])] + (1,) + t.shape[len(net.s.site[v]):])
        out[v] = t
    return out


def upload_oracle(ina, graph, net: O.Net, dtype=None):
    s = product_map(ina, graph, net.s)
    ts = oracle_to_tensors(net, s)
    return ina.ITensorNetworkFunction.from_tensors(s, ts, dtype=dtype), s


def rel_err(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def oracle_to_graph_tensors(net: O.Net, s_prod) -> dict:
    """Per-vertex arrays [site..., bonds to the neighbours in the product
    graph's neighbour order] (the input form for graphs with cycles)."""
    g = s_prod.graph
    out = {}
    for v in g.vertices():
        links = [net.link[frozenset((v, w))] for w in g.neighbors(v)]
        out[v] = net.T[v].permute(net.s.site[v] + links).arr
    return out

"""Generate the golden fixtures in this directory from the CPU oracle.

    python tests/golden/make_golden.py

Each fixture is a small .npz holding seeded inputs (tensors in the device's
canonical layout where a network is random, coordinates) and the oracle's
outputs.  The reference itself (Julia) cannot run here, so the oracle -- pinned
to the reference's known-answer tests in tests/test_oracle_pins.py -- produces
the expected values.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "itensornumericalanalysis.jl_gb300"))

import oracle as O  # noqa: E402
from itensornumericalanalysis.graphs import named_binary_tree, named_comb_tree  # noqa: E402
from itensornumericalanalysis.indexmap import continuous_siteinds  # noqa: E402


def canonical_random(g, map_dimension, chi, seed):
    """Random tensors in the canonical layout of the device for graph g."""
    s = continuous_siteinds(g, map_dimension=map_dimension)
    lay = s.layout
    rng = np.random.default_rng(seed)
    flat, shapes = [], []
    for i, v in enumerate(lay.order):
        shape = tuple(l.base for l in s.legs[v]) + ((chi,) if lay.parent[i] >= 0 else (1,)) + (
            (chi,) * len(lay.children[i]))
        t = rng.standard_normal(shape)
        t /= np.linalg.norm(t)
        flat.append(t.ravel())
        shapes.append(shape)
    return s, flat, shapes


def to_oracle(s, flat, shapes, graph):
    so = O.siteinds(graph, map_dimension=max(l.dim for l in s.inds()))
    lay = s.layout
    chi = {}
    for i, v in enumerate(lay.order):
        if lay.parent[i] >= 0:
            chi[frozenset((v, lay.order[lay.parent[i]]))] = shapes[i][len(s.legs[v])]
    link = {frozenset(e): O.Index(chi[frozenset(e)], "L") for e in so.edges}
    net = O.Net(so, {}, link)
    for i, v in enumerate(lay.order):
        arr = flat[i].reshape(shapes[i])
        nl = len(s.legs[v])
        if lay.parent[i] < 0:
            arr = arr.reshape(arr.shape[:nl] + arr.shape[nl + 1:])
        nb = lay.neighbours_in_layout_order(i)
        net.T[v] = O.Tensor(arr, so.site[v] + [link[frozenset((v, lay.order[j]))] for j in nb])
    return net


def random_tree_fixture():
    g = named_binary_tree(15)
    s, flat, shapes = canonical_random(g, 3, 4, seed=101)
    net = to_oracle(s, flat, shapes, O.binary_tree_graph(15))
    rng = np.random.default_rng(102)
    X = rng.random((128, 3))
    vals = np.array([O.evaluate(net, list(x), [1, 2, 3]) for x in X])
    np.savez_compressed(
        HERE / "random_binary15_chi4.npz",
        tensors=np.concatenate(flat), shapes=np.array([np.pad(sh, (0, 4 - len(sh)), constant_values=0)
                                                       for sh in shapes]),
        X=X, values=vals, integral=O.integrate(net), integral_sum=O.integrate(net, take_sum=True))


def config1_fixture(L=12):
    so = O.siteinds(O.path_graph(L))
    f = O.net_add(O.exp_itn(so, k=-1.0), O.sin_itn(so, k=2 * np.pi))
    F, _ = O.dense_grid_1d(f)
    terms = O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2)
    G = O.apply_terms_dense(terms, F.reshape((2,) * L), {(1, k): k - 1 for k in range(1, L + 1)})
    rng = np.random.default_rng(0)
    X = rng.random((256, 1))
    idx = np.floor(X[:, 0] * 2**L).astype(int)
    np.savez_compressed(HERE / f"config1_path{L}.npz", X=X, f=F.real[idx], d2f=G.reshape(-1).real[idx],
                        f_grid=F.real, d2f_grid=G.reshape(-1).real, integral_f=np.mean(F.real),
                        integral_d2f=np.mean(G.real))


def shift_fixture():
    so = O.siteinds(O.comb_tree_graph((2, 3)))
    F, _ = O.dense_grid_1d(O.poly_itn(so, [1.0, 0.5, 0.25]))
    out = {"f": F.real}
    L = 6
    for b in ["Dirichlet", "Periodic", "Neumann"]:
        for n in [0, 1]:
            for fwd in [True, False]:
                terms = (O.forward_shift_terms if fwd else O.backward_shift_terms)(L, 1, b, n)
                G = O.apply_terms_dense(terms, F.reshape((2,) * L), {(1, k): k - 1 for k in range(1, L + 1)})
                out[f"{'fwd' if fwd else 'bwd'}_{b}_{n}"] = G.reshape(-1).real
    np.savez_compressed(HERE / "shifts_comb2x3_poly.npz", **out)


def complex_fixture():
    graph = O.comb_tree_graph((2, 3))
    so = O.complex_siteinds(graph, [[(1, 1), (1, 2), (1, 3)]], [[(2, 1), (2, 2), (2, 3)]])
    k, a, c = 0.3 + 0.7j, 0.2 - 0.1j, 1.1 + 0.4j
    f = O.cosh_itn(so, k=k, a=a, c=c)
    rng = np.random.default_rng(103)
    Z = rng.random(64) + 1j * rng.random(64)
    vals = np.array([O.evaluate(f, [z]) for z in Z])
    np.savez_compressed(HERE / "complex_cosh_comb2x3.npz", Z=Z, values=vals, k=k, a=a, c=c)


def _pack(flat, shapes):
    return np.concatenate(flat), np.array([np.pad(sh, (0, 5 - len(sh)), constant_values=0) for sh in shapes])


def partial_fixture():
    """A random 3-variable comb (3, 3), chi 3, digits round robin; the dense
    left Riemann sums over subsets of the variables (src/integration.jl:35-54)."""
    from itensornumericalanalysis.graphs import named_comb_tree
    g = named_comb_tree((3, 3))
    s, flat, shapes = canonical_random(g, 3, 3, seed=104)
    net = to_oracle(s, flat, shapes, O.comb_tree_graph((3, 3)))
    so = net.s
    order = sorted((i for v in so.verts for i in so.site[v]), key=lambda i: so.info[i][:2])
    F = O.dense(net, order).reshape(8, 8, 8)
    t, sh = _pack(flat, shapes)
    np.savez_compressed(HERE / "partial_comb3x3_chi3.npz", tensors=t, shapes=sh,
                        p2=F.mean(axis=1), p23=F.mean(axis=(1, 2)), p13=F.mean(axis=(0, 2)),
                        p1_sum=F.sum(axis=0))


def linsolve_fixture(L=9):
    """d2/dx2 x = b on a 9-bit path (Dirichlet, scaled), b random with bond 2:
    the dense FP64 solution with the oracle's stencil matrix."""
    from itensornumericalanalysis.graphs import named_grid
    g = named_grid((L, 1))
    s, flat, shapes = canonical_random(g, 1, 2, seed=105)
    net = to_oracle(s, flat, shapes, O.path_graph(L))
    B, _ = O.dense_grid_1d(net)
    N = 2**L
    eye = np.eye(N).reshape((2,) * L + (N,))
    M = O.apply_terms_dense(O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2), eye,
                            {(1, k): k - 1 for k in range(1, L + 1)}).reshape(N, N)
    x = np.linalg.solve(M, B.real)
    t, sh = _pack(flat, shapes)
    np.savez_compressed(HERE / f"linsolve_path{L}.npz", tensors=t, shapes=sh, b_grid=B.real, x_grid=x,
                        cond=np.linalg.cond(M))


if __name__ == "__main__":
    random_tree_fixture()
    config1_fixture()
    shift_fixture()
    complex_fixture()
    partial_fixture()
    linsolve_fixture()
    print("fixtures written to", HERE)

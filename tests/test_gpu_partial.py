"""partial_integrate, multiply on partially shared vertex sets and the
Fredholm fixed point on the GPU (test/test_integration.jl:40-54,
examples/fredholm_solver.jl:43-65), checked against the oracle's dense
tensors and analytic values."""
import numpy as np
import pytest

import oracle as O
from _helpers import rel_err, upload_oracle

pytestmark = pytest.mark.gpu


def test_partial_integration_3d_reference(ina):
    """test/test_integration.jl:40-54: exp(x) cos(y) exp(z) on three teeth of
    a comb, integrated over y and z, at x = 0.875 within 1e-8."""
    L = 90
    g = ina.named_comb_tree((3, L // 3))
    s = ina.continuous_siteinds(g, [[(i, j) for j in range(1, L // 3 + 1)] for i in range(1, 4)])
    s1, s2, s3 = (ina.reduced_indsnetworkmap(s, d) for d in (1, 2, 3))
    f = ina.exp_itn(s1, dim=1) * ina.cos_itn(s2, dim=2) * ina.exp_itn(s3, dim=3)
    fx = ina.partial_integrate(f, [2, 3])
    assert fx.s.dimensions() == [1]
    x = 0.875
    expect = (np.e - 1) * np.sin(1) * np.exp(x)
    assert abs(fx.evaluate_batch([x])[0] - expect) <= 1e-8


def _dense_by_dim(net, s_or, ndims, L):
    order = sorted((i for v in s_or.verts for i in s_or.site[v]), key=lambda i: s_or.info[i][:2])
    return O.dense(net, order).reshape((2**L,) * ndims)


@pytest.mark.parametrize("dims", [[2], [2, 3], [1, 3], [1]])
@pytest.mark.parametrize("merge", [True, False])
def test_partial_integrate_random_tree(ina, dims, merge):
    """A random 3-variable comb (backbone included): the merged network equals
    the dense tensor averaged over the integrated variables."""
    graph = O.comb_tree_graph((3, 3))
    s_or = O.siteinds(graph, map_dimension=3)
    rng = np.random.default_rng(80)
    net = O.random_net(s_or, 3, rng)
    f, s = upload_oracle(ina, graph, net)
    F = _dense_by_dim(net, s_or, 3, 3)
    g = ina.partial_integrate(f, dims, merge_vertices=merge)
    keep = [d for d in (1, 2, 3) if d not in dims]
    G = F.mean(axis=tuple(d - 1 for d in dims))
    assert sorted(g.s.dimensions()) == keep
    if merge:
        assert all(g.s.legs[v] for v in g.s.vertices())
    else:
        assert g.s.nv() == s.nv()
    grid = np.arange(8) / 8.0
    mesh = np.stack(np.meshgrid(*([grid] * len(keep)), indexing="ij"), axis=-1).reshape(-1, len(keep))
    got = g.evaluate_batch(mesh, keep)
    assert rel_err(got, G.reshape(-1)) < 1e-12


def test_partial_integrate_take_sum_and_complex(ina):
    graph = O.comb_tree_graph((2, 3))
    s_or = O.siteinds(graph, map_dimension=2)
    rng = np.random.default_rng(81)
    net = O.random_net(s_or, 2, rng)
    f, s = upload_oracle(ina, graph, net)
    F = _dense_by_dim(net, s_or, 2, 3)
    g = ina.partial_integrate(f, [1], take_sum=True)
    grid = np.arange(8) / 8.0
    assert rel_err(g.evaluate_batch(grid, [2]), F.sum(axis=0)) < 1e-12
    fc = f.astype(ina._lib.C128)
    fc.scale_vertex(s.layout.order[0], 1j)
    gc = ina.partial_integrate(fc, [2])
    assert rel_err(gc.evaluate_batch(grid, [1]), 1j * F.mean(axis=1)) < 1e-12


def test_partial_integrate_everything_rejected(ina):
    s = ina.continuous_siteinds(ina.named_comb_tree((2, 3)), map_dimension=2)
    f = ina.rand_itn(s, link_space=2, rng=82)
    with pytest.raises(ina.TnfaError, match="integrate"):
        ina.partial_integrate(f, [1, 2])


def test_multiply_partially_shared_vertices(ina):
    """g(x, y) on a 2-D comb times h(y) on the y-tooth: the product lives on
    the comb with bond dims multiplied on the y-tooth."""
    L = 4
    g_ = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g_, [[(1, j) for j in range(1, L + 1)], [(2, j) for j in range(1, L + 1)]])
    s2 = ina.reduced_indsnetworkmap(s, 2)
    g = ina.rand_itn(s, link_space=3, rng=83)
    h = ina.rand_itn(s2, link_space=2, rng=84)
    p = g * h
    assert p.s.same_structure(s)
    X = np.random.default_rng(85).random((300, 2))
    assert rel_err(p.evaluate_batch(X, [1, 2]), g.evaluate_batch(X, [1, 2]) * h.evaluate_batch(X[:, 1], [2])) < 1e-12
    q = h * g
    assert rel_err(q.evaluate_batch(X, [1, 2]), p.evaluate_batch(X, [1, 2])) < 1e-12


def test_fredholm_fixed_point(ina):
    """examples/fredholm_solver.jl:43-65 at 2 x 30 bits: f = e^x + x int_0^1 y
    f(y) dy, whose solution is 3x/2 + e^x."""
    L = 60
    g_ = ina.named_comb_tree((2, L // 2))
    s = ina.continuous_siteinds(g_, [[(i, j) for j in range(1, L // 2 + 1)] for i in range(1, 3)])
    s1, s2 = ina.reduced_indsnetworkmap(s, 1), ina.reduced_indsnetworkmap(s, 2)
    dim_psi = 2
    psi = ina.const_itn(s2)
    kern = ina.poly_itn(s1, [0, 1], dim=1) * ina.poly_itn(s2, [0, 1], dim=2)
    c1, c2 = ina.exp_itn(s1, dim=1), ina.exp_itn(s2, dim=2)
    for _ in range(40):
        psi = psi * kern
        psi = ina.partial_integrate(psi, [dim_psi])
        dim_psi = 1 if dim_psi == 2 else 2
        psi = psi + (c1 if dim_psi == 1 else c2)
    xs = np.array(ina.grid_points(s, 100, dim_psi))
    vals = psi.evaluate_batch(xs, [dim_psi])
    avg_err = np.mean(np.abs(vals - (1.5 * xs + np.exp(xs))))
    assert avg_err < 1e-7, avg_err
    assert psi.maxlinkdim() <= 3

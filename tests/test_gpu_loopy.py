"""Functions on graphs with cycles, evaluated and integrated on the GPU: the
reference's named_grid cases (test/test_realitensorfunction.jl:39-57,147-160,
191-206; test/test_complexitensorfunction.jl:38-56,158-171,212-226) against
their analytic values, and random networks on grids against the oracle's
contraction of the network with its cycles (its evaluate and integrate)."""
import numpy as np
import pytest

import oracle as O
from _helpers import oracle_to_graph_tensors, product_map, rel_err

pytestmark = pytest.mark.gpu

RTOL = np.sqrt(np.finfo(float).eps)  # the reference's default isapprox


def test_const_on_grid(ina):
    """test_realitensorfunction.jl:39-57 and :147-160."""
    s = ina.continuous_siteinds(ina.named_grid((3, 3)))
    assert not s.graph.is_forest()
    assert abs(ina.const_itn(s, c=1.5).evaluate(0.5) - 1.5) <= RTOL * 1.5
    assert abs(ina.const_itn(s, c=1.5, linkdim=4).evaluate(0.5) - 1.5) <= RTOL * 1.5
    s3 = ina.continuous_siteinds(ina.named_grid((3, 3)), map_dimension=3)
    assert abs(ina.const_itn(s3, c=1.5).evaluate([0.5, 0.25, 0.0], [1, 2, 3]) - 1.5) <= RTOL * 1.5


def test_tanh_sum_on_grid(ina):
    """test_realitensorfunction.jl:191-206: c tanh(kx+a) + c tanh(ky+a) on
    named_grid((3, 2)) with 20 series terms each."""
    rng = np.random.default_rng(1234)
    a, k, c = rng.random(3)
    s = ina.continuous_siteinds(ina.named_grid((3, 2)), map_dimension=2)
    f = ina.tanh_itn(s, k=k, a=a, c=c, nterms=20, dim=1) + ina.tanh_itn(s, k=k, a=a, c=c, nterms=20, dim=2)
    x, y = 0.625, 0.875
    exact = c * np.tanh(k * x + a) + c * np.tanh(k * y + a)
    assert abs(f.evaluate([x, y], [1, 2]) - exact) <= RTOL * abs(exact)


def test_complex_maps_on_grid(ina):
    """test_complexitensorfunction.jl:38-56, :158-171 and :212-226."""
    s = ina.complex_continuous_siteinds(ina.named_grid((3, 3)))
    z = 0.5 + 0.625j
    assert abs(ina.const_itn(s, c=1.5).evaluate(z) - 1.5) <= RTOL * 1.5
    assert abs(ina.const_itn(s, c=1.5, linkdim=4).evaluate(z) - 1.5) <= RTOL * 1.5
    s3 = ina.complex_continuous_siteinds(ina.named_grid((3, 3)), map_dimension=3)
    zs = [0.5 + 0.125j, 0.25 + 0.875j, 0.0]
    assert abs(ina.const_itn(s3, c=1.5).evaluate(zs, [1, 2, 3]) - 1.5) <= RTOL * 1.5
    rng = np.random.default_rng(1234)
    a, k, c = rng.random(3) + 1j * rng.random(3)
    s2 = ina.complex_continuous_siteinds(ina.named_grid((3, 2)), map_dimension=2)
    f = (ina.tanh_itn(s2, k=k, a=a, c=c, nterms=50, dim=1)
         + ina.tanh_itn(s2, k=k, a=a, c=c, nterms=50, dim=2))
    z1, z2 = 0.5 + 0.125j, 0.625 + 0.25j
    exact = c * np.tanh(k * z1 + a) + c * np.tanh(k * z2 + a)
    assert abs(f.evaluate([z1, z2], [1, 2]) - exact) <= RTOL * abs(exact)


@pytest.mark.parametrize("dims,chi,nd,cplx", [((3, 3), 3, 1, False), ((3, 3), 2, 3, False),
                                              ((4, 3), 2, 2, True), ((2, 2, 2), 2, 3, False)])
def test_random_network_with_cycles_vs_oracle(ina, dims, chi, nd, cplx):
    """A network on a grid, uploaded from its tensors on the grid, against the
    oracle's contraction of the same network (cycles and all): evaluate at
    64 points and integrate, 1e-12."""
    graph = O.grid_graph(dims)
    rng = np.random.default_rng(len(dims) * 10 + chi)
    s_or = O.siteinds(graph, map_dimension=nd)
    net = O.random_net(s_or, chi, rng, normalize=True)
    if cplx:
        for v in net.T:
            net.T[v].arr = net.T[v].arr * np.exp(1j * rng.random(net.T[v].arr.shape))
    s = product_map(ina, graph, s_or)
    f = ina.ITensorNetworkFunction.from_tensors(s, oracle_to_graph_tensors(net, s))
    X = rng.random((64, nd))
    dims_ = list(range(1, nd + 1))
    got = f.evaluate_batch(X, dims_)
    ref = O.evaluate_batch(net, X, dims_)
    assert rel_err(got, ref) < 1e-12
    assert abs(f.integrate() - O.integrate(net)) <= 1e-12 * max(abs(O.integrate(net)), 1e-300)

"""The accurate mixed evaluation (precision "mixed": FP64 messages, bond-64/128
vertices as exact products of 8-bit integer slices on the tcgen05 tensor
cores) against the oracle and the plain FP64 path, per point."""
import numpy as np
import pytest

import oracle as O
from _helpers import upload_oracle

pytestmark = pytest.mark.gpu

TOL_POINT = 1e-9  # per-point relative error on trees of depth <= 4


def per_point(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)) / np.abs(np.asarray(b))


# a vertex whose first child is internal and whose second is a leaf (its
# output must not overwrite the first child's message while it is read)
LEAF_SECOND = (list(range(1, 7)), [(1, 2), (2, 3), (2, 4), (3, 5), (3, 6)])


@pytest.mark.parametrize("graph_name,chi,nd", [("binary7", 128, 3), ("binary15", 64, 3),
                                               ("binary15", 128, 3), ("binary31", 64, 2),
                                               ("leaf_second", 128, 2), ("leaf_second", 64, 2)])
def test_sliced_tensor_core_matches_oracle(ina, graph_name, chi, nd):
    graph = {"binary7": O.binary_tree_graph(7), "binary15": O.binary_tree_graph(15),
             "binary31": O.binary_tree_graph(31), "leaf_second": LEAF_SECOND}[graph_name]
    rng = np.random.default_rng(300 + chi)
    s_or = O.siteinds(graph, map_dimension=nd)
    net = O.random_net(s_or, chi, rng, normalize=True)
    f, _ = upload_oracle(ina, graph, net)
    X = rng.random((4000, nd))
    dims = list(range(1, nd + 1))
    ctx = f.ctx
    ctx.kernel_stats(reset=True)
    got = f.evaluate_batch(X, dims, precision="mixed")
    st = ctx.kernel_stats(reset=True)
    assert st.get("contract_oz", {}).get("launches", 0) > 0, st
    ref64 = f.evaluate_batch(X, dims, precision="f64")
    e64 = per_point(got, ref64)
    assert np.max(e64) < TOL_POINT, np.max(e64)
    assert np.median(e64) < 1e-13, np.median(e64)
    ref = O.evaluate_batch(net, X[:128], dims)
    eo = per_point(got[:128], ref)
    assert np.max(eo) < TOL_POINT, np.max(eo)


def test_sliced_tensor_core_fp32_network(ina):
    """An FP32 network (the benchmark's storage type): the slices represent
    the FP32 tensors exactly enough that the result matches the FP64
    evaluation of the same (FP32-valued) tensors."""
    graph = O.binary_tree_graph(15)
    rng = np.random.default_rng(17)
    s_or = O.siteinds(graph, map_dimension=3)
    net = O.random_net(s_or, 128, rng, normalize=True)
    for v in net.T:  # round the oracle's tensors to FP32 so both sides hold the same values
        net.T[v].arr = net.T[v].arr.astype(np.float32).astype(np.float64)
    f32, _ = upload_oracle(ina, graph, net, dtype=ina._lib.F32)
    X = rng.random((2000, 3))
    got = f32.evaluate_batch(X, [1, 2, 3], precision="mixed")
    ref = O.evaluate_batch(net, X[:96], [1, 2, 3])
    assert np.max(per_point(got[:96], ref)) < TOL_POINT


def test_benchmark_network_vs_oracle(ina):
    """The benchmark's network (60-vertex binary tree, 3 variables x 20 bits,
    chi = 128, Gaussian FP32 tensors of unit norm, seed 1): 160 points against
    the oracle and 32768 points against the FP64 GPU path, every point within
    1e-8 relative."""
    import bench

    s, ts = bench.config3_tensors(1)
    f = ina.ITensorNetworkFunction.from_tensors(s, ts, dtype=ina._lib.F32)
    X = bench.config3_points(32768, 1)
    got = f.evaluate_batch(X, [1, 2, 3], precision="mixed")
    f64 = ina.ITensorNetworkFunction.from_tensors(s, {v: t.astype(np.float64) for v, t in ts.items()})
    ref64 = f64.evaluate_batch(X, [1, 2, 3], precision="f64")
    e64 = per_point(got, ref64)
    assert np.max(e64) < 1e-8, np.max(e64)
    net = bench.oracle_net(s, ts)
    ref = O.evaluate_batch(net, X[:160], [1, 2, 3])
    assert np.max(per_point(got[:160], ref)) < 1e-8
    assert np.max(per_point(ref64[:160], ref)) < 1e-8


def test_wait_timeout_is_reported_and_recovers(ina):
    """A tensor-core wait that runs out: with the arrive that releases the MMA
    issuer withheld and a budget of 2000 polls, the call returns
    TNFA_ERR_TIMEOUT (every role stops, tensor memory is released); the next
    call on the same context with the normal budget is exact again."""
    graph = O.binary_tree_graph(7)
    rng = np.random.default_rng(9)
    s_or = O.siteinds(graph, map_dimension=3)
    net = O.random_net(s_or, 64, rng, normalize=True)
    f, _ = upload_oracle(ina, graph, net)
    X = rng.random((700, 3))
    ctx = f.ctx
    ref = f.evaluate_batch(X, [1, 2, 3], precision="f64")
    ctx.set_wait_budget(2000, drop_arrive=True)
    try:
        with pytest.raises(ina._lib.TnfaError) as ei:
            f.evaluate_batch(X, [1, 2, 3], precision="mixed")
        assert ei.value.status == ina._lib.ERR_TIMEOUT
    finally:
        ctx.set_wait_budget(1 << 26, drop_arrive=False)
    got = f.evaluate_batch(X, [1, 2, 3], precision="mixed")
    assert np.max(per_point(got, ref)) < TOL_POINT

"""Error paths, exercised without a GPU fault: an injected device-allocation
failure (TNFA_ERR_OUT_OF_MEMORY, the context stays usable), a Jacobi sweep
cap that a truncation cannot meet (TNFA_ERR_NOT_CONVERGED).  The tensor-core
wait timeout is tested in test_gpu_evaluate_mixed.py."""
import numpy as np
import pytest

import oracle as O
from _helpers import product_map, oracle_to_tensors

pytestmark = pytest.mark.gpu


def _net(ina, ctx, graph, chi, seed, nd=3):
    rng = np.random.default_rng(seed)
    s_or = O.siteinds(graph, map_dimension=nd)
    net = O.random_net(s_or, chi, rng, normalize=True)
    s = product_map(ina, graph, s_or)
    return ina.ITensorNetworkFunction.from_tensors(s, oracle_to_tensors(net, s), ctx=ctx)


def test_injected_allocation_failure(ina):
    L = ina._lib
    ctx = L.Context(0)
    f = _net(ina, ctx, O.binary_tree_graph(15), 16, 60)
    X = np.random.default_rng(61).random((3000, 3))
    ref = f.evaluate_batch(X)
    failed = 0
    for n in range(12):
        ctx.inject_faults(fail_alloc_after=n)
        try:
            got = f.evaluate_batch(X)
        except L.TnfaError as e:
            assert e.status == L.ERR_OUT_OF_MEMORY and "injected" in str(e)
            failed += 1
        else:
            assert np.array_equal(got, ref)
        finally:
            ctx.inject_faults(-1)
        assert np.array_equal(f.evaluate_batch(X), ref)  # the context stays usable
    assert failed >= 3
    # the same for a truncation (QR, SVD and GEMM workspaces)
    g = _net(ina, ctx, O.path_graph(10), 12, 62, nd=1)
    ok = ina.truncate(g, cutoff=1e-8)
    xs = np.random.default_rng(63).random(64)
    ctx.inject_faults(fail_alloc_after=2)
    with pytest.raises(L.TnfaError) as e:
        ina.truncate(g, cutoff=1e-8)
    ctx.inject_faults(-1)
    assert e.value.status == L.ERR_OUT_OF_MEMORY
    assert np.allclose(ina.truncate(g, cutoff=1e-8).evaluate_batch(xs), ok.evaluate_batch(xs),
                       rtol=0, atol=1e-12 * np.max(np.abs(ok.evaluate_batch(xs))))


def test_jacobi_sweep_cap_reports_not_converged(ina):
    L = ina._lib
    ctx = L.Context(0)
    g = _net(ina, ctx, O.path_graph(10), 24, 64, nd=1)
    ctx.inject_faults(jacobi_sweep_cap=1)
    try:
        with pytest.raises(L.TnfaError) as e:
            ina.truncate(g, cutoff=1e-12)
        assert e.value.status == L.ERR_NOT_CONVERGED
    finally:
        ctx.inject_faults()
    t = ina.truncate(g, cutoff=1e-12)
    xs = np.random.default_rng(65).random(64)
    a, b = t.evaluate_batch(xs), g.evaluate_batch(xs)
    assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b))

"""The launch autotuner (tnfa_ctx_set_autotune / tnfa_ctx_tuning_report):
the first large call for a shape times every interchangeable variant, keeps
the fastest, and leaves a result equal to the untuned one; later calls reuse
the kept variant."""
import numpy as np
import pytest

import oracle as O
from _helpers import oracle_to_tensors, product_map, rel_err

pytestmark = pytest.mark.gpu


def _net(ina, ctx, graph, chi, seed, dtype):
    s_or = O.siteinds(graph, map_dimension=3)
    net = O.random_net(s_or, chi, np.random.default_rng(seed), normalize=True)
    s = product_map(ina, graph, net.s)
    return ina.ITensorNetworkFunction.from_tensors(s, oracle_to_tensors(net, s), ctx=ctx, dtype=dtype)


@pytest.mark.parametrize("chi", [24, 48, 96])
def test_simt_tiles_tuned_and_exact(ina, chi):
    L = ina._lib
    ctx = L.Context(0)
    f = _net(ina, ctx, O.binary_tree_graph(15), chi, 100 + chi, L.F64)
    X = np.random.default_rng(101).random((20000, 3))
    ctx.set_autotune(False, forget=True)
    ref = f.evaluate_batch(X)
    ctx.set_autotune(True, min_work=0.0)
    first = f.evaluate_batch(X)  # times the candidates
    rep = ctx.tuning_report()
    keys = [k for k in rep if k.startswith("simt:contract_f64:")]
    assert keys, rep
    for k in keys:
        kept, ms = rep[k]
        assert len(ms) >= 2 and 0 <= kept < len(ms) and ms[kept] == min(ms)
    second = f.evaluate_batch(X)  # reuses the kept tiles
    assert ctx.tuning_report() == rep
    assert rel_err(first, ref) < 1e-12 and rel_err(second, ref) < 1e-12


def test_tensor_core_formulation_tuned(ina):
    L = ina._lib
    ctx = L.Context(0)
    f = _net(ina, ctx, O.binary_tree_graph(15), 64, 102, L.F64)
    X = np.random.default_rng(103).random((30000, 3))
    exact = f.evaluate_batch(X)
    ctx.set_autotune(True, min_work=0.0, forget=True)

    def mixed():
        m, e = f.evaluate_batch(X, precision="mixed_fast", out="f32_scaled")
        return np.ldexp(m, e)

    a = mixed()
    rep = ctx.tuning_report()
    assert any(k.startswith("tc:") for k in rep), rep
    b = mixed()
    for got in (a, b):  # split BF16 x3: norm-wise 3e-4 as in the tensor-core path test
        assert np.linalg.norm(got - exact) / np.linalg.norm(exact) < 3e-4


def test_autotune_off_and_threshold(ina):
    L = ina._lib
    ctx = L.Context(0)
    f = _net(ina, ctx, O.binary_tree_graph(7), 40, 104, L.F64)
    X = np.random.default_rng(105).random((5000, 3))
    ctx.set_autotune(False, forget=True)
    f.evaluate_batch(X)
    assert ctx.tuning_report() == {}
    ctx.set_autotune(True, min_work=1e30)  # nothing reaches the threshold
    f.evaluate_batch(X)
    assert ctx.tuning_report() == {}

"""Captured evaluation (tnfa_eval_plan_*): the no-allocation kernel sequence
for fixed device buffers, captured once as a CUDA graph and replayed.  Each
replay must equal tnfa_evaluate on the buffer's current contents; the error
flag of a replay is reported by the check call."""
import numpy as np
import pytest

import oracle as O
from _helpers import upload_oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", ["f64", "f32", "c128"])
def test_plan_replays_match_evaluate(ina, dtype):
    import torch

    L = ina._lib
    rng = np.random.default_rng(95)
    if dtype == "c128":
        s = ina.continuous_siteinds(ina.named_comb_tree((3, 4)), map_dimension=2)
        f = ina.rand_itn(s, link_space=6, rng=96).astype(L.C128)
        f.scale_vertex(s.layout.order[0], 0.5 + 0.25j)
        ndims = 2
    else:
        graph = O.binary_tree_graph(31)
        s_or = O.siteinds(graph, map_dimension=3)
        net = O.random_net(s_or, 16, rng, normalize=True)
        f, _ = upload_oracle(ina, graph, net, dtype=L.F64 if dtype == "f64" else L.F32)
        ndims = 3
    n = 2500
    X = torch.tensor(rng.random((n, ndims)), dtype=torch.float64, device="cuda")
    out = torch.empty(n, dtype=torch.complex128 if dtype == "c128" else torch.float64, device="cuda")
    plan = f.evaluation_plan(X, out, out_kind="f64")
    prec = {"f64": "f64", "f32": "f32", "c128": "f64"}[dtype]
    tol = 2e-5 if dtype == "f32" else 1e-12
    want = f.evaluate_batch(X.cpu().numpy(), precision=prec)
    assert np.max(np.abs(out.cpu().numpy() - want)) <= tol * np.max(np.abs(want))  # the eager run
    for k in range(3):  # new contents in the same buffer, replayed
        Xn = rng.random((n, ndims))
        X.copy_(torch.tensor(Xn))
        out.zero_()
        plan.launch()
        plan.check()
        want = f.evaluate_batch(Xn, precision=prec)
        assert np.max(np.abs(out.cpu().numpy() - want)) <= tol * np.max(np.abs(want)), k
    plan.close()


def test_plan_reports_bad_coordinates_and_recovers(ina):
    import torch

    s = ina.continuous_siteinds(ina.named_path_graph(12))
    f = ina.rand_itn(s, link_space=4, rng=97)
    X = torch.rand((300, 1), dtype=torch.float64, device="cuda")
    out = torch.empty(300, dtype=torch.float64, device="cuda")
    plan = f.evaluation_plan(X, out)
    X[7, 0] = -0.5
    plan.launch()
    with pytest.raises(ina.TnfaError) as e:
        plan.check()
    assert e.value.status == ina._lib.ERR_DOMAIN
    X[7, 0] = 0.25
    plan.launch()
    plan.check()
    want = f.evaluate_batch(X.cpu().numpy())
    assert np.max(np.abs(out.cpu().numpy() - want)) <= 1e-12 * np.max(np.abs(want))
    plan.close()


def test_plan_rejects_bad_arguments(ina):
    import torch

    L = ina._lib
    s = ina.continuous_siteinds(ina.named_path_graph(8))
    f = ina.rand_itn(s, link_space=3, rng=98)
    X = torch.rand((10, 1), dtype=torch.float64, device="cuda")
    out = torch.empty(10, dtype=torch.float64, device="cuda")
    with pytest.raises(ina.TnfaError) as e:  # precision must be the network's own
        f.evaluation_plan(X, out, precision="f32")
    assert e.value.status == L.ERR_UNSUPPORTED
    with pytest.raises(ValueError):
        f.evaluation_plan(X.cpu(), out)

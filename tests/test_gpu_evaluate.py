"""Batched evaluation and integration on the GPU (through the C ABI) against
the CPU oracle and the reference's analytic known answers."""
import numpy as np
import pytest

import oracle as O
from _helpers import product_map, rel_err, upload_oracle

pytestmark = pytest.mark.gpu

TOL_F64 = 1e-12  # plain FP64 path vs the FP64 oracle
TOL_F32 = 2e-5   # FP32 CUDA-core path


GRAPHS = {
    "path12": O.path_graph(12),
    "comb3x4": O.comb_tree_graph((3, 4)),
    "binary15": O.binary_tree_graph(15),
}


def _points(rng, n, ndim):
    return rng.random((n, ndim))


@pytest.mark.parametrize("gname", list(GRAPHS))
@pytest.mark.parametrize("chi", [1, 3, 16])
def test_random_network_f64(ina, gname, chi):
    graph = GRAPHS[gname]
    rng = np.random.default_rng(chi)
    s_or = O.siteinds(graph, map_dimension=2)
    net = O.random_net(s_or, chi, rng, normalize=True)
    f, _ = upload_oracle(ina, graph, net)
    X = _points(rng, 257, 2)
    got = f.evaluate_batch(X, [1, 2], precision="f64")
    ref = np.array([O.evaluate(net, list(x), [1, 2]) for x in X[:64]])
    assert rel_err(got[:64], ref) < TOL_F64
    # per-point calls agree with the batch
    for p in (0, 100, 256):
        assert abs(f.evaluate(list(X[p]), [1, 2]) - got[p]) <= 1e-14 * max(1.0, abs(got[p]))


@pytest.mark.parametrize("precision", ["f32", "mixed_fast", "mixed"])
def test_random_network_f32_paths(ina, precision):
    graph = O.binary_tree_graph(31)
    rng = np.random.default_rng(5)
    s_or = O.siteinds(graph, map_dimension=3)
    net = O.random_net(s_or, 8, rng, normalize=True)
    f, _ = upload_oracle(ina, graph, net)
    X = _points(rng, 1000, 3)
    ref = f.evaluate_batch(X, [1, 2, 3], precision="f64")
    m, e = f.evaluate_batch(X, [1, 2, 3], precision=precision, out="f32_scaled")
    got = np.ldexp(m, e)
    err = np.abs(got - ref) / np.abs(ref)
    assert np.median(err) < TOL_F32
    # the scaled output is finite and nonzero for every point
    assert np.all(np.isfinite(got)) and np.all(got != 0)


FUNCS = [
    ("cosh", "cosh_itn", O.cosh_itn, np.cosh),
    ("sinh", "sinh_itn", O.sinh_itn, np.sinh),
    ("exp", "exp_itn", O.exp_itn, np.exp),
    ("cos", "cos_itn", O.cos_itn, np.cos),
    ("sin", "sin_itn", O.sin_itn, np.sin),
]


@pytest.mark.parametrize("name,pname,onet,fn", FUNCS)
@pytest.mark.parametrize("base", [2, 3])
def test_constructors_match_oracle(ina, name, pname, onet, fn, base):
    """test/test_realitensorfunction.jl:65-104 on the GPU."""
    rng = np.random.default_rng(3)
    a, k, c = rng.random(3)
    graph = O.comb_tree_graph((2, 3))
    s_or = O.siteinds(graph, base=base)
    s = product_map(ina, graph, s_or)
    f = getattr(ina, pname)(s, k=k, a=a, c=c)
    x = 0.625 if base == 2 else 5.0 / 9.0
    val = f.evaluate(x)
    assert abs(val - c * fn(k * x + a)) <= np.sqrt(np.finfo(float).eps) * abs(c * fn(k * x + a))
    X = rng.random((50, 1))
    got = f.evaluate_batch(X)
    ref = np.array([O.evaluate(onet(s_or, k=k, a=a, c=c), [x0]) for x0 in X[:, 0]])
    assert rel_err(got, ref.real if not np.iscomplexobj(got) else ref) < TOL_F64


def test_tanh_and_poly(ina):
    """test/test_realitensorfunction.jl:106-144."""
    rng = np.random.default_rng(4)
    a, k, c = rng.random(3)
    s = ina.continuous_siteinds(ina.named_grid((10, 1)))
    f = ina.tanh_itn(s, k=k, a=a, c=c, nterms=50)
    assert abs(f.evaluate(0.625) - c * np.tanh(k * 0.625 + a)) < 1e-8
    for deg in range(1, 12):
        g = ina.uniform_tree(6, rng)
        s = ina.continuous_siteinds(g)
        k, c = rng.random(2)
        coeffs = rng.random(deg + 1)
        p = ina.poly_itn(s, list(coeffs), k=k, c=c)
        x = 0.875
        exact = c * sum(coeffs[i] * (k * x) ** i for i in range(deg + 1))
        assert abs(p.evaluate(x) - exact) <= 1e-4


def test_poly_matches_oracle_tensors_values(ina):
    graph = O.comb_tree_graph((3, 3))
    s_or = O.siteinds(graph, map_dimension=2)
    s = product_map(ina, graph, s_or)
    coeffs = [1.0, 0.5, 0.25]
    f = ina.poly_itn(s, coeffs, dim=1)
    onet = O.poly_itn(s_or, coeffs, dim=1)
    rng = np.random.default_rng(8)
    X = rng.random((40, 2))
    ref = np.array([O.evaluate(onet, list(x), [1, 2]) for x in X]).real
    assert rel_err(f.evaluate_batch(X, [1, 2]), ref) < TOL_F64


def test_const_and_sums(ina):
    """test/test_realitensorfunction.jl:147-189, on the reference's
    named_grid((3, 3)) (a graph with cycles)."""
    s = ina.continuous_siteinds(ina.named_grid((3, 3)), map_dimension=3)
    assert abs(ina.const_itn(s, c=1.5).evaluate([0.5, 0.25, 0.0], [1, 2, 3]) - 1.5) < 1e-14
    assert abs(ina.const_itn(s, c=-2.0, linkdim=4).evaluate([0.5, 0.25, 0.0], [1, 2, 3]) + 2.0) < 1e-13
    s = ina.continuous_siteinds(ina.named_grid((10, 1)), map_dimension=2)
    rng = np.random.default_rng(9)
    for _, pname, _, fn in FUNCS:
        a, k, c = rng.random(3)
        f = getattr(ina, pname)(s, k=k, a=a, c=c, dim=1) + getattr(ina, pname)(s, k=k, a=a, c=c, dim=2)
        x, y = 0.625, 0.25
        assert abs(f.evaluate([x, y], [1, 2]) - (c * fn(k * x + a) + c * fn(k * y + a))) < 1e-12


def test_delta_p(ina):
    """test/test_realitensorfunction.jl:210-259."""
    L = 10
    s = ina.continuous_siteinds(ina.named_grid((L, 1)), map_dimension=2)
    x0, y0 = 0.625, 0.25
    d = 2.0**-L
    xs = [0.0, d, 0.25, 0.5, 0.625, 0.875, 1 - d]
    psi = ina.delta_p(s, [x0, y0])
    assert abs(psi.evaluate([x0, y0], [1, 2]) - 1) < 1e-14
    assert abs(psi.evaluate([y0, x0], [1, 2])) < 1e-14
    plane = ina.delta_p(s, [y0], [2])
    X = np.array([[x, y0] for x in xs] + [[x, 0.5] for x in xs])
    v = plane.evaluate_batch(X, [1, 2])
    assert np.allclose(v[: len(xs)], 1.0) and np.allclose(v[len(xs):], 0.0)
    both = ina.delta_p(s, [[x0, y0], [0.5]], [[1, 2], [2]])
    assert abs(both.evaluate([x0, y0], [1, 2]) - 1) < 1e-14
    for x in xs:
        assert abs(both.evaluate([x, 0.5], [1, 2]) - 1) < 1e-14
    assert abs(both.evaluate([0.0, 0.0], [1, 2])) < 1e-14


def test_complex_map_functions(ina):
    """test/test_complexitensorfunction.jl:57-80 (complex k, a, c and map)."""
    rng = np.random.default_rng(10)
    graph = O.comb_tree_graph((2, 3))
    rdv, idv = [[(1, 1), (1, 2), (1, 3)]], [[(2, 1), (2, 2), (2, 3)]]
    s_or = O.complex_siteinds(graph, rdv, idv)
    s = product_map(ina, graph, s_or)
    for _, pname, onet, fn in FUNCS:
        a, k, c = rng.random(3) + 1j * rng.random(3)
        f = getattr(ina, pname)(s, k=k, a=a, c=c)
        z = 0.625 + 0.25j
        assert abs(f.evaluate(z) - c * fn(k * z + a)) <= 1e-7 * abs(c * fn(k * z + a))
        Z = rng.random(20) + 1j * rng.random(20)
        got = f.evaluate_batch(Z.reshape(-1, 1))
        ref = np.array([O.evaluate(onet(s_or, k=k, a=a, c=c), [z0]) for z0 in Z])
        assert rel_err(got, ref) < TOL_F64


def test_integrate(ina):
    """test/test_integration.jl:15-38 plus oracle parity."""
    s = ina.continuous_siteinds(ina.named_comb_tree((2, 10)))
    f = ina.exp_itn(s, dim=1)
    assert abs(ina.integrate(f * f) - 0.5 * (np.e**2 - 1)) <= 1e-4
    s = ina.continuous_siteinds(ina.named_comb_tree((3, 10)), map_dimension=2)
    g = ina.exp_itn(s, dim=1) * ina.exp_itn(s, dim=2)
    assert abs(ina.integrate(g) - (np.e - 1) ** 2) <= 1e-4
    graph = O.binary_tree_graph(20)
    rng = np.random.default_rng(12)
    s_or = O.siteinds(graph, map_dimension=2)
    net = O.random_net(s_or, 6, rng)
    fp, _ = upload_oracle(ina, graph, net)
    assert abs(fp.integrate() - O.integrate(net)) <= TOL_F64 * abs(O.integrate(net))
    assert abs(fp.integrate(take_sum=True) - O.integrate(net, take_sum=True)) <= TOL_F64 * abs(
        O.integrate(net, take_sum=True))


def test_sum_and_product_algebra(ina):
    graph = O.comb_tree_graph((3, 3))
    rng = np.random.default_rng(13)
    s_or = O.siteinds(graph, map_dimension=2)
    n1 = O.random_net(s_or, 3, rng)
    n2 = O.random_net(s_or, 2, rng)
    f1, _ = upload_oracle(ina, graph, n1)
    f2, _ = upload_oracle(ina, graph, n2)
    X = rng.random((30, 2))
    r1 = np.array([O.evaluate(n1, list(x), [1, 2]) for x in X])
    r2 = np.array([O.evaluate(n2, list(x), [1, 2]) for x in X])
    assert rel_err((f1 + f2).evaluate_batch(X, [1, 2]), r1 + r2) < TOL_F64
    assert rel_err((f1 * f2).evaluate_batch(X, [1, 2]), r1 * r2) < TOL_F64
    assert rel_err((2.5 * f1).evaluate_batch(X, [1, 2]), 2.5 * r1) < TOL_F64
    assert (f1 + f2).maxlinkdim() == 5 and (f1 * f2).maxlinkdim() == 6


def test_edge_cases(ina):
    s = ina.continuous_siteinds(ina.named_grid((8, 1)))
    f = ina.exp_itn(s)
    d = 2.0**-8
    # x >= 1 saturates to the last grid point, as the reference's greedy loop does
    assert abs(f.evaluate(1.0) - np.exp(1 - d)) < 1e-12
    assert abs(f.evaluate(7.5) - np.exp(1 - d)) < 1e-12
    with pytest.raises(ina.TnfaError) as e:
        f.evaluate(-0.25)
    assert e.value.status == ina._lib.ERR_DOMAIN
    with pytest.raises(ina.TnfaError):
        f.evaluate(float("nan"))
    assert f.evaluate_batch(np.zeros((0, 1))).shape == (0,)
    # a single-vertex network
    s1 = ina.continuous_siteinds(ina.named_grid((1, 1)))
    g = ina.exp_itn(s1, k=2.0)
    assert abs(g.evaluate(0.5) - np.exp(1.0)) < 1e-14
    # a forest: product of functions on disjoint vertex sets
    s2 = ina.continuous_siteinds(ina.named_comb_tree((2, 4)), [[(1, j) for j in range(1, 5)],
                                                             [(2, j) for j in range(1, 5)]])
    sa, sb = ina.reduced_indsnetworkmap(s2, 1), ina.reduced_indsnetworkmap(s2, 2)
    h = ina.exp_itn(sa, dim=1) * ina.cos_itn(sb, dim=2)
    x, y = 0.5, 0.25
    assert abs(h.evaluate([x, y], [1, 2]) - np.exp(x) * np.cos(y)) < 1e-12


def test_deep_tree_underflow_is_scaled(ina):
    """60-vertex binary tree with unit-norm tensors: |f| ~ 1e-40..1e-60, far
    below FP32's range; the FP32 path carries a base-2 exponent per point."""
    graph = O.binary_tree_graph(60)
    rng = np.random.default_rng(14)
    s_or = O.siteinds(graph, map_dimension=3)
    net = O.random_net(s_or, 16, rng, normalize=True)
    f, _ = upload_oracle(ina, graph, net)
    X = rng.random((256, 3))
    ref = np.array([O.evaluate(net, list(x), [1, 2, 3]) for x in X[:16]])
    got = f.evaluate_batch(X, [1, 2, 3], precision="f64")
    assert rel_err(got[:16], ref) < 1e-11
    m, e = f.evaluate_batch(X, [1, 2, 3], precision="f32", out="f32_scaled")
    assert np.median(np.abs(np.ldexp(m, e) - got) / np.abs(got)) < TOL_F32


@pytest.mark.parametrize("graph_name,chi", [("binary7", 128), ("binary15", 64), ("path6", 128)])
def test_tensor_core_path(ina, graph_name, chi):
    """The tcgen05 split-BF16 contraction (precision "mixed_fast", chi in
    {64, 128}; the binary trees' roots use the bilinear mode) against the FP64
    path on the same tensors.
    Split BF16 x3 leaves ~2^-17 per product; random trees amplify it by their
    depth, so the norm-wise bound is 3e-4."""
    graph = {"binary7": O.binary_tree_graph(7), "binary15": O.binary_tree_graph(15),
             "path6": O.path_graph(6)}[graph_name]
    rng = np.random.default_rng(chi)
    s_or = O.siteinds(graph, map_dimension=3 if graph_name != "path6" else 1)
    net = O.random_net(s_or, chi, rng, normalize=True)
    f, _ = upload_oracle(ina, graph, net)
    nd = len(s_or.dims())
    X = rng.random((3000, nd))
    dims = list(range(1, nd + 1))
    ctx = f.ctx
    ctx.kernel_stats(reset=True)
    m, e = f.evaluate_batch(X, dims, precision="mixed_fast", out="f32_scaled")
    st = ctx.kernel_stats(reset=True)
    assert st.get("contract_tc", {}).get("launches", 0) > 0, st
    got = np.ldexp(m, e)
    ref = f.evaluate_batch(X, dims, precision="f64")
    nrm = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert nrm < 3e-4, nrm
    assert np.median(np.abs(got - ref) / np.abs(ref)) < 3e-4
    if graph_name != "path6":
        assert st.get("contract_f32", {}).get("launches", 0) == 0, st


@pytest.mark.parametrize("chi", [3, 5, 12])
def test_batch_composition_invariance(ina, chi):
    """A point's value must not depend on which other points share its batch
    (tiles of the narrow and SIMT contractions mix points of one site value):
    the full 2^12 grid in one call equals the same points in calls of 1, 7 and
    333 points."""
    s = ina.continuous_siteinds(ina.named_path_graph(12))
    f = ina.rand_itn(s, link_space=chi, rng=110 + chi)
    xs = np.arange(2**12) / 2**12
    whole = f.evaluate_batch(xs)
    scale = np.max(np.abs(whole))
    for step in (1, 7, 333):
        idx = np.arange(0, len(xs), 97 if step == 1 else 1)
        parts = np.concatenate([f.evaluate_batch(xs[idx[i:i + step]]) for i in range(0, len(idx), step)])
        assert np.max(np.abs(parts - whole[idx])) <= 1e-13 * scale, step


@pytest.mark.parametrize("graph_name,chi", [("path20", 16), ("path20", 32), ("binary31", 8),
                                            ("binary15", 16), ("comb3x5", 5), ("binary7", 2)])
@pytest.mark.parametrize("dtype", ["f64", "f32", "c128"])
def test_fused_small_bond_path_matches_per_vertex(ina, monkeypatch, graph_name, chi, dtype):
    """The one-launch small-bond evaluation (k_eval_fused) against the
    per-vertex kernels on the same network and points."""
    L = ina._lib
    graph = {"path20": O.path_graph(20), "binary31": O.binary_tree_graph(31),
             "binary15": O.binary_tree_graph(15), "comb3x5": O.comb_tree_graph((3, 5)),
             "binary7": O.binary_tree_graph(7)}[graph_name]
    nd = 1 if graph_name == "path20" else 3
    rng = np.random.default_rng(120 + chi)
    s_or = O.siteinds(graph, map_dimension=nd)
    net = O.random_net(s_or, chi, rng, normalize=True)
    f, _ = upload_oracle(ina, graph, net, dtype=L.F32 if dtype == "f32" else L.F64)
    if dtype == "c128":
        f = f.astype(L.C128)
        f.scale_vertex(f.s.layout.order[0], 0.6 - 0.8j)
    X = rng.random((40000 if chi > 8 else 5000, nd))  # above chi 8 the fused path wants >= 32768 points
    dims = list(range(1, nd + 1))
    prec = "f32" if dtype == "f32" else "f64"
    ctx = f.ctx
    ctx.kernel_stats(reset=True)
    fused = f.evaluate_batch(X, dims, precision=prec)
    st = ctx.kernel_stats(reset=True)
    assert st.get("eval_fused", {}).get("launches", 0) >= 1, st
    monkeypatch.setenv("TNFA_EVAL_FUSED", "0")
    plain = f.evaluate_batch(X, dims, precision=prec)
    st = ctx.kernel_stats(reset=True)
    assert st.get("eval_fused", {}).get("launches", 0) == 0, st
    tol = 2e-5 if dtype == "f32" else 1e-12
    assert rel_err(fused, plain) < tol
    if dtype == "f64":  # and the oracle on a few points
        ref = np.array([O.evaluate(net, list(x), dims) for x in X[:20]])
        assert rel_err(fused[:20], ref) < 1e-12


@pytest.mark.parametrize("graph_name,chi", [("one_child_pair", 128), ("binary15", 128), ("binary15", 64)])
def test_output_never_overwrites_inputs(ina, graph_name, chi):
    """A vertex's output message never shares memory with its children's
    messages.  Two ways it used to go wrong: the autotuner runs one
    contraction several times over the same inputs (the first run had
    overwritten them), and a SIMT tile split over output columns lets one CTA
    overwrite the rows another CTA of the same points has not read yet (more
    CTAs than fit at once).  Autotuning is forced here (threshold 0) and the
    batch spans several waves; the first call must match the oracle and a
    repeat."""
    L = ina._lib
    graph = {"one_child_pair": (list(range(1, 7)), [(1, 2), (2, 3), (2, 4), (3, 5), (4, 6)]),
             "binary15": O.binary_tree_graph(15)}[graph_name]
    rng = np.random.default_rng(77 + chi)
    nd = 2
    s_or = O.siteinds(graph, map_dimension=nd)
    net = O.random_net(s_or, chi, rng, normalize=True)
    ctx = L.Context(0)
    ctx.set_autotune(True, min_work=0.0, forget=True)
    s = product_map(ina, graph, net.s)
    from _helpers import oracle_to_tensors
    f = ina.ITensorNetworkFunction.from_tensors(s, oracle_to_tensors(net, s), ctx=ctx)
    X = rng.random((40000, nd))
    first = f.evaluate_batch(X, [1, 2], precision="f64")
    again = f.evaluate_batch(X, [1, 2], precision="f64")
    assert rel_err(first, again) < 1e-13
    idx = np.linspace(0, len(X) - 1, 96).astype(int)
    ref = O.evaluate_batch(net, X[idx], [1, 2])
    assert rel_err(first[idx], ref) < TOL_F64
    assert np.max(np.abs(first[idx] - ref) / np.abs(ref)) < 1e-9

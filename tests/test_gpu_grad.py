"""Gradient (VJP) of batched evaluation on the GPU: against the oracle's
environment gradient, central finite differences, FP32 vs FP64, and a short
fit through the autograd wrapper (the config-4 workflow at reduced size)."""
import numpy as np
import pytest

import oracle as O
from _helpers import oracle_to_tensors, upload_oracle

pytestmark = pytest.mark.gpu


def _grad_to_layout(net, grads, s_prod):
    tmp = O.Net(net.s, {v: O.Tensor(grads[v], net.T[v].inds) for v in net.s.verts}, net.link)
    return oracle_to_tensors(tmp, s_prod)


@pytest.mark.parametrize("gname", ["binary7", "comb3x3"])
def test_vjp_matches_oracle_gradient(ina, gname):
    graph = {"binary7": O.binary_tree_graph(7), "comb3x3": O.comb_tree_graph((3, 3))}[gname]
    rng = np.random.default_rng(50)
    s_or = O.siteinds(graph, map_dimension=2)
    net = O.random_net(s_or, 3, rng)
    f, s = upload_oracle(ina, graph, net)
    X = rng.random((40, 2))
    dout = rng.standard_normal(40)
    got = ina.evaluate_vjp(f, X, dout, [1, 2])
    ref = _grad_to_layout(net, O.gradient(net, X, [1, 2], dout), s)
    scale = max(np.max(np.abs(r)) for r in ref.values())
    for v in s.layout.order:
        assert np.max(np.abs(got[v] - ref[v])) <= 1e-11 * scale, v


def test_vjp_central_differences(ina):
    """f is linear in every tensor entry, so central differences are exact up
    to rounding: h = 1e-3 as in the config-4 description."""
    graph = O.path_graph(8)
    rng = np.random.default_rng(51)
    s_or = O.siteinds(graph, map_dimension=2)
    net = O.random_net(s_or, 4, rng)
    f, s = upload_oracle(ina, graph, net)
    X = rng.random((64, 2))
    dout = rng.standard_normal(64)
    g = ina.evaluate_vjp(f, X, dout, [1, 2])
    ts = f.tensors()
    h = 1e-3
    for _ in range(12):
        v = s.layout.order[rng.integers(len(s.layout.order))]
        idx = tuple(rng.integers(d) for d in ts[v].shape)
        tp = {k: a.copy() for k, a in ts.items()}
        tm = {k: a.copy() for k, a in ts.items()}
        tp[v][idx] += h
        tm[v][idx] -= h
        fp = ina.ITensorNetworkFunction.from_tensors(s, tp).evaluate_batch(X, [1, 2])
        fm = ina.ITensorNetworkFunction.from_tensors(s, tm).evaluate_batch(X, [1, 2])
        fd = np.dot(dout, fp - fm) / (2 * h)
        assert abs(fd - g[v][idx]) <= 1e-9 * max(1.0, abs(fd)), (v, idx, fd, g[v][idx])


def test_vjp_fp32_vs_fp64_config4_shape(ina):
    """Comb 2 x 12 (a 24-site path), chi 8, N(0, 0.1^2) tensors: FP32 gradient
    agrees with FP64."""
    L = 12
    g = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g, [[(1, j) for j in range(L, 0, -1)], [(2, j) for j in range(1, L + 1)]])
    f64 = ina.rand_itn(s, link_space=8, rng=52)
    ts = {v: 0.1 * a for v, a in f64.tensors().items()}
    f64 = ina.ITensorNetworkFunction.from_tensors(s, ts)
    f32 = ina.ITensorNetworkFunction.from_tensors(s, ts, dtype=ina._lib.F32)
    rng = np.random.default_rng(53)
    X = rng.random((4096, 2))
    dout = rng.standard_normal(4096)
    a = ina.evaluate_vjp(f64, X, dout, [1, 2])
    b = ina.evaluate_vjp(f32, X, dout, [1, 2])
    num = np.sqrt(sum(np.sum((a[v] - b[v].astype(np.float64)) ** 2) for v in a))
    den = np.sqrt(sum(np.sum(a[v] ** 2) for v in a))
    assert num / den < 1e-4


def test_fit_decreases_loss(ina):
    """Gradient descent on sin(3x) cos(5y) exp(-(x^2 + y^2)) through the
    autograd wrapper (config 4 at reduced size)."""
    torch = pytest.importorskip("torch")
    L = 8
    g = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g, [[(1, j) for j in range(L, 0, -1)], [(2, j) for j in range(1, L + 1)]])
    chi = 4
    f = ina.rand_itn(s, link_space=chi, rng=54)
    # variance-preserving start (std 1/sqrt(2 chi)): outputs O(1), gradients alive
    ts = {v: a / np.sqrt(2 * chi) for v, a in f.tensors().items()}
    flat = np.concatenate([ts[v].ravel() for v in s.layout.order])
    template = ina.ITensorNetworkFunction.from_tensors(s, ts)
    params = torch.tensor(flat, dtype=torch.float64, device="cuda", requires_grad=True)
    rng = np.random.default_rng(55)
    Xh = rng.random((1 << 12, 2))
    x, y = Xh[:, 0], Xh[:, 1]
    target = torch.tensor(np.sin(3 * x) * np.cos(5 * y) * np.exp(-(x**2 + y**2)), device="cuda")
    X = torch.tensor(Xh, device="cuda")
    opt = torch.optim.Adam([params], lr=0.02)
    losses = []
    for _ in range(60):
        opt.zero_grad()
        pred = ina.TTNEvaluate.apply(params, X, template, [1, 2])
        loss = torch.mean((pred - target) ** 2)
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    assert losses[-1] < 0.6 * losses[0], losses[::10]
    assert all(np.isfinite(losses))


def test_config4_shape_fd_and_oracle(ina):
    """Config 4 at its stated shape: comb 2 x 12 (a 24-site path), chi 32,
    FP32 tensors N(0, 0.1^2) (seed 2), MSE loss against
    sin(3x) cos(5y) exp(-(x^2 + y^2)) at 2^20 points.  The FP32 backward
    kernels' gradient against central differences (h = 1e-3; the loss is
    quadratic in each entry, so central differences of an FP64 evaluation of
    the same FP32 tensors are exact up to rounding) on sampled entries, and
    against the oracle's gradient on a 48-point subset."""
    L, chi = 12, 32
    g = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g, [[(1, j) for j in range(1, L + 1)], [(2, j) for j in range(1, L + 1)]])
    rng = np.random.default_rng(2)
    lay = s.layout
    ts = {}
    for i, v in enumerate(lay.order):
        shape = (2, chi if lay.parent[i] >= 0 else 1) + (chi,) * len(lay.children[i])
        ts[v] = (0.1 * rng.standard_normal(shape)).astype(np.float32)
    f32 = ina.ITensorNetworkFunction.from_tensors(s, ts, dtype=ina._lib.F32)
    P = 1 << 20
    X = rng.random((P, 2))
    x, y = X[:, 0], X[:, 1]
    target = np.sin(3 * x) * np.cos(5 * y) * np.exp(-(x**2 + y**2))
    pred = f32.evaluate_batch(X, [1, 2], precision="f32", out="f64")
    dout = 2.0 * (pred - target) / P  # d MSE / d pred
    grad = ina.evaluate_vjp(f32, X, dout, [1, 2])
    t64 = {v: a.astype(np.float64) for v, a in ts.items()}

    def loss(tens):
        fx = ina.ITensorNetworkFunction.from_tensors(s, tens).evaluate_batch(X, [1, 2])
        return np.mean((fx - target) ** 2)

    h = 1e-3
    gscale = max(np.max(np.abs(a)) for a in grad.values())
    for _ in range(6):
        v = lay.order[rng.integers(len(lay.order))]
        idx = tuple(rng.integers(d) for d in ts[v].shape)
        tp = dict(t64)
        tm = dict(t64)
        tp[v] = t64[v].copy()
        tm[v] = t64[v].copy()
        tp[v][idx] += h
        tm[v][idx] -= h
        fd = (loss(tp) - loss(tm)) / (2 * h)
        assert abs(fd - float(grad[v][idx])) <= 1e-3 * gscale + 1e-3 * abs(fd), (v, idx, fd, grad[v][idx])
    # the oracle's gradient of sum_p dout_p f(x_p) on a subset of points
    sub = rng.choice(P, 48, replace=False)
    gsub = ina.evaluate_vjp(f32.astype(ina._lib.F64), X[sub], dout[sub], [1, 2])
    so = O.siteinds(O.comb_tree_graph((2, L)), [[(1, j) for j in range(1, L + 1)],
                                                 [(2, j) for j in range(1, L + 1)]])
    from _helpers import product_map  # noqa: F401
    net = O.Net(so, {}, {frozenset(e): O.Index(chi, "L") for e in so.edges})
    for i, v in enumerate(lay.order):
        nb = lay.neighbours_in_layout_order(i)
        arr = t64[v] if lay.parent[i] >= 0 else t64[v][:, 0]
        inds = so.site[v] + [net.link[frozenset((v, lay.order[j]))] for j in nb]
        net.T[v] = O.Tensor(arr, inds)
    ref = _grad_to_layout(net, O.gradient(net, X[sub], [1, 2], dout[sub]), s)
    sc = max(np.max(np.abs(r)) for r in ref.values())
    for v in lay.order:
        assert np.max(np.abs(gsub[v] - ref[v])) <= 1e-10 * sc, v


@pytest.mark.parametrize("cplx", [False, True])
def test_operate_vjp(ina, cplx):
    """The adjoint of the exact operator contraction: for
    l(f) = sum_p w_p (O f)(x_p), df = operate_vjp(O, f, evaluate_vjp(O f, ...)).
    l is multilinear in the V site tensors (degree one in each entry), so
    <df, f> = V l(f) (Euler), central differences are exact on single entries,
    and a small step along a random direction matches <df, d>."""
    L = 8
    s = ina.continuous_siteinds(ina.named_grid((L, 1)))
    f = ina.rand_itn(s, link_space=3, rng=70)
    if cplx:
        f = f.astype(ina._lib.C128)
        f.scale_vertex(s.layout.order[2], 0.3 + 0.7j)
    op = ina.second_derivative_operator(s)
    if cplx:
        op = op.astype(ina._lib.C128)
    rng = np.random.default_rng(71)
    X = rng.random(200)
    w = rng.standard_normal(200)
    y = ina.operate_exact(op, f)
    dyv = ina.evaluate_vjp(y, X, w, [1])
    dy = np.concatenate([dyv[v].ravel() for v in s.layout.order])
    df = ina.operate_vjp(op, f, dy)
    ts = f.tensors()
    flat = np.concatenate([ts[v].ravel() for v in s.layout.order])

    def unflat(a):
        out, off = {}, 0
        for v in s.layout.order:
            n = ts[v].size
            out[v] = a[off:off + n].reshape(ts[v].shape)
            off += n
        return out

    def loss(a):
        g = ina.ITensorNetworkFunction.from_tensors(s, unflat(a))
        return np.dot(w, ina.operate_exact(op, g).evaluate_batch(X, [1]))

    l0 = loss(flat)
    assert abs(L * l0 - np.dot(df, flat)) <= 1e-10 * max(1.0, abs(L * l0))
    d = rng.standard_normal(flat.shape) * (1 + (1j if cplx else 0))
    eps = 1e-5
    dd = (loss(flat + eps * d) - loss(flat - eps * d)) / (2 * eps)
    assert abs(dd - np.dot(df, d)) <= 1e-6 * max(1.0, abs(np.dot(df, d)))
    h = 1e-3
    for k in rng.choice(len(flat), 5, replace=False):
        e = np.zeros_like(flat)
        e[k] = h
        fd = (loss(flat + e) - loss(flat - e)) / (2 * h)
        assert abs(fd - df[k]) <= 1e-8 * max(1.0, abs(fd))

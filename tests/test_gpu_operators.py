"""Operators, operator application, truncation and inner products on the GPU,
against the reference's operator tests (test/test_operators.jl,
test/test_integration.jl) and the oracle's dense-grid operator."""
import numpy as np
import pytest

import oracle as O
from _helpers import product_map, rel_err, upload_oracle

pytestmark = pytest.mark.gpu


def _grid(L):
    return np.arange(2**L) / 2.0**L


@pytest.mark.parametrize("n", [0, 1])
@pytest.mark.parametrize("boundary", ["Dirichlet", "Periodic", "Neumann"])
def test_shift_operators_tree(ina, boundary, n):
    """test/test_operators.jl:168-287: exact shift identities at 1e-8."""
    s = ina.continuous_siteinds(ina.named_comb_tree((2, 3)))
    L = 6
    N = 2**L
    f = ina.poly_itn(s, [1.0, 0.5, 0.25])
    xs = _grid(L)
    F = f.evaluate_batch(xs)
    step = n + 1
    fwd = ina.operate(ina.forward_shift_op(s, boundary=boundary, n=n,
                                           truncate_kwargs={"cutoff": 1e-10}), f, cutoff=1e-12)
    bwd = ina.operate(ina.backward_shift_op(s, boundary=boundary, n=n,
                                            truncate_kwargs={"cutoff": 1e-10}), f, cutoff=1e-12)
    Fw, Bw = fwd.evaluate_batch(xs), bwd.evaluate_batch(xs)
    for i in range(N):
        if i + step < N:
            exp_f = F[i + step]
        elif boundary == "Dirichlet":
            exp_f = 0.0
        elif boundary == "Periodic":
            exp_f = F[i + step - N]
        else:
            exp_f = F[i]
        assert abs(Fw[i] - exp_f) < 1e-8, (i, Fw[i], exp_f)
        if i - step >= 0:
            exp_b = F[i - step]
        elif boundary == "Dirichlet":
            exp_b = 0.0
        elif boundary == "Periodic":
            exp_b = F[i - step + N]
        else:
            exp_b = F[i]
        assert abs(Bw[i] - exp_b) < 1e-8, (i, Bw[i], exp_b)


def test_shift_operators_2d(ina):
    """test/test_operators.jl:289-351 (shift in dim 2 of a 2D function)."""
    s = ina.continuous_siteinds(ina.named_comb_tree((3, 3)), map_dimension=2)
    Ly = s.ndigits(2)
    d = 2.0**-Ly
    f = ina.poly_itn(s, [1.0, 0.5, 0.25], dim=1) + ina.cos_itn(s, dim=2)
    ys = _grid(Ly)
    X = np.stack([np.full_like(ys, 0.5), ys], axis=1)
    F = f.evaluate_batch(X, [1, 2])
    for boundary in ["Dirichlet", "Periodic", "Neumann"]:
        op = ina.forward_shift_op(s, boundary=boundary, dim=2, truncate_kwargs={"cutoff": 1e-10})
        G = ina.operate(op, f, cutoff=1e-12).evaluate_batch(X, [1, 2])
        for i in range(len(ys) - 1):
            assert abs(G[i] - F[i + 1]) < 1e-8
        last = {"Dirichlet": 0.0, "Periodic": F[0], "Neumann": F[-1]}[boundary]
        assert abs(G[-1] - last) < 1e-8


def test_derivatives_periodic_mps(ina):
    """test/test_operators.jl:16-46: d1..d4 of sin(2 pi x), rtol 1e-3 (after +1)."""
    L = 9
    s = ina.continuous_siteinds(ina.named_grid((L, 1)))
    d = 2.0**-L
    f = ina.sin_itn(s, k=2.0 * np.pi)
    ops = {
        1: ina.first_derivative_operator(s, cutoff=1e-12, left_boundary="Periodic",
                                         right_boundary="Periodic"),
        2: ina.second_derivative_operator(s, cutoff=1e-12, left_boundary="Periodic",
                                          right_boundary="Periodic"),
        3: ina.third_derivative_operator(s, cutoff=1e-12, left_boundary="Periodic",
                                         right_boundary="Periodic"),
        4: ina.fourth_derivative_operator(s, cutoff=1e-12, left_boundary="Periodic",
                                          right_boundary="Periodic"),
    }
    exact = {
        1: lambda x: 2 * np.pi * np.cos(2 * np.pi * x),
        2: lambda x: -(2 * np.pi) ** 2 * np.sin(2 * np.pi * x),
        3: lambda x: -(2 * np.pi) ** 3 * np.cos(2 * np.pi * x),
        4: lambda x: (2 * np.pi) ** 4 * np.sin(2 * np.pi * x),
    }
    xs = np.array([0.0, 0.25, 0.625, 0.875, 1.0 - d])
    for p, op in ops.items():
        g = ina.operate(op, f, cutoff=1e-8)
        v = g.evaluate_batch(xs)
        for x, val in zip(xs, v):
            e = exact[p](x)
            assert abs((1 + val) - (1 + e)) <= 1e-3 * max(abs(1 + val), abs(1 + e)), (p, x, val, e)


def test_derivative_on_tree(ina):
    """test/test_operators.jl:48-64: first derivative of sin(pi x) on a comb."""
    s = ina.continuous_siteinds(ina.named_comb_tree((4, 3)))
    L = 12
    d = 2.0**-L
    f = ina.sin_itn(s, k=np.pi)
    g = ina.operate(ina.first_derivative_operator(s, cutoff=1e-10), f, cutoff=1e-12)
    xs = np.array([d, 0.125, 0.25, 0.625, 0.875])
    v = g.evaluate_batch(xs)
    assert np.max(np.abs(v - np.pi * np.cos(np.pi * xs))) < 1e-3


def test_derivative_3d_function(ina):
    """test/test_operators.jl:66-97: d/dy of (x^2 - x) sin(pi y) sin(pi z) on a 45-site path."""
    L = 45
    s = ina.continuous_siteinds(ina.named_grid((L, 1)), map_dimension=3)
    f = ina.poly_itn(s, [0.0, -1.0, 1.0], dim=1) * ina.sin_itn(s, k=np.pi, dim=2) * ina.sin_itn(
        s, k=np.pi, dim=3)
    op = ina.first_derivative_operator(s, dim=2, cutoff=1e-10)
    g = ina.operate([op], f, cutoff=1e-10)
    pts = np.array([[x, y, z] for x in [0.125, 0.25, 0.675] for y in [0.125, 0.25, 0.675]
                    for z in [0.125, 0.25, 0.675]])
    fv = f.evaluate_batch(pts, [1, 2, 3])
    gv = g.evaluate_batch(pts, [1, 2, 3])
    x, y, z = pts.T
    assert np.max(np.abs(fv - (x**2 - x) * np.sin(np.pi * y) * np.sin(np.pi * z))) < 1e-3
    assert np.max(np.abs(gv - np.pi * (x**2 - x) * np.cos(np.pi * y) * np.sin(np.pi * z))) < 1e-3


def test_multiplication_and_operator_proj(ina):
    """test/test_operators.jl:99-166."""
    s = ina.continuous_siteinds(ina.named_comb_tree((4, 3)))
    g = ina.sin_itn(s, k=0.5 * np.pi)
    f = ina.cos_itn(s, k=0.25 * np.pi)
    xs = np.array([0.025, 0.1, 0.25, 0.625, 0.875])
    exact_fg = np.sin(0.5 * np.pi * xs) * np.cos(0.25 * np.pi * xs)
    exact_ff = np.cos(0.25 * np.pi * xs) ** 2
    assert np.max(np.abs((g * f).evaluate_batch(xs) - exact_fg)) < 1e-3
    assert np.max(np.abs((f * f).evaluate_batch(xs) - exact_ff)) < 1e-3
    P = ina.operator_proj(f)
    assert np.max(np.abs(ina.operate(P, g, cutoff=1e-14).evaluate_batch(xs) - exact_fg)) < 1e-3
    assert np.max(np.abs(ina.operate(P, f, cutoff=1e-14).evaluate_batch(xs) - exact_ff)) < 1e-3


def test_map_to_zeros(ina):
    """test/test_operators.jl:353-414 (boundary operator, 1D and 2D)."""
    s = ina.continuous_siteinds(ina.named_comb_tree((2, 3)))
    L = 6
    last = 1 - 2.0**-L
    f = ina.poly_itn(s, [1.0, 0.5, 0.25])
    phi = ina.map_to_zeros(f, [0.0, last], cutoff=1e-16, maxdim=10)
    xs = np.array([0.0, 2.0**-L, 0.25, 0.5, 0.625, 0.875, last])
    v = phi.evaluate_batch(xs)
    assert abs(v[0]) < 1e-8 and abs(v[-1]) < 1e-8
    assert np.all(np.abs(v[1:-1]) > 1e-3)
    s2 = ina.continuous_siteinds(ina.named_comb_tree((3, 3)), map_dimension=2)
    Ly = s2.ndigits(2)
    last2 = 1 - 2.0**-Ly
    f2 = ina.poly_itn(s2, [1.0, 0.5, 0.25], dim=1) + ina.cos_itn(s2, dim=2)
    Z = ina.map_to_zero_operator(s2, [0, last2, 0, last2], [1, 1, 2, 2])
    phi2 = ina.operate([Z], f2, cutoff=0.0, maxdim=10, normalize=False)
    ys = np.array([0.0, 2.0**-Ly, 0.25, 0.5, 0.625, 0.875, last2])
    for x in [0.0, last2]:
        vals = phi2.evaluate_batch(np.stack([np.full_like(ys, x), ys], 1), [1, 2])
        assert np.all(np.abs(vals) < 1e-8)


def test_truncate_recovers_rank(ina):
    """f + f has bond 2 chi and rank chi: truncation restores chi and the values."""
    graph = O.comb_tree_graph((3, 4))
    rng = np.random.default_rng(21)
    s_or = O.siteinds(graph, map_dimension=2)
    net = O.random_net(s_or, 3, rng)
    f, s = upload_oracle(ina, graph, net)
    ff = f + f
    assert ff.maxlinkdim() == 6
    t = ina.truncate(ff, cutoff=1e-14)
    X = rng.random((200, 2))
    assert rel_err(t.evaluate_batch(X, [1, 2]), 2 * f.evaluate_batch(X, [1, 2])) < 1e-12
    assert t.maxlinkdim() <= 3
    # bond spectra agree with the oracle's dense Schmidt values
    lay = s.layout
    order = [i for v in s_or.verts for i in s_or.site[v]]
    Fd = O.dense(O.net_add(net, net), order)
    for i, v in enumerate(lay.order):
        if lay.parent[i] < 0:
            continue
        # site legs of the subtree below v
        sub, stack = set(), [i]
        while stack:
            u = stack.pop()
            sub.add(lay.order[u])
            stack.extend(lay.children[u])
        axes = [k for k, ind in enumerate(order) if any(ind in s_or.site[w] for w in sub)]
        sv = O.bond_spectrum(Fd, axes)
        kept = sv[sv > 1e-10 * sv[0]]
        assert len(kept) == t.linkdims()[(lay.order[lay.parent[i]], v)]


@pytest.mark.parametrize("dtype", [float, complex])
def test_truncate_large_bonds(ina, dtype):
    """Bonds of 96 doubled to 192 by f + f (the SVDs of the middle bonds are
    large enough for the cluster-parallel Jacobi kernel): truncation restores
    the generic ranks min(96, 2^k, 2^(L-k)) and the values."""
    L = 16
    s = ina.continuous_siteinds(ina.named_path_graph(L))
    f = ina.rand_itn(s, link_space=96, rng=24, dtype=dtype, normalize=True)
    ff = f + f
    assert ff.maxlinkdim() == 192
    t = ina.truncate(ff, cutoff=1e-14)
    X = np.random.default_rng(25).random(512)
    assert rel_err(t.evaluate_batch(X), 2 * f.evaluate_batch(X)) < 1e-10
    expect = sorted(min(96, 2**k, 2 ** (L - k)) for k in range(1, L))
    assert sorted(t.linkdims().values()) == expect


@pytest.mark.parametrize("L,chi", [(12, 16), (20, 64)])
def test_mixed_truncation_matches_fp64(ina, L, chi):
    """FP32-preconditioned Jacobi (precision "mixed") gives the FP64 result:
    same ranks, values within 1e-9 of the plain FP64 path; single and batched."""
    s = ina.continuous_siteinds(ina.named_path_graph(L))
    f = ina.rand_itn(s, link_space=chi, rng=26, normalize=True)
    op = ina.first_derivative_operator(s)
    a = ina.operate(op, f, cutoff=1e-10, precision="f64")
    b = ina.operate(op, f, cutoff=1e-10, precision="mixed")
    X = np.random.default_rng(27).random(1000)
    assert a.linkdims() == b.linkdims()
    ref = a.evaluate_batch(X)
    assert rel_err(b.evaluate_batch(X), ref) < 1e-9
    # the batched sweeps (rank-revealing QR front ends) in both precisions
    for prec in ("mixed", "f64"):
        bb = ina.operate_batched([op] * 3, [f] * 3, cutoff=1e-10, precision=prec)
        for g in bb:
            assert g.linkdims() == a.linkdims()
            assert rel_err(g.evaluate_batch(X), ref) < 1e-9


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_apply_without_cutoff_is_exact(ina, precision):
    """cutoff 0 keeps every direction above the rounding floor: the result is
    the exact d/dx f on the dense grid (oracle stencil terms), in both the
    plain and the FP32-preconditioned factorisation."""
    L = 10
    s = ina.continuous_siteinds(ina.named_path_graph(L))
    f = ina.rand_itn(s, link_space=16, rng=28, normalize=True)
    g = ina.operate(ina.first_derivative_operator(s), f, cutoff=0.0, precision=precision)
    xs = np.arange(2**L) / 2.0**L
    F = f.evaluate_batch(xs)
    G = O.apply_terms_dense(O.stencil_terms(L, [0.0, 0.5, 0.0, -0.5, 0.0], 1), F.reshape((2,) * L),
                            {(1, k): k - 1 for k in range(1, L + 1)}).reshape(-1)
    assert rel_err(g.evaluate_batch(xs), G) < 1e-11


def test_truncate_maxdim_and_normalize(ina):
    graph = O.path_graph(10)
    rng = np.random.default_rng(22)
    s_or = O.siteinds(graph)
    net = O.random_net(s_or, 8, rng)
    f, _ = upload_oracle(ina, graph, net)
    t = ina.truncate(f, cutoff=0.0, maxdim=4)
    assert t.maxlinkdim() <= 4
    # the maxdim-truncated network is the best rank-4 TT in the sweep sense:
    # its norm is at most that of f and its overlap is real positive
    n = ina.truncate(f, cutoff=1e-14, normalize=True)
    assert abs(n.norm() - 1.0) < 1e-12
    assert abs(ina.inner(f, f) - f.norm() ** 2) < 1e-9 * f.norm() ** 2


def test_inner_and_integrate_operator(ina):
    graph = O.comb_tree_graph((3, 3))
    rng = np.random.default_rng(23)
    s_or = O.siteinds(graph, map_dimension=2)
    n1, n2 = O.random_net(s_or, 3, rng), O.random_net(s_or, 4, rng)
    f1, s = upload_oracle(ina, graph, n1)
    f2, _ = upload_oracle(ina, graph, n2)
    order = [i for v in s_or.verts for i in s_or.site[v]]
    D1, D2 = O.dense(n1, order), O.dense(n2, order)
    assert abs(ina.inner(f1, f2) - np.vdot(D1, D2)) < 1e-12 * np.linalg.norm(D1) * np.linalg.norm(D2)
    # integrate(operator_proj(f1), f2) = mean over the grid of f1 f2
    P = ina.operator_proj(f1)
    val = ina.integrate(P, f2)
    assert abs(val - np.mean(D1 * D2)) < 1e-12 * np.mean(np.abs(D1 * D2))
    # test/test_integration.jl:15-26
    s3 = ina.continuous_siteinds(ina.named_comb_tree((2, 10)))
    e = ina.exp_itn(s3, dim=1)
    assert abs(ina.integrate(ina.operator_proj(e), e) - 0.5 * (np.e**2 - 1)) < 1e-4


def test_config1_apply_truncate_evaluate_integrate(ina):
    """The reference's CPU case: f = exp(-x) + sin(2 pi x) on a 20-site path,
    second derivative (Dirichlet), truncate (cutoff 1e-12, maxdim 32), 4096
    points (seed 0), integrate -- against the oracle's dense-grid operator."""
    L = 20
    s = ina.continuous_siteinds(ina.named_grid((L, 1)))
    f = ina.exp_itn(s, k=-1.0) + ina.sin_itn(s, k=2 * np.pi)
    op = ina.second_derivative_operator(s)
    g = ina.operate(op, f, cutoff=1e-12, maxdim=32)
    rng = np.random.default_rng(0)
    X = rng.random((4096, 1))
    got = g.evaluate_batch(X)
    so = O.siteinds(O.path_graph(L))
    fo = O.net_add(O.exp_itn(so, k=-1.0), O.sin_itn(so, k=2 * np.pi))
    F, inds = O.dense_grid_1d(fo)
    terms = O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2)
    G = O.apply_terms_dense(terms, F.reshape((2,) * L), {(1, k): k - 1 for k in range(1, L + 1)})
    G = G.reshape(-1).real
    idx = np.floor(X[:, 0] * 2**L).astype(int)
    ref = G[idx]
    scale = np.max(np.abs(G))
    assert np.max(np.abs(got - ref)) / scale < 1e-8
    assert abs(g.integrate() - np.mean(G)) / scale < 1e-8
    assert g.maxlinkdim() <= 32


def test_batched_apply_matches_single(ina):
    """Config-5 shapes at reduced size: paths of uneven length and bond
    dimension applied and truncated in one batched pass equal the per-network
    results (function values)."""
    from itensornumericalanalysis.workloads import uneven_mps_batch, upload_batch

    batch = uneven_mps_batch(n=12, seed=3, lmin=6, lmax=14, chimin=2, chimax=24)
    fs = upload_batch(batch)
    ops = {}
    for s, _ in batch:
        L = s.nv()
        if L not in ops:
            ops[L] = ina.first_derivative_operator(s)
    oplist = [ops[s.nv()] for s, _ in batch]
    outs = ina.operate_batched(oplist, fs, cutoff=1e-10)
    rng = np.random.default_rng(60)
    X = rng.random((200, 1))
    for o, f, g in zip(oplist, fs, outs):
        single = ina.operate(o, f, cutoff=1e-10)
        a, b = g.evaluate_batch(X), single.evaluate_batch(X)
        assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(b))
        assert g.linkdims() == single.linkdims()
    tr = ina.truncate_batched(outs, cutoff=1e-6)
    for g, t in zip(outs, tr):
        a, b = t.evaluate_batch(X), g.evaluate_batch(X)
        assert np.linalg.norm(a - b) <= 1e-2 * np.linalg.norm(b)


@pytest.mark.parametrize("block", [8, 1000])
def test_general_opsum_compiles_to_its_dense_operator(ina, block, monkeypatch):
    """A long OpSum of digit operators and explicit 2 x 2 site matrices (the
    ttn(OpSum) call of src/elementary_operators.jl:151, widened to arbitrary
    product terms): the compiled operator applied to f equals the term-by-term
    sum on the dense grid, whether it is compiled in one direct sum or in
    blocks of 8 terms summed with recompression."""
    import itensornumericalanalysis.elementary_operators as eo
    from oracle.itn import OPS

    monkeypatch.setattr(eo, "OPSUM_BLOCK", block)
    L = 8
    s = ina.continuous_siteinds(ina.named_path_graph(L))
    f = ina.rand_itn(s, link_space=4, rng=90, normalize=True)
    rng = np.random.default_rng(91)
    names = ["D+", "D-", "Dup", "Ddn"]
    opsum = ina.OpSum()
    dense_terms = []
    for _ in range(150):
        digits = rng.choice(np.arange(1, L + 1), size=int(rng.integers(1, 4)), replace=False)
        ops, mats = {}, {}
        for k in digits:
            if rng.random() < 0.3:
                m = rng.standard_normal((2, 2))
                ops[(1, int(k))], mats[int(k)] = m, m
            else:
                nm = names[int(rng.integers(0, 4))]
                ops[(1, int(k))], mats[int(k)] = nm, OPS[nm]
        c = float(rng.standard_normal())
        opsum.add(c, ops)
        dense_terms.append((c, mats))
    op = ina.ttn(opsum, s, cutoff=1e-15)
    g = ina.operate(op, f, cutoff=0.0)
    xs = _grid(L)
    F = f.evaluate_batch(xs).reshape((2,) * L)
    G = np.zeros_like(F)
    for c, mats in dense_terms:
        H = F
        for k, m in mats.items():  # digit k is axis k - 1 (most significant first)
            H = np.moveaxis(np.tensordot(m, H, axes=([1], [k - 1])), 0, k - 1)
        G = G + c * H
    assert rel_err(g.evaluate_batch(xs), G.reshape(-1)) < 1e-10
    assert op.maxlinkdim() <= 4 ** (L // 2)  # the rank bound of an operator on L / 2 digits

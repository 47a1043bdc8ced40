"""Pin the CPU oracle to the reference's own known-answer tests.

Each case restates a testset of ITensorNumericalAnalysis.jl (file:line given)
with the same graphs, points and tolerances.  Where the reference draws
random parameters with Julia's RNG (seed 1234 / 42), numpy-seeded values are
used instead: the expected value is analytic either way.
"""
import zlib

import numpy as np
import pytest

import oracle as O
from oracle import itn as OI

RTOL = np.sqrt(np.finfo(float).eps)  # Julia's default isapprox rtol


def approx(a, b, rtol=RTOL, atol=0.0):
    return abs(a - b) <= atol + rtol * max(abs(a), abs(b))


# --------------------------------------------------------- index maps ----
def test_indexmap_real_roundtrip():  # test/test_indexmaps.jl:16-31
    s = O.siteinds(O.grid_graph((4, 4)))
    iv = O.calculate_ind_values(s, [0.625], [1])
    assert set(iv) == {i for v in s.verts for i in s.site[v]}
    assert O.calculate_p(s, iv, [1])[0] == 0.625


def test_indexmap_complex_roundtrip():  # test/test_indexmaps.jl:33-48
    s = O.complex_siteinds(O.grid_graph((4, 4)))
    z = 0.625 + 0.5j
    iv = O.calculate_ind_values(s, [z], [1])
    assert O.calculate_p(s, iv, [1])[0] == z


def test_indexmap_complex_multidim():  # test/test_indexmaps.jl:50-71
    L = 10
    dv = [[(i, j) for i in range(1, L + 1)] for j in range(1, L + 1)]
    s = O.complex_siteinds(O.grid_graph((L, L)), dv, dv)
    z1, z2 = 0.5 + 0.125j, 0.75 + 0.625j
    iv = O.calculate_ind_values(s, [z1, z2], [1, 2])
    p = O.calculate_p(s, iv, [1, 2])
    assert p[0] == z1 and p[1] == z2
    rng = np.random.default_rng(1234)
    xs = rng.random(L) + 1j * rng.random(L)
    iv = O.calculate_ind_values(s, list(xs), list(range(1, L + 1)))
    back = O.calculate_p(s, iv, list(range(1, L + 1)))
    assert np.allclose(back, xs, atol=2.0**-L * 2)


def test_digits_base2_are_binary_expansion():
    rng = np.random.default_rng(0)
    for x in rng.random(200):
        d = O.digits_greedy(x, 2, 30)
        assert d == [int(np.floor(x * 2**k)) % 2 for k in range(1, 31)]


# ------------------------------------------------------- constructors ----
def test_const():  # test/test_realitensorfunction.jl:39-57
    s = O.siteinds(O.grid_graph((3, 3)))
    assert approx(O.evaluate(O.const_itn(s, c=1.5), [0.5]), 1.5)
    assert approx(O.evaluate(O.const_itn(s, c=1.5, linkdim=4), [0.5]), 1.5)


FUNCS = [
    ("cosh", O.cosh_itn, np.cosh),
    ("sinh", O.sinh_itn, np.sinh),
    ("exp", O.exp_itn, np.exp),
    ("cos", O.cos_itn, np.cos),
    ("sin", O.sin_itn, np.sin),
]


@pytest.mark.parametrize("name,net,fn", FUNCS)
def test_functions_binary(name, net, fn):  # test/test_realitensorfunction.jl:65-80
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    a, k, c = rng.random(3)
    s = O.siteinds(O.comb_tree_graph((2, 3)))
    x = 0.625
    assert approx(O.evaluate(net(s, k=k, a=a, c=c), [x]), c * fn(k * x + a))


@pytest.mark.parametrize("name,net,fn", FUNCS)
def test_functions_trinary(name, net, fn):  # test/test_realitensorfunction.jl:89-104
    rng = np.random.default_rng(zlib.crc32(name.encode()) + 1)
    a, k, c = rng.random(3)
    s = O.siteinds(O.comb_tree_graph((2, 3)), base=3)
    x = 5.0 / 9.0
    assert approx(O.evaluate(net(s, k=k, a=a, c=c), [x]), c * fn(k * x + a))


def test_tanh():  # test/test_realitensorfunction.jl:106-121
    rng = np.random.default_rng(7)
    a, k, c = rng.random(3)
    s = O.siteinds(O.grid_graph((10, 1)))
    x = 0.625
    assert approx(O.evaluate(O.tanh_itn(s, k=k, a=a, c=c, nterms=50), [x]), c * np.tanh(k * x + a))


def _random_tree(n, rng):
    """Pruefer-code random tree on vertices (i, 1), as Graphs.uniform_tree."""
    verts = [(i, 1) for i in range(1, n + 1)]
    code = list(rng.integers(1, n + 1, size=n - 2))
    deg = [1] * (n + 1)
    for x in code:
        deg[x] += 1
    edges = []
    for x in code:
        leaf = next(i for i in range(1, n + 1) if deg[i] == 1)
        edges.append(((leaf, 1), (int(x), 1)))
        deg[leaf] -= 1
        deg[x] -= 1
    u, w = [i for i in range(1, n + 1) if deg[i] == 1]
    edges.append(((u, 1), (w, 1)))
    return verts, edges


def test_poly():  # test/test_realitensorfunction.jl:123-144
    rng = np.random.default_rng(1234)
    for deg in range(1, 12):
        s = O.siteinds(_random_tree(6, rng))
        k, c = rng.random(2)
        coeffs = rng.random(deg + 1)
        x = 0.875
        val = O.evaluate(O.poly_itn(s, list(coeffs), k=k, c=c), [x])
        exact = c * sum(coeffs[i] * (k * x) ** i for i in range(deg + 1))
        assert abs(val - exact) <= 1e-4


def test_const_3d():  # test/test_realitensorfunction.jl:147-160
    s = O.siteinds(O.grid_graph((3, 3)), map_dimension=3)
    assert approx(O.evaluate(O.const_itn(s, c=1.5), [0.5, 0.25, 0.0], [1, 2, 3]), 1.5)


@pytest.mark.parametrize("name,net,fn", FUNCS)
def test_sum_of_1d_functions_2d(name, net, fn):  # test/test_realitensorfunction.jl:162-189
    rng = np.random.default_rng(zlib.crc32(name.encode()) + 2)
    a, k, c = rng.random(3)
    s = O.siteinds(O.grid_graph((10, 1)), map_dimension=2)
    x, y = 0.625, 0.25
    f = O.net_add(net(s, k=k, a=a, c=c, dim=1), net(s, k=k, a=a, c=c, dim=2))
    assert approx(O.evaluate(f, [x, y], [1, 2]), c * fn(k * x + a) + c * fn(k * y + a))


def test_tanh_2d():  # test/test_realitensorfunction.jl:191-208
    rng = np.random.default_rng(11)
    a, k, c = rng.random(3)
    s = O.siteinds(O.grid_graph((3, 2)), map_dimension=2)
    x, y = 0.625, 0.875
    f = O.net_add(O.tanh_itn(s, k=k, a=a, c=c, nterms=20, dim=1),
                  O.tanh_itn(s, k=k, a=a, c=c, nterms=20, dim=2))
    assert approx(O.evaluate(f, [x, y], [1, 2]), c * np.tanh(k * x + a) + c * np.tanh(k * y + a))


def test_delta_p():  # test/test_realitensorfunction.jl:210-259
    L = 10
    s = O.siteinds(O.grid_graph((L, 1)), map_dimension=2)
    x0, y0 = 0.625, 0.25
    d = 2.0 ** -L
    xs = [0.0, d, 0.25, 0.5, 0.625, 0.875, 1 - d]
    psi = O.delta_p(s, [x0, y0])
    assert approx(O.evaluate(psi, [x0, y0], [1, 2]), 1.0)
    assert abs(O.evaluate(psi, [y0, x0], [1, 2])) < 1e-14
    plane = O.delta_p(s, [y0], [2])
    for x in xs:
        assert approx(O.evaluate(plane, [x, y0], [1, 2]), 1.0)
        assert abs(O.evaluate(plane, [x, 0.5], [1, 2])) < 1e-14


@pytest.mark.parametrize("name,net,fn", FUNCS)
def test_complex_functions(name, net, fn):  # test/test_complexitensorfunction.jl:57-80
    rng = np.random.default_rng(zlib.crc32(name.encode()) + 3)
    a, k, c = rng.random(3) + 1j * rng.random(3)
    s = O.complex_siteinds(O.comb_tree_graph((2, 3)), [[(1, 1), (1, 2), (1, 3)]],
                           [[(2, 1), (2, 2), (2, 3)]])
    z = 0.625 + 0.25j
    assert approx(O.evaluate(net(s, k=k, a=a, c=c), [z]), c * fn(k * z + a))


@pytest.mark.parametrize("name,net,fn", FUNCS)
def test_complex_functions_trinary(name, net, fn):  # test/test_complexitensorfunction.jl:92-110
    rng = np.random.default_rng(zlib.crc32(name.encode()) + 4)
    a, k, c = rng.random(3) + 1j * rng.random(3)
    s = O.complex_siteinds(O.comb_tree_graph((2, 3)), [[(1, 1), (1, 2), (1, 3)]],
                           [[(2, 1), (2, 2), (2, 3)]], base=3)
    z = 5.0 / 9.0 + 4.0j / 9.0
    assert approx(O.evaluate(net(s, k=k, a=a, c=c), [z]), c * fn(k * z + a))


def test_complex_tanh():  # test/test_complexitensorfunction.jl:113-130
    rng = np.random.default_rng(13)
    a, k, c = rng.random(3) + 1j * rng.random(3)
    L = 10
    s = O.complex_siteinds(O.grid_graph((L, 1)), [[(i, 1) for i in range(1, L + 1, 2)]],
                           [[(i, 1) for i in range(2, L + 1, 2)]])
    z = 0.625 + 0.125j
    assert approx(O.evaluate(O.tanh_itn(s, k=k, a=a, c=c, nterms=50), [z]), c * np.tanh(k * z + a))


def test_complex_poly():  # test/test_complexitensorfunction.jl:132-157
    rng = np.random.default_rng(4321)
    L = 6
    for deg in range(1, 12):
        s = O.complex_siteinds(_random_tree(L, rng), [[(i, 1) for i in range(1, L + 1, 2)]],
                               [[(i, 1) for i in range(2, L + 1, 2)]])
        k, c = rng.random(2) + 1j * rng.random(2)
        coeffs = rng.random(deg + 1) + 1j * rng.random(deg + 1)
        z = 0.875 + 0.25j
        val = O.evaluate(O.poly_itn(s, list(coeffs), k=k, c=c), [z])
        exact = c * sum(coeffs[i] * (k * z) ** i for i in range(deg + 1))
        assert abs(val - exact) <= 1e-4


def test_complex_const_3d():  # test/test_complexitensorfunction.jl:161-172
    s = O.complex_siteinds(O.grid_graph((3, 3)), map_dimension=3)
    z = [0.5 + 0.125j, 0.25 + 0.875j, 0.0]
    assert approx(O.evaluate(O.const_itn(s, c=1.5), z, [1, 2, 3]), 1.5)


@pytest.mark.parametrize("name,net,fn", FUNCS)
def test_complex_sum_of_1d_functions_2d(name, net, fn):  # test/test_complexitensorfunction.jl:174-208
    rng = np.random.default_rng(zlib.crc32(name.encode()) + 5)
    a, k, c = rng.random(3) + 1j * rng.random(3)
    L = 10
    h = L // 2
    real_dv = [[(i, 1) for i in range(1, h + 1)], [(i, 1) for i in range(h + 1, L + 1)]]
    imag_dv = [[(i, 1) for i in range(h + 1, L + 1)], [(i, 1) for i in range(1, h + 1)]]
    s = O.complex_siteinds(O.grid_graph((L, 1)), real_dv, imag_dv)
    z1, z2 = 0.625 + 0.875j, 0.25 + 0.125j
    f = O.net_add(net(s, k=k, a=a, c=c, dim=1), net(s, k=k, a=a, c=c, dim=2))
    assert approx(O.evaluate(f, [z1, z2], [1, 2]), c * fn(k * z1 + a) + c * fn(k * z2 + a))


def test_complex_tanh_2d():  # test/test_complexitensorfunction.jl:210-227
    rng = np.random.default_rng(17)
    a, k, c = rng.random(3) + 1j * rng.random(3)
    s = O.complex_siteinds(O.grid_graph((3, 2)), map_dimension=2)
    z1, z2 = 0.5 + 0.125j, 0.625 + 0.25j
    f = O.net_add(O.tanh_itn(s, k=k, a=a, c=c, nterms=50, dim=1),
                  O.tanh_itn(s, k=k, a=a, c=c, nterms=50, dim=2))
    assert approx(O.evaluate(f, [z1, z2], [1, 2]), c * np.tanh(k * z1 + a) + c * np.tanh(k * z2 + a))


# ------------------------------------------------------------ operators ----
def _dense_1d(f):
    F, inds = O.dense_grid_1d(f)
    return F, len(inds)


def _shift_dense(F, L, fwd, boundary, n=0):
    terms = (O.forward_shift_terms if fwd else O.backward_shift_terms)(L, 1, boundary, n)
    T = F.reshape((2,) * L)
    G = O.apply_terms_dense(terms, T, {(1, k): k - 1 for k in range(1, L + 1)})
    return G.reshape(-1)


@pytest.mark.parametrize("n", [0, 1])
@pytest.mark.parametrize("boundary", ["Dirichlet", "Periodic", "Neumann"])
def test_shift_operators(boundary, n):  # test/test_operators.jl:168-287
    s = O.siteinds(O.comb_tree_graph((2, 3)))
    L = 6
    N = 2**L
    F, _ = _dense_1d(O.poly_itn(s, [1.0, 0.5, 0.25]))
    step = n + 1
    fwd = _shift_dense(F, L, True, boundary, n)
    bwd = _shift_dense(F, L, False, boundary, n)
    for i in range(N):
        if i + step < N:
            assert abs(fwd[i] - F[i + step]) < 1e-8
        elif boundary == "Dirichlet":
            assert abs(fwd[i]) < 1e-8
        elif boundary == "Periodic":
            assert abs(fwd[i] - F[i + step - N]) < 1e-8
        else:  # Neumann: the top block reads itself
            assert abs(fwd[i] - F[i]) < 1e-8
        if i - step >= 0:
            assert abs(bwd[i] - F[i - step]) < 1e-8
        elif boundary == "Dirichlet":
            assert abs(bwd[i]) < 1e-8
        elif boundary == "Periodic":
            assert abs(bwd[i] - F[i - step + N]) < 1e-8
        else:
            assert abs(bwd[i] - F[i]) < 1e-8


def test_derivatives_periodic_mps():  # test/test_operators.jl:16-46
    L = 9
    s = O.siteinds(O.grid_graph((L, 1)))
    F, _ = _dense_1d(O.sin_itn(s, k=2 * np.pi))
    d = 2.0**-L
    stencils = {
        1: [0.0, 0.5, 0.0, -0.5, 0.0],
        2: [0.0, 1.0, -2.0, 1.0, 0.0],
        3: [0.5, -1.0, 0.0, 1.0, -0.5],
        4: [1.0, -4.0, 6.0, -4.0, 1.0],
    }
    exact = {
        1: lambda x: 2 * np.pi * np.cos(2 * np.pi * x),
        2: lambda x: -(2 * np.pi) ** 2 * np.sin(2 * np.pi * x),
        3: lambda x: -(2 * np.pi) ** 3 * np.cos(2 * np.pi * x),
        4: lambda x: (2 * np.pi) ** 4 * np.sin(2 * np.pi * x),
    }
    for p, sh in stencils.items():
        terms = O.stencil_terms(L, sh, p, 1, "Periodic", "Periodic")
        G = O.apply_terms_dense(terms, F.reshape((2,) * L), {(1, k): k - 1 for k in range(1, L + 1)})
        G = G.reshape(-1)
        for x in [0.0, 0.25, 0.625, 0.875, 1.0 - d]:
            i = int(round(x / d))
            assert approx(1.0 + G[i].real, 1.0 + exact[p](x), rtol=1e-3)


# ----------------------------------------------------------- integration ----
def test_integrate_operator_times_function():  # test/test_integration.jl:15-26
    L = 20
    s = O.siteinds(O.comb_tree_graph((2, L // 2)))
    f = O.exp_itn(s, dim=1)
    # integrate(operator_proj(f), f) = integral of f*f
    ans = O.integrate(O.net_multiply(f, f))
    assert abs(ans - 0.5 * (np.e**2 - 1)) <= 1e-4


def test_integrate_2d():  # test/test_integration.jl:28-38
    L = 30
    s = O.siteinds(O.comb_tree_graph((3, L // 3)), map_dimension=2)
    f = O.net_multiply(O.exp_itn(s, dim=1), O.exp_itn(s, dim=2))
    assert abs(O.integrate(f) - (np.e - 1) ** 2) <= 1e-4


def _grid(f, dims):
    """f on the full grid of the listed variables (axes: each variable's digits
    1..L in turn, so the flat index is the grid position) and the
    (dimension, digit) -> axis map apply_terms_dense takes."""
    inds, axis = [], {}
    for d in dims:
        di = sorted((i for i, (dd, k, r) in f.s.info.items() if dd == d and r), key=lambda i: f.s.info[i][1])
        for i in di:
            axis[(d, f.s.info[i][1])] = len(inds)
            inds.append(i)
    return O.dense(f, inds), axis


def test_first_derivative_on_comb():  # test/test_operators.jl:48-64
    s = O.siteinds(O.comb_tree_graph((4, 3)))
    L = 12
    F, axis = _grid(O.sin_itn(s, k=np.pi), [1])
    G = O.apply_terms_dense(O.stencil_terms(L, [0.0, 0.5, 0.0, -0.5, 0.0], 1), F, axis).reshape(-1)
    d = 2.0**-L
    for x in [d, 0.125, 0.25, 0.625, 0.875]:
        assert abs(G[int(round(x / d))].real - np.pi * np.cos(np.pi * x)) <= 1e-3


def test_first_derivative_of_3d_function():  # test/test_operators.jl:66-97
    """On the 45-site path (15 digits per variable) the derivative along y is
    taken on the y-grid of f(x, ., z), the x and z digits projected out as
    evaluate does: the stencil only acts on y's digits."""
    s = O.siteinds(O.path_graph(45), map_dimension=3)
    f = O.net_multiply(O.net_multiply(O.poly_itn(s, [0.0, -1.0, 1.0], dim=1), O.sin_itn(s, k=np.pi, dim=2)),
                       O.sin_itn(s, k=np.pi, dim=3))
    pts = [0.125, 0.25, 0.675]
    Ly = 15
    d = 2.0**-Ly
    yinds = sorted((i for i, (dd, k, r) in s.info.items() if dd == 2), key=lambda i: s.info[i][1])
    terms = O.stencil_terms(Ly, [0.0, 0.5, 0.0, -0.5, 0.0], 1, dim=2)
    for x in pts:
        for z in pts:
            iv = O.calculate_ind_values(s, [x, z], [1, 3])
            ts = []
            for v, T in f.T.items():
                for i in s.site[v]:
                    if i in iv:
                        T = O.contract([T, OI.onehot(i, iv[i])])
                ts.append(T)
            Fy = O.contract(ts).permute(yinds).arr
            G = O.apply_terms_dense(terms, Fy, {(2, k): k - 1 for k in range(1, Ly + 1)}).reshape(-1)
            for y in pts:
                exact = (x * x - x) * np.sin(np.pi * y) * np.sin(np.pi * z)
                assert abs(O.evaluate(f, [x, y, z], [1, 2, 3]).real - exact) <= 1e-3
                dexact = np.pi * (x * x - x) * np.cos(np.pi * y) * np.sin(np.pi * z)
                assert abs(G[int(y / d)].real - dexact) <= 1e-3


def test_multiplication_1d():  # test/test_operators.jl:99-116 and :148-166
    """g f on a comb; operator_proj(f) applied to g is the same pointwise product."""
    s = O.siteinds(O.comb_tree_graph((4, 3)))
    g, f = O.sin_itn(s, k=0.5 * np.pi), O.cos_itn(s, k=0.25 * np.pi)
    fg, ff = O.net_multiply(g, f), O.net_multiply(f, f)
    for x in [0.025, 0.1, 0.25, 0.625, 0.875]:
        assert abs(O.evaluate(fg, [x]).real - np.sin(0.5 * np.pi * x) * np.cos(0.25 * np.pi * x)) <= 1e-3
        assert abs(O.evaluate(ff, [x]).real - np.cos(0.25 * np.pi * x) ** 2) <= 1e-3


def test_multiplication_2d_random_tree():  # test/test_operators.jl:118-146
    s = O.siteinds(_random_tree(8, np.random.default_rng(8)), map_dimension=2)
    fx, gy = O.cos_itn(s, k=0.25 * np.pi, dim=1), O.sin_itn(s, k=0.5 * np.pi, dim=2)
    fg, gg = O.net_multiply(fx, gy), O.net_multiply(gy, gy)
    pts = [0.125, 0.25, 0.625, 0.875]
    for x in pts:
        for y in pts:
            assert approx(O.evaluate(fx, [x, y], [1, 2]).real, np.cos(0.25 * np.pi * x))
            assert approx(O.evaluate(gy, [x, y], [1, 2]).real, np.sin(0.5 * np.pi * y))
            assert abs(O.evaluate(fg, [x, y], [1, 2]).real
                       - np.cos(0.25 * np.pi * x) * np.sin(0.5 * np.pi * y)) <= 1e-3
            assert abs(O.evaluate(gg, [x, y], [1, 2]).real - np.sin(0.5 * np.pi * y) ** 2) <= 1e-3


@pytest.mark.parametrize("boundary", ["Dirichlet", "Periodic", "Neumann"])
@pytest.mark.parametrize("case", ["reference", "x_plus_y"])
def test_shift_operators_2d(boundary, case):  # test/test_operators.jl:289-351
    """Shifts of variable 2 on a 3 x 3 comb.  The reference's function is
    f_x + f_x (a function of x alone, so only the boundary rows move); the
    second case adds cos(y) so every row moves."""
    s = O.siteinds(O.comb_tree_graph((3, 3)), map_dimension=2)
    fx = O.poly_itn(s, [1.0, 0.5, 0.25], dim=1)
    f = O.net_add(fx, fx) if case == "reference" else O.net_add(fx, O.cos_itn(s, dim=2))
    L1 = sum(1 for (d, k, r) in s.info.values() if d == 1)
    L2 = sum(1 for (d, k, r) in s.info.values() if d == 2)
    F, axis = _grid(f, [1, 2])
    fwd = O.apply_terms_dense(O.forward_shift_terms(L2, 2, boundary), F, axis).reshape(2**L1, 2**L2)
    bwd = O.apply_terms_dense(O.backward_shift_terms(L2, 2, boundary), F, axis).reshape(2**L1, 2**L2)
    F = F.reshape(2**L1, 2**L2)
    d = 2.0**-L2
    ix = int(0.5 * 2**L1)
    for y in [0.0, d, 0.25, 0.5, 0.625, 0.875, 1.0 - d]:
        iy = int(round(y / d))
        if y + d < 1:
            assert abs(fwd[ix, iy] - F[ix, iy + 1]) <= 1e-8
        else:
            want = {"Dirichlet": 0.0, "Periodic": F[ix, 0], "Neumann": F[ix, iy]}[boundary]
            assert abs(fwd[ix, iy] - want) <= 1e-8
        if y - d >= 0:
            assert abs(bwd[ix, iy] - F[ix, iy - 1]) <= 1e-8
        else:
            want = {"Dirichlet": 0.0, "Periodic": F[ix, -1], "Neumann": F[ix, 0]}[boundary]
            assert abs(bwd[ix, iy] - want) <= 1e-8


def test_partial_integrate_3d():  # test/test_integration.jl:40-54 (src/integration.jl:35-54)
    """exp(x) cos(y) exp(z) on a 3 x 30 comb (one tooth per variable), its
    y and z digits summed with weight 1/2 each (partial_integrate over [2, 3];
    merging the leg-less vertices does not change the value), then evaluated
    at x = 0.875."""
    L = 90
    s = O.siteinds(O.comb_tree_graph((3, L // 3)), [[(i, j) for j in range(1, L // 3 + 1)] for i in range(1, 4)])
    f = O.net_multiply(O.net_multiply(O.exp_itn(s, dim=1), O.cos_itn(s, dim=2)), O.exp_itn(s, dim=3))
    x = 0.875
    iv = O.calculate_ind_values(s, [x], [1])
    ts = []
    for v in s.verts:
        t = f.T[v]
        for i in s.site[v]:
            w = np.full(i.dim, 1.0 / s.base) if s.info[i][0] in (2, 3) else OI.onehot(i, iv[i]).arr
            t = O.contract([t, O.Tensor(w, [i])])
        ts.append(t)
    val = O.contract(ts).scalar()
    assert abs(val - (np.e - 1) * np.sin(1) * np.exp(x)) <= 1e-8


def test_multi_dimensional_complex_example():  # examples/construct_multi_dimensional_function.jl
    """z1^3 (z2 + z2^2) + cosh(pi z3)^2 on a 3 x 4 comb, each variable's real
    digits on one tooth and its imaginary digits on another, reversed."""
    L = 4
    real_dv = [[(j, i) for i in range(1, L + 1)] for j in range(1, 4)]
    imag_dv = [[(j, i) for i in range(L, 0, -1)] for j in range(3, 0, -1)]
    s = O.complex_siteinds(O.comb_tree_graph((3, L)), real_dv, imag_dv)
    f = O.net_add(O.net_multiply(O.poly_itn(s, [0.0, 0.0, 0.0, 1.0], dim=1), O.poly_itn(s, [0.0, 1.0, 1.0], dim=2)),
                  O.net_multiply(O.cosh_itn(s, k=np.pi, dim=3), O.cosh_itn(s, k=np.pi, dim=3)))
    z1, z2, z3 = 0.125 + 0.5j, 0.625 + 0.875j, 0.5
    exact = z1**3 * (z2 + z2**2) + np.cosh(np.pi * z3) ** 2
    assert approx(O.evaluate(f, [z1, z2, z3], [1, 2, 3]), exact)

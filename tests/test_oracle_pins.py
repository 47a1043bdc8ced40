"""Pin the CPU oracle to the reference's own known-answer tests.

Each case restates a testset of ITensorNumericalAnalysis.jl (file:line given)
with the same graphs, points and tolerances.  Where the reference draws
random parameters with Julia's RNG (seed 1234 / 42), numpy-seeded values are
used instead: the expected value is analytic either way.
"""
import numpy as np
import pytest

import oracle as O

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
    rng = np.random.default_rng(hash(name) % 2**32)
    a, k, c = rng.random(3)
    s = O.siteinds(O.comb_tree_graph((2, 3)))
    x = 0.625
    assert approx(O.evaluate(net(s, k=k, a=a, c=c), [x]), c * fn(k * x + a))


@pytest.mark.parametrize("name,net,fn", FUNCS)
def test_functions_trinary(name, net, fn):  # test/test_realitensorfunction.jl:89-104
    rng = np.random.default_rng(hash(name) % 2**32 + 1)
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
    from itertools import count  # noqa: F401

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
    rng = np.random.default_rng(hash(name) % 2**32 + 2)
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
    rng = np.random.default_rng(hash(name) % 2**32 + 3)
    a, k, c = rng.random(3) + 1j * rng.random(3)
    s = O.complex_siteinds(O.comb_tree_graph((2, 3)), [[(1, 1), (1, 2), (1, 3)]],
                           [[(2, 1), (2, 2), (2, 3)]])
    z = 0.625 + 0.25j
    assert approx(O.evaluate(net(s, k=k, a=a, c=c), [z]), c * fn(k * z + a))


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

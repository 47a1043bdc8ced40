"""CPU tests: the C-ABI library loads and exports every declared symbol; the
host-side graph / digit-map / constructor logic agrees with the oracle."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import oracle as O

ROOT = Path(__file__).resolve().parent.parent


def _declared_symbols():
    text = (ROOT / "include" / "tnfa.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tnfa_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import itensornumericalanalysis._build as b

    if not b.LIB_PATH.exists():
        b.build()
    return C.CDLL(str(b.LIB_PATH))


def test_library_exports_every_declared_symbol(lib):
    syms = _declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_ctypes_signatures_cover_the_header():
    from itensornumericalanalysis import _lib

    assert set(_declared_symbols()) == set(_lib.SIGNATURES)


def test_version_and_null_arguments(lib):
    from itensornumericalanalysis import _lib

    L = _lib.load()
    assert L.tnfa_version().decode().startswith("tnfa ")
    # null handles are rejected without touching a device
    assert L.tnfa_net_destroy(None) == _lib.ERR_INVALID_ARGUMENT
    assert L.tnfa_ctx_destroy(None) == _lib.ERR_INVALID_ARGUMENT
    assert L.tnfa_net_info(None, None, None, None, None) == _lib.ERR_INVALID_ARGUMENT
    assert L.tnfa_last_error_string(None) == b"null context"


def test_graph_generators_match_oracle():
    import itensornumericalanalysis as ina

    for g, (ov, oe) in [
        (ina.named_grid((4, 3)), O.grid_graph((4, 3))),
        (ina.named_comb_tree((3, 4)), O.comb_tree_graph((3, 4))),
        (ina.named_binary_tree(60), O.binary_tree_graph(60)),
    ]:
        assert g.vertices() == ov
        assert set(map(frozenset, g.edges())) == set(map(frozenset, oe))
    assert ina.named_comb_tree((2, 16)).is_tree()
    assert not ina.named_grid((3, 3)).is_forest()
    t = ina.uniform_tree(30, 0)
    assert t.is_tree() and t.nv() == 30


def test_tree_layout_is_topological():
    import itensornumericalanalysis as ina

    for g in [ina.named_comb_tree((4, 3)), ina.named_binary_tree(60), ina.uniform_tree(40, 3)]:
        lay = ina.continuous_siteinds(g).layout
        assert lay.parent[0] == -1
        assert all(p < i for i, p in enumerate(lay.parent) if p >= 0)
        for i, ch in enumerate(lay.children):
            assert ch == sorted(ch)
            assert all(lay.parent[c] == i for c in ch)
    with pytest.raises(ValueError):
        ina.continuous_siteinds(ina.named_grid((3, 3))).layout


def test_host_digit_map_matches_oracle():
    import itensornumericalanalysis as ina

    rng = np.random.default_rng(0)
    for base in (2, 3):
        g = ina.named_comb_tree((3, 4))
        s = ina.continuous_siteinds(g, base=base, map_dimension=2)
        so = O.siteinds(O.comb_tree_graph((3, 4)), base=base, map_dimension=2)
        for _ in range(50):
            xs = list(rng.random(2))
            iv = s.calculate_ind_values(xs, [1, 2])
            ivo = O.calculate_ind_values(so, xs, [1, 2])
            a = sorted((l.dim, l.digit, v) for l, v in iv.items())
            b = sorted((so.info[i][0], so.info[i][1], v) for i, v in ivo.items())
            assert a == b
        pts = s.calculate_p(s.calculate_ind_values([0.625, 0.25], [1, 2]), [1, 2])
        if base == 2:
            assert pts == [0.625, 0.25]
    with pytest.raises(ValueError):
        s.calculate_ind_values([-0.5, 0.1], [1, 2])


def test_grid_points():
    import itensornumericalanalysis as ina

    s = ina.continuous_siteinds(ina.named_grid((8, 1)))
    pts = s.grid_points(16, 1)
    assert pts[0] == 0.0 and all(p < 1 for p in pts)
    assert np.allclose(np.diff(pts), 1 / 16)
    assert ina.grid_points(s, 1) == [i / 256 for i in range(256)]  # every point (abstractindexmap.jl:149-155)
    assert ina.grid_points(s, 16, 1) == pts
    # complex map: the N x N products of the real and imaginary grids (complexindexmap.jl:134-144)
    sc = ina.complex_continuous_siteinds(ina.named_grid((8, 1)), [[(i, 1) for i in range(1, 5)]],
                                         [[(i, 1) for i in range(5, 9)]])
    zs = ina.grid_points(sc, 4, 1)
    assert len(zs) == 16 and set(zs) == {i / 4 + 1j * j / 4 for i in range(4) for j in range(4)}


def test_reduced_maps():
    import itensornumericalanalysis as ina

    g = ina.named_comb_tree((3, 5))
    s = ina.continuous_siteinds(g, [[(i, j) for j in range(1, 6)] for i in range(1, 4)])
    s2 = ina.reduced_indsnetworkmap(s, 2)
    assert s2.dimensions() == [2]
    assert s2.vertices() == [(2, j) for j in range(1, 6)]
    assert s2.is_tree()


def test_plan_and_autotune_entry_points_reject_null_handles(lib):
    from itensornumericalanalysis import _lib

    L = _lib.load()
    assert L.tnfa_eval_plan_destroy(None) == _lib.OK  # like free(NULL)
    assert L.tnfa_eval_plan_launch(None, None) == _lib.ERR_INVALID_ARGUMENT
    assert L.tnfa_eval_plan_check(None, None) == _lib.ERR_INVALID_ARGUMENT
    assert L.tnfa_eval_plan_create(None, None, None, 1, 0, None, None, 0, 0, None) == _lib.ERR_INVALID_ARGUMENT
    assert L.tnfa_ctx_set_autotune(None, 1, -1.0, 0) == _lib.ERR_INVALID_ARGUMENT
    need = C.c_int64()
    assert L.tnfa_ctx_tuning_report(None, None, 0, C.byref(need)) == _lib.ERR_INVALID_ARGUMENT


def test_opsum_site_operators_are_validated():
    """OpSum terms name a digit operator or give a base x base matrix."""
    from itensornumericalanalysis.elementary_operators import _op_matrix

    assert np.array_equal(_op_matrix("D+", 2), np.array([[0.0, 1.0], [0.0, 0.0]]))
    assert np.array_equal(_op_matrix("I", 3), np.eye(3))
    m = np.arange(4.0).reshape(2, 2)
    assert np.array_equal(_op_matrix(m, 2), m)
    with pytest.raises(ValueError, match="2x2"):
        _op_matrix(np.eye(3), 2)
    with pytest.raises(ValueError, match="unknown"):
        _op_matrix("Dx", 2)
    with pytest.raises(ValueError, match="base 2"):
        _op_matrix("D+", 3)


def test_reference_named_free_functions():
    """The reference's exported helpers (src/ITensorNumericalAnalysis.jl:20-66)
    as free functions on a map or a function's map: digit round trip through
    calculate_ind_values / calculate_p on grid points, vertex <-> (dimension,
    digit) bookkeeping, the index map and its type."""
    import itensornumericalanalysis as ina

    L = 5
    g = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g, [[(1, j) for j in range(L, 0, -1)], [(2, j) for j in range(1, L + 1)]])
    assert ina.dimensions(s) == [1, 2] and ina.dimension(s) == 2
    assert sorted(ina.dimension_vertices(s, 2)) == sorted((2, j) for j in range(1, L + 1))
    for v in s.vertices():
        d, k = ina.vertex_dimension(s, v), ina.vertex_digit(s, v)
        assert s.vertex(d, k) == v and ina.vertex(s, d, k) == v
        assert ina.vertex_dimensions(s, v) == [d] and ina.vertex_digits(s, v) == [k]
        (leg,) = s.inds(v)
        assert ina.digit(s, leg) == k and ina.index_value_to_scalar(s, leg, 1) == 2.0**-k
    assert ina.base(s) == 2 and ina.base(ina.continuous_siteinds(g, base=3)) == 3
    assert ina.indsnetworkmap(s) is s
    sc = ina.ComplexIndsNetworkMap(g)
    legs = ina.complex_digit_siteinds(g)
    assert sc.is_complex and all(sc.inds(v) == legs[v] for v in g.vertices())
    assert all([l.kind for l in legs[v]] == ["real", "imag"] or len(legs[v]) != 2 for v in g.vertices())
    assert ina.RealIndsNetworkMap is ina.continuous_siteinds
    vs = s.vertices()
    assert ina.vertices_dimensions(s, vs) == [ina.vertex_dimension(s, v) for v in vs]
    assert ina.vertices_digits(s, vs) == [ina.vertex_digit(s, v) for v in vs]
    assert len(ina.dimension_inds(s, 1)) == L
    rng = np.random.default_rng(130)
    for _ in range(20):
        x = np.floor(rng.random(2) * 2**L) / 2**L
        iv = ina.calculate_ind_values(s, list(x), [1, 2])
        assert np.allclose(ina.calculate_p(s, iv, [1, 2]), x)
    graph, legs = ina.indsnetwork(s)
    assert graph is s.graph and set(legs) == set(s.vertices())
    im = ina.indexmap(s)
    assert sorted(im.values()) == sorted((d, k) for d in (1, 2) for k in range(1, L + 1))
    assert isinstance(im, ina.RealIndexMap) and isinstance(im, ina.AbstractIndexMap)
    assert ina.indexmaptype(s) is ina.RealIndexMap
    sc = ina.complex_continuous_siteinds(ina.named_path_graph(4))
    assert ina.indexmaptype(sc) is ina.ComplexIndexMap and isinstance(ina.indexmap(sc), ina.ComplexIndexMap)


@pytest.mark.parametrize("boundary", ["Dirichlet", "Periodic", "Neumann"])
@pytest.mark.parametrize("n", [0, 1])
def test_shift_opsums_match_oracle_terms(boundary, n):
    """The product's OpSum term lists for the shift operators
    (src/elementary_operators.jl:32-103) equal the oracle's, term for term."""
    import itensornumericalanalysis as ina

    L = 7
    s = ina.continuous_siteinds(ina.named_path_graph(L))

    def canon(terms):
        return sorted((complex(c).real, complex(c).imag, tuple(sorted(o.items()))) for c, o in terms)

    for fwd in (True, False):
        mine = (ina.forward_shift_opsum if fwd else ina.backward_shift_opsum)(s, 1, boundary, n)
        ref = (O.forward_shift_terms if fwd else O.backward_shift_terms)(L, 1, boundary, n)
        assert canon(mine.terms) == canon(ref), (fwd, boundary, n)


def _on(s, x, p, d):
    """1 when the digits of point x agree with those of p on dims d."""
    full = s.calculate_ind_values(list(x), list(range(1, len(x) + 1)))
    part = s.calculate_ind_values(list(p), list(d))
    return float(all(full[l] == v for l, v in part.items()))


def _kernel_value(s, x, points, dims, coeff=-1.0):
    from itensornumericalanalysis.elementary_functions import _delta_overlaps

    over_p, over_d = _delta_overlaps(points, dims)
    val = 1.0 + coeff * sum(_on(s, x, p, d) for p, d in zip(points, dims))
    return val - coeff * sum(_on(s, x, p, d) for p, d in zip(over_p, over_d))


def test_delta_kernel_overlaps_match_reference_cases():
    """test/test_operators.jl:415-515 restated through the indicator the
    kernel stands for (1 + coeff sum of point/plane deltas - coeff sum of the
    overlaps that _delta_overlaps lists), at the reference's points."""
    import itensornumericalanalysis as ina

    # 1D: one point
    g = ina.named_comb_tree((2, 3))
    s = ina.continuous_siteinds(g)
    delta = 2.0 ** -g.nv()
    assert _kernel_value(s, [0.5], [[0.5]], [[1]]) == 0
    for x in [0.0, delta, 0.25, 0.625, 0.875, 1 - delta]:
        assert _kernel_value(s, [x], [[0.5]], [[1]]) == 1
    # 2D, intersecting lines and line + point
    g = ina.named_comb_tree((2, 3))
    s = ina.continuous_siteinds(g, map_dimension=2)
    delta = 2.0 ** -(g.nv() // 2)
    xs = [0.0, delta, 0.25, 0.625, 0.875, 1 - delta]
    P, D = [[0.5], [0.5]], [[1], [2]]
    assert _kernel_value(s, [0.5, 0.5], P, D) == 0
    for x in xs:
        assert _kernel_value(s, [x, 0.5], P, D) == 0
        assert _kernel_value(s, [0.5, x], P, D) == 0
        assert _kernel_value(s, [x, delta], P, D) == 1
        assert _kernel_value(s, [delta, x], P, D) == 1
    P, D = [[0.5], [0.5, 0.1]], [[1], [1, 2]]
    assert _kernel_value(s, [0.5, 0.5], P, D) == 0
    assert _kernel_value(s, [0.5, 0.1], P, D) == 0
    for x in xs:
        assert _kernel_value(s, [0.5, x], P, D) == 0
        assert _kernel_value(s, [x, delta], P, D) == 1
        assert _kernel_value(s, [delta, x], P, D) == 1
    # 3D, intersecting planes, plane + line, two lines meeting at an endpoint
    g = ina.named_comb_tree((3, 2))
    s = ina.continuous_siteinds(g, map_dimension=3)
    delta = 2.0 ** -(g.nv() // 3)
    xs, zs = [0.0, delta, 1 - delta], [0, delta, 0.5, 1 - delta]
    for P, D in (([[0.5], [0.5]], [[1], [2]]), ([[0.5], [0.5, 0]], [[1], [1, 2]])):
        for z in zs:
            assert _kernel_value(s, [0.5, 0.5, z], P, D) == 0
            for x in xs:
                if len(P[1]) == 1:  # two planes: the second one too
                    assert _kernel_value(s, [x, 0.5, z], P, D) == 0
                assert _kernel_value(s, [0.5, x, z], P, D) == 0
                assert _kernel_value(s, [x, delta, z], P, D) == 1
                assert _kernel_value(s, [delta, x, z], P, D) == 1
    P, D = [[0.5, 0], [0, 0.5]], [[2, 3], [1, 2]]
    assert _kernel_value(s, [0.0, 0.5, 0.5], P, D) == 0
    for x in xs:
        assert _kernel_value(s, [x, 0.5, 0], P, D) == 0
        assert _kernel_value(s, [x, delta, 0], P, D) == 1
        assert _kernel_value(s, [delta, x, 0], P, D) == 1


_NAMES = {(0.0, 1.0, 0.0, 0.0): "D+", (0.0, 0.0, 1.0, 0.0): "D-", (1.0, 0.0, 0.0, 0.0): "Ddn",
          (0.0, 0.0, 0.0, 1.0): "Dup"}


@pytest.mark.parametrize("weights,power", [([0.0, 0.5, 0.0, -0.5, 0.0], 1), ([0.0, 1.0, -2.0, 1.0, 0.0], 2),
                                           ([0.5, -1.0, 0.0, 1.0, -0.5], 3), ([1.0, -4.0, 6.0, -4.0, 1.0], 4)])
@pytest.mark.parametrize("left,right", [("Dirichlet", "Dirichlet"), ("Neumann", "Periodic"),
                                        ("Periodic", "Neumann")])
def test_library_stencil_terms_match_oracle(weights, power, left, right):
    """The carry-string terms the library builds its stencils from
    (tnfa_op_stencil_terms, no device involved) equal the oracle's
    (src/elementary_operators.jl:32-160) term by term, for variable 2 of a
    two-variable comb."""
    import itensornumericalanalysis as ina
    from itensornumericalanalysis import _lib
    from itensornumericalanalysis.network import topology_struct

    L = _lib.load()
    s = ina.continuous_siteinds(ina.named_comb_tree((2, 5)), map_dimension=2)
    t, _keep = topology_struct(s, [1] * s.layout.n)
    nlegs, ldim, lvar, ldig, lkind = s.leg_arrays()
    bc = {"Dirichlet": 0, "Neumann": 1, "Periodic": 2}
    w = (C.c_double * 5)(*weights)
    nt, nf = C.c_int32(0), C.c_int32(0)
    assert L.tnfa_op_stencil_terms(C.byref(t), 2, w, bc[left], bc[right], 0, 0, None, None, None, None,
                                   C.byref(nt), C.byref(nf)) == 0
    coefs = (C.c_double * nt.value)()
    nfac = (C.c_int32 * nt.value)()
    legs = (C.c_int32 * max(nf.value, 1))()
    mats = (C.c_double * max(4 * nf.value, 1))()
    assert L.tnfa_op_stencil_terms(C.byref(t), 2, w, bc[left], bc[right], nt, nf, coefs, nfac, legs, mats,
                                   C.byref(nt), C.byref(nf)) == 0
    got, k = [], 0
    for i in range(nt.value):
        ops = {}
        for _ in range(nfac[i]):
            ops[(lvar[legs[k]], ldig[legs[k]])] = _NAMES[tuple(mats[4 * k:4 * k + 4])]
            k += 1
        got.append((coefs[i], ops))
    Lv = s.ndigits(2)
    ref = O.stencil_terms(Lv, weights, power, dim=2, left=left, right=right, scale=False)
    assert len(got) == len(ref)
    for (cg, og), (cr, orf) in zip(got, ref):
        assert cg == cr and og == orf, ((cg, og), (cr, orf))


def test_library_stencil_terms_reject_bad_input():
    import itensornumericalanalysis as ina
    from itensornumericalanalysis import _lib
    from itensornumericalanalysis.network import topology_struct

    L = _lib.load()
    s = ina.continuous_siteinds(ina.named_path_graph(4))
    t, _keep = topology_struct(s, [1] * s.layout.n)
    w = (C.c_double * 5)(0.0, 1.0, -2.0, 1.0, 0.0)
    nt, nf = C.c_int32(0), C.c_int32(0)
    # variable 2 has no digits; a boundary code out of range
    assert L.tnfa_op_stencil_terms(C.byref(t), 2, w, 0, 0, 0, 0, None, None, None, None,
                                   C.byref(nt), C.byref(nf)) == _lib.ERR_INVALID_ARGUMENT
    assert L.tnfa_op_stencil_terms(C.byref(t), 1, w, 7, 0, 0, 0, None, None, None, None,
                                   C.byref(nt), C.byref(nf)) == _lib.ERR_INVALID_ARGUMENT


def test_complex_map_legs_match_oracle():
    """The product's complex maps carry, vertex by vertex, the same (variable,
    digit, real/imaginary) legs in the same order as the oracle's
    complex_siteinds (src/digit_inds.jl:88-115), for default and explicit
    vertex lists."""
    import itensornumericalanalysis as ina

    cases = [(ina.named_comb_tree((2, 3)), O.comb_tree_graph((2, 3)), None, None, 1),
             (ina.named_comb_tree((2, 3)), O.comb_tree_graph((2, 3)), [[(1, 1), (1, 2), (1, 3)]],
              [[(2, 1), (2, 2), (2, 3)]], 1),
             (ina.named_grid((3, 2)), O.grid_graph((3, 2)), None, None, 2)]
    for g, og, rdv, idv, md in cases:
        s = ina.complex_continuous_siteinds(g, rdv, idv, map_dimension=md)
        so = O.complex_siteinds(og, rdv, idv, map_dimension=md)
        for v in g.vertices():
            mine = [(l.dim, l.digit, l.kind == "real") for l in s.inds(v)]
            theirs = [so.info[i] for i in so.site[v]]
            assert mine == theirs, (v, mine, theirs)

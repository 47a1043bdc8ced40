"""The operator builders of the C ABI (tnfa_op_build_stencil,
tnfa_op_from_terms) called through ctypes as a foreign caller would, against
the oracle's dense stencil operators (src/elementary_operators.jl:32-189) and
against the same terms assembled on the host."""
import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

STENCILS = [
    ([0.0, 0.5, 0.0, -0.5, 0.0], 1),   # first derivative (:162-164)
    ([0.0, 1.0, -2.0, 1.0, 0.0], 2),   # second (:166-168)
    ([0.5, -1.0, 0.0, 1.0, -0.5], 3),  # third (:170-172)
    ([1.0, -4.0, 6.0, -4.0, 1.0], 4),  # fourth (:174-176)
]
BCS = {"Dirichlet": 0, "Neumann": 1, "Periodic": 2}


def _abi_stencil(ina, s, weights, power, dim=1, left="Dirichlet", right="Dirichlet", scale=True,
                 cutoff=1e-15):
    from itensornumericalanalysis.elementary_operators import ITensorNetworkOperator, operator_legs
    from itensornumericalanalysis.network import topology_struct

    L = ina._lib
    ctx = L.default_context()
    t, _keep = topology_struct(s, [1] * s.layout.n)
    h = C.c_void_p()
    w = (C.c_double * 5)(*weights)
    ctx.call("tnfa_op_build_stencil", C.byref(t), dim, w, power, BCS[left], BCS[right], int(scale),
             cutoff, C.byref(h))
    return ITensorNetworkOperator(s, h, ctx, operator_legs(s))


@pytest.mark.parametrize("weights,power", STENCILS)
@pytest.mark.parametrize("left,right", [("Dirichlet", "Dirichlet"), ("Neumann", "Periodic"),
                                        ("Periodic", "Neumann")])
def test_abi_stencil_matches_dense(ina, weights, power, left, right):
    """The stencil built by the library applied to a random function on a
    3 x 3 comb (9 digits) equals the oracle's dense stencil on the 2^9 grid."""
    Lb = 9
    s = ina.continuous_siteinds(ina.named_comb_tree((3, 3)))
    f = ina.rand_itn(s, link_space=3, rng=90)
    op = _abi_stencil(ina, s, weights, power, left=left, right=right)
    g1 = ina.operate(op, f, cutoff=0.0)
    xs = np.arange(2**Lb) / 2.0**Lb
    F = f.evaluate_batch(xs)
    terms = O.stencil_terms(Lb, weights, power, left=left, right=right)
    G = O.apply_terms_dense(terms, F.reshape((2,) * Lb), {(1, k): k - 1 for k in range(1, Lb + 1)})
    G = G.reshape(-1)
    assert np.max(np.abs(g1.evaluate_batch(xs) - G)) <= 1e-10 * np.max(np.abs(G))


def test_abi_stencil_second_variable_unscaled(ina):
    """Variable 2 of a two-variable map, scale off: only variable 2 moves."""
    Lb = 4
    s = ina.continuous_siteinds(ina.named_path_graph(2 * Lb), map_dimension=2)
    f = ina.rand_itn(s, link_space=2, rng=91)
    op = _abi_stencil(ina, s, [0.0, 1.0, -2.0, 1.0, 0.0], 2, dim=2, scale=False)
    g1 = ina.operate(op, f, cutoff=0.0)
    xs = np.arange(2**Lb) / 2.0**Lb
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    P = np.stack([X.ravel(), Y.ravel()], axis=1)
    F = f.evaluate_batch(P, [1, 2]).reshape(2**Lb, 2**Lb)
    G = np.zeros_like(F)
    G += -2.0 * F
    G[:, :-1] += F[:, 1:]  # f(x, y + d), Dirichlet
    G[:, 1:] += F[:, :-1]  # f(x, y - d)
    got = g1.evaluate_batch(P, [1, 2]).reshape(2**Lb, 2**Lb)
    assert np.max(np.abs(got - G)) <= 1e-11 * np.max(np.abs(G))


def test_abi_terms_match_host_assembly(ina):
    """tnfa_op_from_terms on random real terms (digit operators and explicit
    2 x 2 matrices, more than one 64-term block) against the same terms
    assembled on the host and compressed on the device."""
    from itensornumericalanalysis import elementary_operators as E
    from itensornumericalanalysis.truncation import truncate

    rng = np.random.default_rng(92)
    s = ina.continuous_siteinds(ina.named_binary_tree(7))
    names = ["I", "D+", "D-", "Dup", "Ddn"]
    os_ = E.OpSum()
    for _ in range(150):
        ops = {}
        for k in rng.choice(7, size=rng.integers(1, 4), replace=False):
            ops[(1, int(k) + 1)] = (names[rng.integers(5)] if rng.random() < 0.6
                                    else rng.standard_normal((2, 2)))
        os_.add(float(rng.standard_normal()), ops)
    native = E.opsum_to_operator(s, os_, cutoff=1e-14)
    host = None
    for b0 in range(0, len(os_.terms), 64):
        part = truncate(E._direct_sum(s, os_.terms[b0:b0 + 64]), cutoff=1e-14)
        host = part if host is None else truncate(host + part, cutoff=1e-14)
    f = ina.rand_itn(s, link_space=3, rng=93)
    xs = np.arange(2**7) / 2.0**7
    a = ina.operate(native, f, cutoff=0.0).evaluate_batch(xs)
    b = ina.operate(host, f, cutoff=0.0).evaluate_batch(xs)
    assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b))


def test_abi_builders_reject_bad_input(ina):
    L = ina._lib
    s = ina.continuous_siteinds(ina.named_path_graph(5))
    with pytest.raises(ina.TnfaError) as e:
        _abi_stencil(ina, s, [0.0, 1.0, -2.0, 1.0, 0.0], 2, dim=3)
    assert e.value.status == L.ERR_INVALID_ARGUMENT
    from itensornumericalanalysis.network import topology_struct

    ctx = L.default_context()
    t, _keep = topology_struct(s, [1] * s.layout.n)
    h = C.c_void_p()
    one = (C.c_double * 1)(1.0)
    nf = (C.c_int32 * 1)(1)
    leg = (C.c_int32 * 1)(99)
    m = (C.c_double * 4)(1.0, 0.0, 0.0, 1.0)
    with pytest.raises(ina.TnfaError) as e:
        ctx.call("tnfa_op_from_terms", C.byref(t), 1, one, nf, leg, m, 1e-14, C.byref(h))
    assert "leg out of range" in str(e.value)

"""The device path reproduces the committed golden fixtures (tests/golden/)."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
G = Path(__file__).resolve().parent / "golden"


def test_random_tree_fixture(ina):
    d = np.load(G / "random_binary15_chi4.npz")
    s = ina.continuous_siteinds(ina.named_binary_tree(15), map_dimension=3)
    flat, ts, off = d["tensors"], {}, 0
    for v, sh in zip(s.layout.order, d["shapes"]):
        sh = tuple(int(x) for x in sh if x > 0)
        n = int(np.prod(sh))
        ts[v] = flat[off:off + n].reshape(sh)
        off += n
    f = ina.ITensorNetworkFunction.from_tensors(s, ts)
    got = f.evaluate_batch(d["X"], [1, 2, 3])
    assert np.max(np.abs(got - d["values"])) <= 1e-12 * np.max(np.abs(d["values"]))
    assert abs(f.integrate() - d["integral"]) <= 1e-12 * abs(d["integral"])
    assert abs(f.integrate(take_sum=True) - d["integral_sum"]) <= 1e-12 * abs(d["integral_sum"])


def test_config1_fixture(ina):
    d = np.load(G / "config1_path12.npz")
    s = ina.continuous_siteinds(ina.named_grid((12, 1)))
    f = ina.exp_itn(s, k=-1.0) + ina.sin_itn(s, k=2 * np.pi)
    assert np.max(np.abs(f.evaluate_batch(d["X"]) - d["f"])) < 1e-12
    op = ina.second_derivative_operator(s)
    scale = np.max(np.abs(d["d2f_grid"]))
    xs = np.arange(2**12) / 2**12
    # cutoff 0: the exact product, up to rounding
    g = ina.operate(op, f, cutoff=0.0)
    assert np.max(np.abs(g.evaluate_batch(d["X"]) - d["d2f"])) / scale < 1e-10
    assert np.max(np.abs(g.evaluate_batch(xs) - d["d2f_grid"])) / scale < 1e-10
    assert abs(ina.integrate(g) - d["integral_d2f"]) / scale < 1e-10
    # cutoff 1e-15: each bond may drop sqrt(1e-15) of the 2-norm
    gt = ina.operate(op, f, cutoff=1e-15)
    err = np.linalg.norm(gt.evaluate_batch(xs) - d["d2f_grid"])
    assert err <= 11 * np.sqrt(1e-15) * np.linalg.norm(d["d2f_grid"])


@pytest.mark.parametrize("boundary", ["Dirichlet", "Periodic", "Neumann"])
@pytest.mark.parametrize("n", [0, 1])
def test_shift_fixture(ina, boundary, n):
    d = np.load(G / "shifts_comb2x3_poly.npz")
    s = ina.continuous_siteinds(ina.named_comb_tree((2, 3)))
    f = ina.poly_itn(s, [1.0, 0.5, 0.25])
    xs = np.arange(64) / 64
    for fwd in (True, False):
        mk = ina.forward_shift_op if fwd else ina.backward_shift_op
        g = ina.operate(mk(s, boundary=boundary, n=n), f, cutoff=1e-14)
        key = f"{'fwd' if fwd else 'bwd'}_{boundary}_{n}"
        assert np.max(np.abs(g.evaluate_batch(xs) - d[key])) < 1e-10


def test_complex_fixture(ina):
    d = np.load(G / "complex_cosh_comb2x3.npz")
    g = ina.named_comb_tree((2, 3))
    s = ina.complex_continuous_siteinds(g, [[(1, 1), (1, 2), (1, 3)]], [[(2, 1), (2, 2), (2, 3)]])
    f = ina.cosh_itn(s, k=complex(d["k"]), a=complex(d["a"]), c=complex(d["c"]))
    got = f.evaluate_batch(d["Z"].reshape(-1, 1))
    assert np.max(np.abs(got - d["values"])) <= 1e-12 * np.max(np.abs(d["values"]))


def _fixture_net(ina, d, s):
    flat, ts, off = d["tensors"], {}, 0
    for v, sh in zip(s.layout.order, d["shapes"]):
        sh = tuple(int(x) for x in sh if x > 0)
        n = int(np.prod(sh))
        ts[v] = flat[off:off + n].reshape(sh)
        off += n
    return ina.ITensorNetworkFunction.from_tensors(s, ts)


def test_partial_fixture(ina):
    d = np.load(G / "partial_comb3x3_chi3.npz")
    s = ina.continuous_siteinds(ina.named_comb_tree((3, 3)), map_dimension=3)
    f = _fixture_net(ina, d, s)
    g = np.arange(8) / 8.0
    mesh = lambda k: np.stack(np.meshgrid(*([g] * k), indexing="ij"), axis=-1).reshape(-1, k)
    cases = [([2], [1, 3], d["p2"], False), ([2, 3], [1], d["p23"], False),
             ([1, 3], [2], d["p13"], False), ([1], [2, 3], d["p1_sum"], True)]
    for dims, keep, ref, take_sum in cases:
        h = ina.partial_integrate(f, dims, take_sum=take_sum)
        got = h.evaluate_batch(mesh(len(keep)), keep)
        assert np.max(np.abs(got - ref.reshape(-1))) <= 1e-12 * np.max(np.abs(ref)), dims


def test_linsolve_fixture(ina):
    d = np.load(G / "linsolve_path9.npz")
    L = 9
    s = ina.continuous_siteinds(ina.named_grid((L, 1)))
    b = _fixture_net(ina, d, s)
    xs = np.arange(2**L) / 2.0**L
    assert np.max(np.abs(b.evaluate_batch(xs) - d["b_grid"])) <= 1e-12 * np.max(np.abs(d["b_grid"]))
    x = ina.linsolve(ina.second_derivative_operator(s), b, nsweeps=4, cutoff=0.0, tol=1e-13)
    ref = d["x_grid"]
    # forward error <= cond * residual; cond ~ 1e5 here
    assert np.max(np.abs(x.evaluate_batch(xs) - ref)) <= 1e-9 * np.max(np.abs(ref))
    assert x.rel_residual < 1e-12

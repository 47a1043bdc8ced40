"""Linear solve by two-site sweeps on the GPU, against a dense FP64 solve with
the oracle's operator matrix (the finite-difference stencils of
src/elementary_operators.jl:122-189 written out as dense digit operators)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _dense_operator(terms, n_sites, axis_of):
    """The operator matrix M[i, j] on the 2^n_sites grid (row-major digits)."""
    N = 2**n_sites
    eye = np.eye(N).reshape((2,) * n_sites + (N,))
    return O.apply_terms_dense(terms, eye, axis_of).reshape(N, N)


def _grid_1d(L):
    return np.arange(2**L) / 2.0**L


def _grid_2d(L):
    g = _grid_1d(L)
    X, Y = np.meshgrid(g, g, indexing="ij")
    return np.stack([X.ravel(), Y.ravel()], axis=1)


def _check(M, a0, a1, bv, xv, rel_residual):
    K = a0 * np.eye(M.shape[0]) + a1 * M
    ref = np.linalg.solve(K, bv)
    err = np.linalg.norm(xv - ref) / np.linalg.norm(ref)
    res = np.linalg.norm(K @ xv - bv) / np.linalg.norm(bv)
    return err, res


def test_second_derivative_path(ina):
    """d2/dx2 x = b on a 9-bit path with Dirichlet boundaries."""
    L = 9
    s = ina.continuous_siteinds(ina.named_path_graph(L))
    b = ina.rand_itn(s, link_space=2, rng=70)
    A = ina.second_derivative_operator(s)
    x = ina.linsolve(A, b, nsweeps=4, cutoff=1e-15, tol=1e-12)
    M = _dense_operator(O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2), L,
                        {(1, k): k - 1 for k in range(1, L + 1)})
    xs = _grid_1d(L)
    err, res = _check(M, 0.0, 1.0, b.evaluate_batch(xs), x.evaluate_batch(xs), x.rel_residual)
    assert err < 1e-9, err
    assert res < 1e-11, res
    assert x.rel_residual < 1e-11
    # the reported residual is the dense one up to rounding
    assert abs(x.rel_residual - res) < 1e-11 + 1e-3 * res


def test_large_local_systems(ina):
    """A 12-bit path with a random right-hand side of full rank: the middle
    two-site systems reach 32 x 2 x 2 x 32 = 4096 unknowns, so the dense LU
    runs its global-memory panels (more than 1600 rows left), its 16-column
    shared-memory panels (801-1600) and its 32-column ones (800 or fewer)."""
    L = 12
    s = ina.continuous_siteinds(ina.named_path_graph(L))
    b = ina.truncate(ina.rand_itn(s, link_space=64, rng=78), cutoff=0.0)  # bonds at full rank
    A = ina.second_derivative_operator(s)
    a0, a1 = 1.0, -1e-6  # (1 - 1e-6 d2/dx2): condition number ~ 70
    x = ina.linsolve(A, b, b, a0=a0, a1=a1, nsweeps=2, maxdim=64, cutoff=0.0, tol=0.0)
    assert x.maxlinkdim() == 64
    M = _dense_operator(O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2), L,
                        {(1, k): k - 1 for k in range(1, L + 1)})
    xs = _grid_1d(L)
    err, res = _check(M, a0, a1, b.evaluate_batch(xs), x.evaluate_batch(xs), x.rel_residual)
    assert res < 1e-11, res
    assert err < 1e-10, err


@pytest.mark.parametrize("a0,a1", [(0.0, 1.0), (1.0, -1e-3), (2.0, 0.5)])
def test_laplacian_comb(ina, a0, a1):
    """(a0 + a1 Laplacian) u = b on a 2 x 5 comb (a 10-site path whose layout
    root sits mid-path), x0 random."""
    L = 5
    g = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g, [[(1, j) for j in range(L, 0, -1)],
                                    [(2, j) for j in range(1, L + 1)]])
    b = ina.rand_itn(s, link_space=3, rng=71)
    x0 = ina.rand_itn(s, link_space=2, rng=72)
    A = ina.laplacian_operator(s)
    # no truncation: any discarded weight is amplified by ||A|| in the residual
    x = ina.linsolve(A, b, x0, a0=a0, a1=a1, nsweeps=6, cutoff=0.0, tol=1e-12)
    terms = (O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2, dim=1)
             + O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2, dim=2))
    axis_of = {(1, k): k - 1 for k in range(1, L + 1)}
    axis_of.update({(2, k): L + k - 1 for k in range(1, L + 1)})
    M = _dense_operator(terms, 2 * L, axis_of)
    X = _grid_2d(L)
    err, res = _check(M, a0, a1, b.evaluate_batch(X, [1, 2]), x.evaluate_batch(X, [1, 2]),
                      x.rel_residual)
    # forward error <= cond(K) * residual; cond(K) is up to ~500 here
    assert res < 1e-10, (res, x.rel_residual)
    assert err < 1e-7, (err, res)
    assert abs(x.rel_residual - res) < 1e-11 + 1e-3 * res


def test_poisson_sine_source(ina):
    """Laplacian u = sin(pi x) sin(pi y) (the Laplace workload's source term)
    on a 2 x 6 comb: the solution tracks -sin(pi x) sin(pi y) / (2 pi^2) up to
    the discretisation error, and the bond dimension stays small."""
    L = 6
    g = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g, [[(1, j) for j in range(L, 0, -1)],
                                    [(2, j) for j in range(1, L + 1)]])
    b = ina.sin_itn(s, k=np.pi, dim=1) * ina.sin_itn(s, k=np.pi, dim=2)
    A = ina.laplacian_operator(s)
    x = ina.linsolve(A, b, nsweeps=6, maxdim=16, cutoff=1e-24, tol=1e-10)
    assert x.rel_residual < 1e-9
    X = _grid_2d(L)
    exact = -np.sin(np.pi * X[:, 0]) * np.sin(np.pi * X[:, 1]) / (2 * np.pi**2)
    got = x.evaluate_batch(X, [1, 2])
    # O(h) boundary error (the grid's left Dirichlet node sits at x = -h)
    assert np.max(np.abs(got - exact)) < 0.05 * np.max(np.abs(exact))
    assert x.maxlinkdim() <= 16


def test_refinement_lowers_residual(ina):
    """Iterative refinement on the 1/h^2 Laplacian (2 x 8 bits): one step takes
    the residual left by the truncated sweep down by orders of magnitude."""
    L = 8
    g = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g, [[(1, j) for j in range(L, 0, -1)],
                                    [(2, j) for j in range(1, L + 1)]])
    b = ina.sin_itn(s, k=np.pi, dim=1) * ina.sin_itn(s, k=np.pi, dim=2)
    A = ina.laplacian_operator(s)
    x0 = ina.linsolve(A, b, nsweeps=2, maxdim=24, cutoff=1e-20, tol=0.0)
    x1 = ina.linsolve(A, b, nsweeps=2, maxdim=24, cutoff=1e-20, tol=0.0, refinements=2)
    assert x1.rel_residual < 1e-2 * x0.rel_residual, (x0.rel_residual, x1.rel_residual)
    assert x1.rel_residual < 1e-8


def test_maxdim_caps_solution(ina):
    L = 8
    s = ina.continuous_siteinds(ina.named_path_graph(L))
    b = ina.rand_itn(s, link_space=6, rng=73)
    A = ina.second_derivative_operator(s)
    x = ina.linsolve(A, b, nsweeps=2, maxdim=3, cutoff=0.0, tol=0.0)
    assert x.maxlinkdim() <= 3
    assert np.isfinite(x.rel_residual) and x.rel_residual > 0


@pytest.mark.parametrize("a0,a1", [(0.0, 1.0), (1.0, -1e-3)])
def test_linsolve_binary_tree(ina, a0, a1):
    """(a0 + a1 d2/dx2) x = b on a 7-vertex binary tree (the root has two
    children, so the sweep is the tree tour, not the path one), against the
    dense solve."""
    L = 7
    s = ina.continuous_siteinds(ina.named_binary_tree(L))
    b = ina.rand_itn(s, link_space=2, rng=74)
    A = ina.second_derivative_operator(s)
    x = ina.linsolve(A, b, a0=a0, a1=a1, nsweeps=6, cutoff=0.0, tol=1e-12)
    M = _dense_operator(O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2), L,
                        {(1, k): k - 1 for k in range(1, L + 1)})
    xs = _grid_1d(L)
    err, res = _check(M, a0, a1, b.evaluate_batch(xs), x.evaluate_batch(xs), x.rel_residual)
    assert res < 1e-10, (res, x.rel_residual)
    assert err < 1e-8, err
    assert abs(x.rel_residual - res) < 1e-11 + 1e-3 * res


def _random_tree_laplacian(ina, n_vertices, seed):
    """A uniformly random labelled tree with one digit per vertex and two
    variables (continuous_siteinds(g; map_dimension=2)), and the dense
    unscaled Laplacian on its 2^n grid."""
    g = ina.uniform_tree(n_vertices, seed)
    s = ina.continuous_siteinds(g, map_dimension=2)
    L = n_vertices // 2
    terms = (O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2, dim=1, scale=False)
             + O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2, dim=2, scale=False))
    axis_of = {(1, k): k - 1 for k in range(1, L + 1)}
    axis_of.update({(2, k): L + k - 1 for k in range(1, L + 1)})
    return g, s, _dense_operator(terms, 2 * L, axis_of), L


def test_dmrg_random_tree_laplace_example(ina):
    """examples/2d_laplace_solver.jl: a random tree of 12 vertices
    (uniform_tree(12)), two variables, the unscaled Laplacian, two-site DMRG
    with maxdim 30 from a random start.  The energy is the lowest eigenvalue
    of the dense stencil matrix and the state its eigenvector."""
    g, s, M, L = _random_tree_laplacian(ina, 12, 1234)
    assert max(len(list(g.neighbors(v))) for v in g.vertices()) >= 3  # not a path
    A = ina.laplacian_operator(s, scale=False)
    psi0 = ina.rand_itn(s, link_space=3, rng=80)
    E, psi = ina.dmrg(A, psi0, nsweeps=15, maxdim=30, cutoff=1e-12)
    w, V = np.linalg.eigh((M + M.T) / 2)
    assert abs(E - w[0]) < 1e-8 * abs(w[0]), (E, w[:3])
    v = psi.evaluate_batch(_grid_2d(L), [1, 2])
    assert abs(abs(v @ V[:, 0]) / np.linalg.norm(v) - 1) < 1e-7
    assert psi.maxlinkdim() <= 30


def test_linsolve_random_tree(ina):
    """(1 - 0.05 Laplacian) x = b on a random 10-vertex tree, against the dense
    solve."""
    g, s, M, L = _random_tree_laplacian(ina, 10, 7)
    b = ina.rand_itn(s, link_space=2, rng=81)
    A = ina.laplacian_operator(s, scale=False)
    x = ina.linsolve(A, b, a0=1.0, a1=-0.05, nsweeps=8, cutoff=0.0, tol=1e-12)
    X = _grid_2d(L)
    err, res = _check(M, 1.0, -0.05, b.evaluate_batch(X, [1, 2]), x.evaluate_batch(X, [1, 2]),
                      x.rel_residual)
    assert res < 1e-10, (res, x.rel_residual)
    assert err < 1e-9, err


def test_dmrg_lowest_laplacian_mode(ina):
    """examples/2d_laplace_solver.jl on a 2 x 5 comb: DMRG finds the lowest
    eigenpair of the unscaled Laplacian (eigenvalues of the dense stencil
    matrix; the most negative one is approached as the grid grows)."""
    L = 5
    g = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g, [[(1, j) for j in range(L, 0, -1)],
                                    [(2, j) for j in range(1, L + 1)]])
    A = ina.laplacian_operator(s, scale=False)
    psi0 = ina.rand_itn(s, link_space=3, rng=75)
    E, psi = ina.dmrg(A, psi0, nsweeps=8, maxdim=32, cutoff=1e-14)
    terms = (O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2, dim=1, scale=False)
             + O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2, dim=2, scale=False))
    axis_of = {(1, k): k - 1 for k in range(1, L + 1)}
    axis_of.update({(2, k): L + k - 1 for k in range(1, L + 1)})
    M = _dense_operator(terms, 2 * L, axis_of)
    w, V = np.linalg.eigh((M + M.T) / 2)
    assert abs(E - w[0]) < 1e-9 * abs(w[0]), (E, w[:3])
    v = psi.evaluate_batch(_grid_2d(L), [1, 2])
    assert abs(abs(v @ V[:, 0]) / np.linalg.norm(v) - 1) < 1e-8


_MATFREE_SCRIPT = r"""
import json, sys
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[2]); sys.path.insert(0, sys.argv[3])
import numpy as np
import itensornumericalanalysis as ina
import oracle as O
from test_gpu_linsolve import _dense_operator, _grid_2d, _check
L = 4
g = ina.named_comb_tree((2, L))
s = ina.continuous_siteinds(g, [[(1, j) for j in range(L, 0, -1)], [(2, j) for j in range(1, L + 1)]])
terms = (O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2, dim=1)
         + O.stencil_terms(L, [0.0, 1.0, -2.0, 1.0, 0.0], 2, dim=2))
axis_of = {(1, k): k - 1 for k in range(1, L + 1)}
axis_of.update({(2, k): L + k - 1 for k in range(1, L + 1)})
M = _dense_operator(terms, 2 * L, axis_of)
A = ina.laplacian_operator(s)
b = ina.rand_itn(s, link_space=2, rng=76)
x = ina.linsolve(A, b, a0=1.0, a1=-1e-3, nsweeps=4, cutoff=0.0, tol=1e-12)
err, res = _check(M, 1.0, -1e-3, b.evaluate_batch(_grid_2d(L), [1, 2]), x.evaluate_batch(_grid_2d(L), [1, 2]), 0)
Au = ina.laplacian_operator(s, scale=False)
E, psi = ina.dmrg(Au, ina.rand_itn(s, link_space=3, rng=77), nsweeps=6, maxdim=32, cutoff=1e-14)
Mu = _dense_operator([(c / 4.0**L, o) for c, o in terms], 2 * L, axis_of)
w = np.linalg.eigvalsh((Mu + Mu.T) / 2)
print(json.dumps({"lin_err": err, "lin_res": res, "E": E, "E_ref": float(w[0])}))
"""


def test_matrix_free_two_site_paths(ina):
    """The matrix-free two-site operator (GMRES for linsolve, Lanczos for
    dmrg), forced at every size, gives the dense answers."""
    import json
    import os
    import subprocess
    import sys
    from pathlib import Path
    here = Path(__file__).resolve().parent
    env = dict(os.environ, TNFA_LOCAL_MATRIX_FREE="1")
    r = subprocess.run([sys.executable, "-c", _MATFREE_SCRIPT, str(here.parent / "itensornumericalanalysis.jl_gb300"),
                        str(here.parent), str(here)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["lin_res"] < 1e-9 and out["lin_err"] < 1e-9, out
    assert abs(out["E"] - out["E_ref"]) < 1e-9 * abs(out["E_ref"]), out


def test_laplace_residual_is_at_its_fp64_floor_2x12(ina):
    """The Laplace workload at 2 x 12 bits (the 1/h^2 Laplacian, source
    sin(pi x) sin(pi y)): the residual tnfa_linsolve reports equals the true
    residual of the stored solution, measured on the dense 4096 x 4096 grid
    in extended precision, and sits within a small factor of the FP64 floor
    eps || |A| |x| || / ||b|| that rounding x to FP64 alone causes.  The same
    floor, computed on the networks, is what bench.py reports at 2 x 16 bits,
    where it lies above the 1e-8 the workload asks for."""
    L = 12
    g = ina.named_comb_tree((2, L))
    s = ina.continuous_siteinds(g, [[(1, j) for j in range(L, 0, -1)],
                                    [(2, j) for j in range(1, L + 1)]])
    b = ina.sin_itn(s, k=np.pi, dim=1) * ina.sin_itn(s, k=np.pi, dim=2)
    A = ina.laplacian_operator(s)
    x = ina.linsolve(A, b, nsweeps=2, maxdim=40, cutoff=1e-20, tol=1e-12, refinements=3)
    n = 2**L
    P = _grid_2d(L)
    X = x.evaluate_batch(P, [1, 2]).reshape(n, n)
    B = b.evaluate_batch(P, [1, 2]).reshape(n, n)
    # A X - B with Dirichlet zeros outside the grid, in extended precision
    # (the factor 4^L is a power of two: exact)
    Xl = X.astype(np.longdouble)
    AX = -4.0 * Xl
    AX[1:, :] += Xl[:-1, :]
    AX[:-1, :] += Xl[1:, :]
    AX[:, 1:] += Xl[:, :-1]
    AX[:, :-1] += Xl[:, 1:]
    AX *= np.longdouble(4.0) ** L
    res_true = float(np.sqrt(np.sum((AX - B.astype(np.longdouble)) ** 2) / np.sum(B.astype(np.longdouble) ** 2)))
    aX = np.abs(X)
    absAX = 4.0 * aX
    absAX[1:, :] += aX[:-1, :]
    absAX[:-1, :] += aX[1:, :]
    absAX[:, 1:] += aX[:, :-1]
    absAX[:, :-1] += aX[:, 1:]
    absAX *= 4.0**L
    floor_dense = 2.0**-53 * np.linalg.norm(absAX) / np.linalg.norm(B)
    # the floor on the networks (what bench.py computes at 16 bits)
    absA = None
    for d in (1, 2):
        op = ina.stencil(s, [0.0, 1.0, 2.0, 1.0, 0.0], 2, dim=d)
        absA = op if absA is None else absA + op
    floor_net = 2.0**-53 * ina.operate(absA, x, cutoff=0.0).norm() / b.norm()
    assert abs(floor_net - floor_dense) <= 1e-3 * floor_dense, (floor_net, floor_dense)
    # the dense values come from an FP64 evaluation of the network, whose own
    # rounding is of the order of the floor
    assert abs(x.rel_residual - res_true) <= 0.5 * res_true + 2.0 * floor_dense, (x.rel_residual, res_true)
    assert res_true <= 30.0 * floor_dense, (res_true, floor_dense)

"""Tensor cross interpolation: the cross (host) part on CPU."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "itensornumericalanalysis.jl_gb300"))
from itensornumericalanalysis.tci import _aca_full, tci_path  # noqa: E402


def _mps_values(cores, idx):
    out = np.ones((idx.shape[0], 1))
    for l, A in enumerate(cores):
        out = np.einsum("pa,pab->pb", out, A[:, idx[:, l], :].transpose(1, 0, 2))
    return out[:, 0]


def _bits_to_x(idx):
    L = idx.shape[1]
    return idx @ (2.0 ** -np.arange(1, L + 1))


def test_aca_recovers_low_rank():
    rng = np.random.default_rng(1)
    M = rng.standard_normal((30, 3)) @ rng.standard_normal((3, 40))
    rows, cols, err, scale = _aca_full(M, 1e-12, 10)
    assert len(rows) == 3 and err <= 1e-10 * scale
    # the cross reproduces M
    C, R, P = M[:, cols], M[rows, :], M[np.ix_(rows, cols)]
    assert np.allclose(C @ np.linalg.solve(P, R), M, atol=1e-10)


def test_tci_1d_smooth_function():
    L = 24
    f = lambda x: np.exp(-x) * np.sin(20 * x) + x**2
    sample = lambda idx: f(_bits_to_x(idx))
    cores, info = tci_path(sample, [2] * L, tol=1e-12, maxbonddim=32)
    rng = np.random.default_rng(2)
    idx = rng.integers(0, 2, (2000, L))
    err = np.max(np.abs(_mps_values(cores, idx) - sample(idx)))
    assert err < 1e-9, (err, info)
    assert max(info["ranks"]) <= 12, info["ranks"]


def test_tci_exact_low_rank_2d():
    """exp(x y) on interleaved digits is not low rank exactly, but
    cos(x + y) = cos x cos y - sin x sin y has rank 2 across the split."""
    L = 10
    f = lambda x, y: np.cos(3 * x + 2 * y)
    def sample(idx):
        return f(_bits_to_x(idx[:, :L]), _bits_to_x(idx[:, L:][:, ::-1]))
    cores, info = tci_path(sample, [2] * (2 * L), tol=1e-12, maxbonddim=16)
    idx = np.random.default_rng(3).integers(0, 2, (1000, 2 * L))
    assert np.max(np.abs(_mps_values(cores, idx) - sample(idx))) < 1e-10
    assert info["ranks"][L - 1] == 2

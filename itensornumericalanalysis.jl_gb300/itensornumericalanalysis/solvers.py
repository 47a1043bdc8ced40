"""Linear solve on tree tensor networks.

The reference hands its solver sweeps to ITensorNetworks (``dmrg`` in
examples/2d_laplace_solver.jl:33-34, and ``linsolve`` with the signature
``linsolve(A, b, x0; nsweeps, ...)`` solving ``(a0 + a1 A) x = b``); here the
sweep runs in libtnfa (tnfa_linsolve).
"""
from __future__ import annotations

import ctypes as C

from . import _lib
from .truncation import PRECISIONS


def linsolve(A, b, x0=None, a0: float = 0.0, a1: float = 1.0, nsweeps: int = 10,
             maxdim: int | None = None, cutoff: float = 1e-14, tol: float = 1e-10,
             krylov_dim: int = 0, precision: str = "f64", refinements: int = 0,
             refine_cutoff: float = 1e-28):
    """Solve (a0 + a1 A) x = b for x, A an ITensorNetworkOperator and b an
    ITensorNetworkFunction on the same tree (one site leg per vertex).

    Two-site alternating sweeps: each update solves the system projected onto
    the environments of the other edges and splits the two-site solution by
    an SVD truncated with ``cutoff`` / ``maxdim``.  On a path (a comb of two
    dimensions is one) the sweep runs left to right and back and the local
    system is solved densely on the device (FP64 LU with partial pivoting) or
    matrix-free by GMRES when large; on any other tree the orthogonality
    centre walks a depth-first tour from the root (every edge updated on the
    way down and on the way back) and each two-site system is solved
    matrix-free by GMRES.  Sweeps stop after ``nsweeps`` or as soon as
    ||(a0 + a1 A) x - b|| / ||b|| <= tol; that residual, evaluated exactly in
    FP64, is stored on the result as ``x.rel_residual``.  ``x0`` (default b)
    seeds the sweep.

    ``refinements`` > 0 adds iterative refinement: the residual b - (a0 +
    a1 A) x is formed exactly, truncated with ``refine_cutoff``, the same
    sweeps solve for a correction, and x + correction is truncated with
    ``refine_cutoff`` again -- for ill-conditioned operators (the 1/h^2
    Laplacian) this recovers the digits the sweep's own truncation loses.
    """
    if x0 is None:
        x0 = b
    p = _lib.LinsolveParams(int(nsweeps), int(maxdim or 0), float(cutoff), float(tol),
                            int(krylov_dim), PRECISIONS[precision], float(a0), float(a1),
                            int(refinements), float(refine_cutoff))
    h = C.c_void_p()
    res = C.c_double(0.0)
    b.ctx.call("tnfa_linsolve", A.handle, b.handle, x0.handle, C.byref(p), C.byref(h),
               C.byref(res))
    x = b._wrap(h)
    x.rel_residual = float(res.value)
    return x


def dmrg(H, psi0, nsweeps: int = 10, maxdim: int | None = None, cutoff: float = 1e-12,
         tol: float = 1e-12, krylov_dim: int = 30, restarts: int = 4, nsites: int = 2,
         normalize: bool = True):
    """Lowest eigenpair of the symmetric operator H, (energy, psi), by two-site
    DMRG sweeps from psi0 on any tree with one site leg per vertex
    (examples/2d_laplace_solver.jl calls ITensorNetworks.dmrg with nsites = 2
    and normalize = true on a uniform random tree; those are the only modes
    here).  Lanczos with full re-orthogonalisation finds the lowest
    eigenvector of the two-site operator (built densely on the device for
    small systems on a path, applied matrix-free otherwise); the split is an
    SVD truncated with cutoff / maxdim.  On trees that are not paths the
    orthogonality centre walks a depth-first tour of the edges."""
    if nsites != 2 or not normalize:
        raise ValueError("dmrg: nsites = 2 with normalize = True only")
    p = _lib.DmrgParams(int(nsweeps), int(maxdim or 0), float(cutoff), float(tol), int(krylov_dim),
                        int(restarts))
    h = C.c_void_p()
    e = C.c_double(0.0)
    psi0.ctx.call("tnfa_dmrg", H.handle, psi0.handle, C.byref(p), C.byref(h), C.byref(e))
    return float(e.value), psi0._wrap(h)

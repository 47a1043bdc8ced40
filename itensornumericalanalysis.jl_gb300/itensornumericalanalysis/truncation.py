"""Truncation of tree tensor networks (mirrors src/itensornetworkfunction.jl:114-118)."""
from __future__ import annotations

import ctypes as C

from . import _lib

PRECISIONS = {"f64": _lib.PREC_F64, "f32": _lib.PREC_F32, "mixed": _lib.PREC_MIXED}


def trunc_params(cutoff=1e-15, maxdim=None, mindim=1, normalize=False, precision="f64"):
    return _lib.TruncParams(float(cutoff if cutoff is not None else 0.0), int(maxdim or 0),
                            int(mindim or 1), int(bool(normalize)), PRECISIONS[precision])


def truncate(f, cutoff=1e-15, maxdim=None, mindim=1, normalize=False, precision="f64"):
    """Orthogonalise toward the root (QR) then SVD-truncate every bond, keeping
    the smallest rank whose discarded weight sum(s^2)/sum(s^2) <= cutoff."""
    p = trunc_params(cutoff, maxdim, mindim, normalize, precision)
    h = C.c_void_p()
    f.ctx.call("tnfa_truncate", f.handle, C.byref(p), C.byref(h))
    return f._wrap(h)


def truncate_batched(fs, cutoff=1e-15, maxdim=None, mindim=1, normalize=False, precision="f64"):
    """truncate() of many networks in one scheduled pass."""
    n = len(fs)
    if n == 0:
        return []
    p = trunc_params(cutoff, maxdim, mindim, normalize, precision)
    fh = (C.c_void_p * n)(*[f.handle.value for f in fs])
    out = (C.c_void_p * n)()
    fs[0].ctx.call("tnfa_truncate_batched", n, fh, C.byref(p), out)
    return [f._wrap(C.c_void_p(out[i])) for i, f in enumerate(fs)]

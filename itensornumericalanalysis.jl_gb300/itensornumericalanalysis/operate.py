"""Operator application (mirrors src/elementary_operators.jl:294-319)."""
from __future__ import annotations

import ctypes as C

from .truncation import trunc_params


def operate(op, f, cutoff=1e-15, maxdim=None, normalize=False, precision="f64", **_ignored):
    """O f contracted exactly vertex by vertex, then truncated with cutoff /
    maxdim (the reference calls ITensorNetworks.contract(O, f; alg="fit"))."""
    if isinstance(op, (list, tuple)):
        out = f
        for o in op:
            out = operate(o, out, cutoff, maxdim, normalize, precision)
        return out
    p = trunc_params(cutoff, maxdim, 1, normalize, precision)
    h = C.c_void_p()
    f.ctx.call("tnfa_apply", op.handle, f.handle, C.byref(p), C.byref(h))
    return type(f)(f.s, h, f.ctx)

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


def operate_batched(ops, fs, cutoff=1e-15, maxdim=None, normalize=False, precision="f64"):
    """[O_i f_i] for many independent (operator, function) pairs in one
    scheduled pass (paths of uneven length and bond dimension are processed
    step by step together)."""
    n = len(fs)
    if len(ops) != n:
        raise ValueError("ops and fs differ in length")
    p = trunc_params(cutoff, maxdim, 1, normalize, precision)
    oh = (C.c_void_p * max(n, 1))(*[o.handle.value for o in ops])
    fh = (C.c_void_p * max(n, 1))(*[f.handle.value for f in fs])
    out = (C.c_void_p * max(n, 1))()
    if n == 0:
        return []
    fs[0].ctx.call("tnfa_apply_batched", n, oh, fh, C.byref(p), out)
    return [type(f)(f.s, C.c_void_p(out[i]), f.ctx) for i, f in enumerate(fs)]

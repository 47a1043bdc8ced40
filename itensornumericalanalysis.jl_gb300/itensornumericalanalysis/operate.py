"""Operator application (mirrors src/elementary_operators.jl:294-319)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
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


def operate_exact(op, f):
    """O f contracted exactly vertex by vertex, no truncation (bond dims
    multiply): the forward map differentiated by operate_vjp."""
    h = C.c_void_p()
    f.ctx.call("tnfa_apply_exact", op.handle, f.handle, C.byref(h))
    return type(f)(f.s, h, f.ctx)


def operate_vjp(op, f, dy) -> np.ndarray:
    """J^T dy for y = operate_exact(op, f): the cotangent of f's tensors (flat,
    canonical layout) from dy, the cotangent of y's (flat, y's canonical
    layout).  The backward pass of an rrule for operate through its exact
    contraction."""
    _, dt, ne, _ = f.info()
    npdt = {_lib.F64: np.float64, _lib.C128: np.complex128}[dt]
    dy = np.ascontiguousarray(np.asarray(dy, dtype=npdt).ravel())
    df = np.zeros(ne, dtype=npdt)
    f.ctx.call("tnfa_apply_vjp", op.handle, f.handle, dy.ctypes.data_as(C.c_void_p), _lib.MEM_HOST,
               df.ctypes.data_as(C.c_void_p), _lib.MEM_HOST)
    return df

"""Integration of tensor network functions (mirrors src/integration.jl)."""
from __future__ import annotations

import ctypes as C

from .network import ITensorNetworkFunction


def integrate(f, g=None, take_sum: bool = False):
    """integrate(f): left Riemann sum of f over [0,1)^n (src/integration.jl:6-17);
    integrate(O, f): integral of O*f (src/integration.jl:20-32)."""
    if g is None:
        return f.integrate(take_sum=take_sum)
    op, fn = f, g
    out = (C.c_double * 2)()
    fn.ctx.call("tnfa_integrate_operator", op.handle, fn.handle, int(take_sum), out)
    return complex(out[0], out[1]) if (fn.is_complex or op.is_complex) else out[0]


def partial_integrate(f: ITensorNetworkFunction, dims, take_sum: bool = False):
    """Integrate over the variables `dims` only, merging vertices left without
    digits into a neighbour (src/integration.jl:35-54)."""
    raise NotImplementedError("partial_integrate")

"""Gradients of batched evaluation (the rrule of evaluate).

The reference has no automatic differentiation; a Julia caller binds a
hand-written backward pass behind a ChainRulesCore.rrule.  Here
`tnfa_evaluate_vjp` is that backward pass; `evaluate_vjp` returns it per
vertex, and `TTNEvaluate` wraps forward + backward as a torch.autograd.Function
(the Python analogue of an rrule) for fitting tensors to data by gradient
descent.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .network import ITensorNetworkFunction, _i32


def evaluate_vjp(f: ITensorNetworkFunction, X, dout, dims=None) -> dict:
    """sum_p dout[p] * d f(x_p) / d T_v, as arrays in canonical layout
    [site legs..., parent, children...] keyed by vertex."""
    dims = f.s.dimensions() if dims is None else list(dims)
    X = np.ascontiguousarray(np.asarray(X, dtype=np.float64).reshape(len(dout), len(dims)))
    dout = np.ascontiguousarray(np.asarray(dout, dtype=np.float64))
    _, dt, ne, _ = f.info()
    npdt = {_lib.F64: np.float64, _lib.F32: np.float32, _lib.C128: np.complex128}[dt]
    acc = np.zeros(ne, dtype=npdt)
    f.ctx.call("tnfa_evaluate_vjp", f.handle, X.ctypes.data_as(C.c_void_p), len(X), len(dims),
               _i32(dims), _lib.MEM_HOST, dout.ctypes.data_as(C.c_void_p), _lib.MEM_HOST,
               acc.ctypes.data_as(C.c_void_p), _lib.MEM_HOST)
    tens = f.tensors()
    out, off = {}, 0
    for v in f.s.layout.order:
        n = tens[v].size
        out[v] = acc[off:off + n].reshape(tens[v].shape)
        off += n
    return out


def _torch():
    import torch

    return torch


class TTNEvaluate:
    """f(X) for a flat parameter tensor (canonical layout, on the GPU) with a
    backward pass through tnfa_evaluate_vjp; use TTNEvaluate.apply(params, X)."""

    _fn = None

    @classmethod
    def function(cls):
        if cls._fn is None:
            torch = _torch()

            class _F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, params, X, template, dims):
                    net = template.with_tensors_device(params)
                    n = X.shape[0]
                    out = torch.empty(n, dtype=torch.float64, device=X.device)
                    torch.cuda.synchronize()
                    template.ctx.call("tnfa_evaluate", net.handle, X.data_ptr(), n, len(dims),
                                      _i32(dims), _lib.MEM_DEVICE, out.data_ptr(), _lib.OUT_F64,
                                      _lib.MEM_DEVICE, _lib.PREC_F64 if params.dtype == torch.float64
                                      else _lib.PREC_F32)
                    ctx.save_for_backward(params, X)
                    ctx.net, ctx.dims = net, dims
                    return out.to(params.dtype)

                @staticmethod
                def backward(ctx, gout):
                    params, X = ctx.saved_tensors
                    g = torch.zeros_like(params)
                    d = gout.detach().to(torch.float64).contiguous()
                    torch.cuda.synchronize()
                    ctx.net.ctx.call("tnfa_evaluate_vjp", ctx.net.handle, X.data_ptr(), X.shape[0],
                                     len(ctx.dims), _i32(ctx.dims), _lib.MEM_DEVICE, d.data_ptr(),
                                     _lib.MEM_DEVICE, g.data_ptr(), _lib.MEM_DEVICE)
                    return g, None, None, None

            cls._fn = _F
        return cls._fn

    @classmethod
    def apply(cls, params, X, template: ITensorNetworkFunction, dims):
        return cls.function().apply(params, X, template, list(dims))

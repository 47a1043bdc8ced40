"""Integration of tensor network functions (mirrors src/integration.jl)."""
from __future__ import annotations

import ctypes as C

from .graphs import NamedGraph
from .indexmap import IndsNetworkMap
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


def partial_integrate(f: ITensorNetworkFunction, dims, merge_vertices: bool = True,
                      take_sum: bool = False) -> ITensorNetworkFunction:
    """Integrate over the variables `dims` only (src/integration.jl:35-54):
    their digit legs are contracted with 1/base (1 with take_sum), and with
    merge_vertices every vertex left without legs is absorbed into its first
    neighbour in graph order (merge_internal_tensors, src/utils.jl:99-113).
    The result lives on the surviving vertices, in the input's vertex order."""
    dims = [dims] if isinstance(dims, int) else list(dims)
    s = f.s
    lay = s.layout
    gpos = {v: i for i, v in enumerate(s.vertices())}
    rank = (C.c_int32 * lay.n)(*[gpos[v] for v in lay.order])
    vars_ = (C.c_int32 * max(1, len(dims)))(*dims)
    ov = (C.c_int32 * lay.n)()
    h = C.c_void_p()
    f.ctx.call("tnfa_partial_integrate", f.handle, len(dims), vars_, int(take_sum),
               int(merge_vertices), rank, C.byref(h), ov)
    nv = C.c_int32()
    dt, ne = C.c_int32(), C.c_int64()
    f.ctx.check(f.ctx.lib.tnfa_net_info(h, C.byref(nv), C.byref(dt), C.byref(ne), None))
    W = nv.value
    parent = (C.c_int32 * W)()
    f.ctx.check(f.ctx.lib.tnfa_net_topology(h, parent, None, None, None, None, None, None, None))
    names = [lay.order[ov[k]] for k in range(W)]
    verts = sorted(names, key=lambda v: gpos[v])
    edges = []
    for k in range(W):
        if parent[k] >= 0:
            u, w = names[parent[k]], names[k]
            edges.append((u, w) if gpos[u] < gpos[w] else (w, u))
    edges.sort(key=lambda e: (gpos[e[0]], gpos[e[1]]))
    legs = {v: [l for l in s.legs[v] if l.dim not in dims] for v in verts}
    out_map = IndsNetworkMap(NamedGraph(verts, edges), legs, s.is_complex)
    if out_map.layout.order != names:
        f.ctx.lib.tnfa_net_destroy(h)
        raise RuntimeError("partial_integrate: layout of the merged tree disagrees with the library's")
    return ITensorNetworkFunction(out_map, h, f.ctx)

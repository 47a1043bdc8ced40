"""ITensorNetworkFunction: a tree tensor network on the GPU plus its digit map.

Mirrors src/itensornetworkfunction.jl (struct :18-22, evaluate :96-112,
truncate :114-118).  The tensors live in device memory owned by libtnfa; this
object holds the handle, the IndsNetworkMap and the device layout.  Every
numerical method calls the C ABI -- there is no host compute path.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import TnfaError
from .indexmap import IndsNetworkMap

PRECISIONS = {"f64": _lib.PREC_F64, "f32": _lib.PREC_F32, "mixed": _lib.PREC_MIXED,
              "mixed_fast": _lib.PREC_MIXED_FAST}


def _i32(a) -> C.Array:
    a = list(a)
    return (C.c_int32 * max(1, len(a)))(*a)


def topology_struct(s: IndsNetworkMap, link_dims: Sequence[int], legs=None):
    """A tnfa_topology for the layout of `s` (plus the arrays it points into)."""
    lay = s.layout
    nlegs, ldim, lvar, ldig, lkind = legs if legs is not None else s.leg_arrays()
    arrays = [_i32(lay.parent), _i32(link_dims), _i32(nlegs), _i32(ldim), _i32(lvar),
              _i32(ldig), _i32(lkind)]
    t = _lib.Topology(lay.n, *[C.cast(a, C.POINTER(C.c_int32)) for a in arrays])
    return t, arrays


class ITensorNetworkFunction:
    """f(x_1..x_n) as a tree tensor network whose site legs are digits."""

    def __init__(self, s: IndsNetworkMap, handle: C.c_void_p, ctx: _lib.Context | None = None,
                 legs=None):
        self.s = s
        self._h = handle
        self._ctx = ctx or _lib.default_context()
        self._legs = legs  # explicit leg arrays (operators); None = from s

    # -- construction ---------------------------------------------------------
    @classmethod
    def from_tensors(cls, s: IndsNetworkMap, tensors: dict, ctx=None, legs=None, dtype=None):
        """Upload per-vertex tensors given in canonical layout
        [site legs..., parent bond, child bonds...] (keys are vertex names).
        On a map whose graph has cycles the tensors have axes [site legs...,
        bonds to the neighbours in graph neighbour order]; the function is
        then held exactly on the map's tree image (merge_to_tree_image)."""
        ctx = ctx or _lib.default_context()
        if not s.graph.is_forest():
            from .indexmap import merge_to_tree_image

            return cls.from_tensors(s.tree_image, merge_to_tree_image(s, tensors), ctx=ctx,
                                    dtype=dtype)
        lay = s.layout
        arrs = [np.asarray(tensors[v]) for v in lay.order]
        is_c = any(np.iscomplexobj(a) for a in arrs)
        if dtype is None:
            dtype = _lib.C128 if is_c else _lib.F64
        npdt = {_lib.F64: np.float64, _lib.F32: np.float32, _lib.C128: np.complex128}[dtype]
        link = [1] * lay.n
        nlegs = (legs or s.leg_arrays())[0]
        for i, a in enumerate(arrs):
            p = lay.parent[i]
            k = nlegs[i]
            if p >= 0:
                link[i] = a.shape[k]
        for i, a in enumerate(arrs):
            expect = list(a.shape[: nlegs[i]]) + [link[i]] + [link[c] for c in lay.children[i]]
            if list(a.shape) != expect:
                raise ValueError(
                    f"tensor of vertex {lay.order[i]!r} has shape {a.shape}, expected {tuple(expect)}"
                )
        flat = np.concatenate([np.ascontiguousarray(a, dtype=npdt).ravel() for a in arrs])
        topo, keep = topology_struct(s, link, legs)
        h = C.c_void_p()
        ctx.call("tnfa_net_create", C.byref(topo), dtype, flat.ctypes.data_as(C.c_void_p),
                 _lib.MEM_HOST, C.byref(h))
        return cls(s, h, ctx, legs)

    def with_tensors_device(self, flat) -> "ITensorNetworkFunction":
        """A network with this one's shape and tensors from a flat device
        buffer (anything with data_ptr(), e.g. a CUDA torch tensor) in
        canonical layout; FP64 or FP32 from the buffer's element size."""
        _, _, ne, link = self.info()
        es = flat.element_size()
        dtype = {8: _lib.F64, 4: _lib.F32}[es]
        if flat.numel() != ne:
            raise ValueError(f"flat buffer has {flat.numel()} elements, network needs {ne}")
        topo, keep = topology_struct(self.s, link, self._legs)
        h = C.c_void_p()
        self._ctx.call("tnfa_net_create", C.byref(topo), dtype, C.c_void_p(flat.data_ptr()),
                       _lib.MEM_DEVICE, C.byref(h))
        return self._wrap(h)

    def _wrap(self, handle: C.c_void_p, s: IndsNetworkMap | None = None, legs="same"):
        return type(self)(s or self.s, handle, self._ctx, self._legs if legs == "same" else legs)

    def __del__(self):
        # the library keeps the context alive while networks exist, so this
        # is safe in any finalisation order
        try:
            if self._h:
                self._ctx.lib.tnfa_net_destroy(self._h)
                self._h = None
        except Exception:
            pass

    # -- shape ---------------------------------------------------------------
    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def ctx(self) -> _lib.Context:
        return self._ctx

    def info(self):
        nv, dt, ne = C.c_int32(), C.c_int32(), C.c_int64()
        link = (C.c_int32 * self.s.layout.n)()
        self._ctx.check(self._ctx.lib.tnfa_net_info(self._h, C.byref(nv), C.byref(dt),
                                                    C.byref(ne), link))
        return nv.value, dt.value, ne.value, list(link)

    @property
    def dtype(self) -> int:
        return self.info()[1]

    @property
    def is_complex(self) -> bool:
        return self.dtype == _lib.C128

    def linkdims(self) -> dict:
        """Bond dimension per edge (child vertex name -> dim of its parent bond)."""
        lay = self.s.layout
        link = self.info()[3]
        return {(lay.order[lay.parent[i]], lay.order[i]): link[i]
                for i in range(lay.n) if lay.parent[i] >= 0}

    def lift(self, u: IndsNetworkMap) -> "ITensorNetworkFunction":
        """This function as a network on the tree of `u` (a map containing this
        one's vertices, edges and legs): constant along the legs and vertices
        it lacks, bond 1 on the edges it lacks (tnfa_net_gather)."""
        fl, ul = self.s.layout, u.layout
        link = self.info()[3]
        bond = {}
        for i in range(fl.n):
            if fl.parent[i] >= 0:
                bond[frozenset((fl.order[i], fl.order[fl.parent[i]]))] = link[i]
        link_u = [1] * ul.n
        for t, v in enumerate(ul.order):
            if ul.parent[t] >= 0:
                link_u[t] = bond.get(frozenset((v, ul.order[ul.parent[t]])), 1)
        nlegs_f, ldim_f = self._leg_shape()
        src, strides = [], []
        for t, v in enumerate(ul.order):
            nbs = ([ul.order[ul.parent[t]]] if ul.parent[t] >= 0 else [None]) + [
                ul.order[c] for c in ul.children[t]]
            if v not in fl.pos:
                src.append(-1)
                strides += [0] * (len(u.legs[v]) + len(nbs))
                continue
            i = fl.pos[v]
            src.append(i)
            dims = list(ldim_f[i]) + [link[i]] + [link[c] for c in fl.children[i]]
            st = [1] * len(dims)
            for a in range(len(dims) - 2, -1, -1):
                st[a] = st[a + 1] * dims[a + 1]
            key = {(l.dim, l.digit, l.kind): k for k, l in enumerate(self.s.legs[v])}
            for l in u.legs[v]:
                k = key.get((l.dim, l.digit, l.kind))
                strides.append(st[k] if k is not None else 0)
            nl = nlegs_f[i]
            axis = {}
            if fl.parent[i] >= 0:
                axis[fl.order[fl.parent[i]]] = nl
            for k, c in enumerate(fl.children[i]):
                axis[fl.order[c]] = nl + 1 + k
            for w in nbs:
                strides.append(st[axis[w]] if w in axis else 0)
        topo, keep = topology_struct(u, link_u)
        srcv = (C.c_int32 * ul.n)(*src)
        stv = (C.c_int64 * max(1, len(strides)))(*strides)
        h = C.c_void_p()
        self._ctx.call("tnfa_net_gather", self._h, C.byref(topo), srcv, stv, C.byref(h))
        return type(self)(u, h, self._ctx)

    def maxlinkdim(self) -> int:
        d = self.linkdims()
        return max(d.values()) if d else 1

    def tensors(self) -> dict:
        """Download the tensors: vertex name -> array [site legs..., parent, children...]."""
        _, dt, ne, link = self.info()
        npdt = {_lib.F64: np.float64, _lib.F32: np.float32, _lib.C128: np.complex128}[dt]
        flat = np.empty(ne, dtype=npdt)
        self._ctx.call("tnfa_net_download", self._h, flat.ctypes.data_as(C.c_void_p), _lib.MEM_HOST)
        lay = self.s.layout
        nlegs, ldim = self._leg_shape()
        out, off = {}, 0
        for i, v in enumerate(lay.order):
            shape = tuple(ldim[i]) + (link[i],) + tuple(link[c] for c in lay.children[i])
            n = int(np.prod(shape))
            out[v] = flat[off : off + n].reshape(shape)
            off += n
        return out

    def _leg_shape(self):
        nlegs, ldim, *_ = self._legs or self.s.leg_arrays()
        per, k = [], 0
        for n in nlegs:
            per.append(ldim[k : k + n])
            k += n
        return nlegs, per

    # -- evaluation (hot path) ----------------------------------------------
    def evaluate_batch(self, X, dims=None, precision: str = "f64", out: str = "f64",
                       device_out=None) -> np.ndarray:
        """f at every row of X (n_points x len(dims)); complex maps take complex X.

        precision: "f64" (plain FP64), "f32" (FP32 CUDA cores), "mixed"
        (FP64 messages; bond-64/128 vertices as exact products of 8-bit
        integer slices on the tcgen05 tensor cores, FP64-class accuracy) or
        "mixed_fast" (FP32 messages, split-BF16 tensor-core products, about
        1e-5 relative on random bond-128 trees)."""
        dims = self.s.dimensions() if dims is None else ([dims] if isinstance(dims, int) else list(dims))
        X = np.asarray(X)
        if X.ndim == 1:
            X = X.reshape(-1, len(dims)) if len(dims) > 1 else X.reshape(-1, 1)
        if X.shape[1] != len(dims):
            raise ValueError(f"X has {X.shape[1]} columns for {len(dims)} dims")
        if self.s.is_complex:
            Xc = np.asarray(X, dtype=np.complex128)
            Xd = np.ascontiguousarray(np.stack([Xc.real, Xc.imag], axis=-1).reshape(len(X), -1))
        else:
            if np.iscomplexobj(X):
                raise ValueError("complex coordinates need a complex index map")
            Xd = np.ascontiguousarray(X, dtype=np.float64)
        P = len(Xd)
        cplx = self.is_complex
        if cplx:
            res = np.empty(P, dtype=np.complex128)
            kind = _lib.OUT_C128
        elif out == "f32":
            res = np.empty(P, dtype=np.float32)
            kind = _lib.OUT_F32
        elif out == "f32_scaled":
            res = np.empty(2 * P, dtype=np.float32)
            kind = _lib.OUT_F32_SCALED
        else:
            res = np.empty(P, dtype=np.float64)
            kind = _lib.OUT_F64
        self._ctx.call(
            "tnfa_evaluate", self._h, Xd.ctypes.data_as(C.c_void_p), P, len(dims), _i32(dims),
            _lib.MEM_HOST, res.ctypes.data_as(C.c_void_p), kind, _lib.MEM_HOST,
            PRECISIONS[precision] if not cplx else _lib.PREC_F64,
        )
        if kind == _lib.OUT_F32_SCALED:
            m = res[:P].astype(np.float64)
            e = res[P:].view(np.int32)
            return m, e
        return res

    def evaluation_plan(self, X, out, dims=None, precision: str | None = None,
                        out_kind: str = "f64") -> "EvaluationPlan":
        """A captured evaluation (tnfa_eval_plan_create) of this network at the
        rows of the CUDA tensor X (n_points x len(dims), float64, contiguous)
        into the CUDA tensor out, replayed by EvaluationPlan.launch() with one
        graph launch; X's contents may change between launches.  precision
        defaults to the network's own type ("f64" for FP64 and complex
        networks, "f32" for FP32 ones)."""
        dims = self.s.dimensions() if dims is None else ([dims] if isinstance(dims, int) else list(dims))
        if precision is None:
            precision = "f32" if self.dtype == _lib.F32 else "f64"
        kinds = {"f64": _lib.OUT_F64, "f32": _lib.OUT_F32, "f32_scaled": _lib.OUT_F32_SCALED,
                 "c128": _lib.OUT_C128}
        kind = _lib.OUT_C128 if self.is_complex else kinds[out_kind]
        if not (X.is_cuda and out.is_cuda and X.is_contiguous() and out.is_contiguous()):
            raise ValueError("an evaluation plan needs contiguous CUDA tensors for X and out")
        P = X.shape[0]
        h = C.c_void_p()
        self._ctx.call("tnfa_eval_plan_create", self._h, C.c_void_p(X.data_ptr()), P, len(dims),
                       _i32(dims), C.c_void_p(out.data_ptr()), kind,
                       PRECISIONS[precision] if not self.is_complex else _lib.PREC_F64, C.byref(h))
        return EvaluationPlan(self, h, X, out)

    def evaluate(self, xs, dims=None, **kw):
        """evaluate (src/itensornetworkfunction.jl:96-112): f at one point."""
        xs = [xs] if np.isscalar(xs) else list(xs)
        if dims is None:
            dims = self.s.dimensions()[: len(xs)] if len(xs) < len(self.s.dimensions()) else self.s.dimensions()
        dims = [dims] if isinstance(dims, int) else list(dims)
        r = self.evaluate_batch(np.asarray([xs]), dims, **kw)
        return r[0]

    __call__ = evaluate

    # -- reductions ------------------------------------------------------------
    def integrate(self, take_sum: bool = False):
        """integrate (src/integration.jl:6-17)."""
        out = (C.c_double * 2)()
        self._ctx.call("tnfa_integrate", self._h, int(take_sum), out)
        return complex(out[0], out[1]) if self.is_complex else out[0]

    def inner(self, other: "ITensorNetworkFunction"):
        """<self|other> = sum over the grid of conj(self) * other."""
        a, b = self._promote(other)
        out = (C.c_double * 2)()
        self._ctx.call("tnfa_inner", a._h, b._h, out)
        return complex(out[0], out[1]) if a.is_complex else out[0]

    def norm(self) -> float:
        return float(abs(self.inner(self)) ** 0.5)

    # -- algebra -------------------------------------------------------------
    def copy(self) -> "ITensorNetworkFunction":
        h = C.c_void_p()
        self._ctx.call("tnfa_net_copy", self._h, C.byref(h))
        return self._wrap(h)

    def astype(self, dtype: int) -> "ITensorNetworkFunction":
        h = C.c_void_p()
        self._ctx.call("tnfa_net_convert", self._h, dtype, C.byref(h))
        return self._wrap(h)

    def scale_vertex(self, v, c) -> None:
        """In place: multiply the tensor of vertex v by c."""
        c = complex(c)
        if c.imag != 0 and not self.is_complex:
            raise TypeError("complex factor on a real network; convert with astype(C128) first")
        self._ctx.call("tnfa_net_scale", self._h, self.s.layout.pos[v], c.real, c.imag)

    def _promote(self, other):
        a, b = self, other
        if a.is_complex != b.is_complex:
            if not a.is_complex:
                a = a.astype(_lib.C128)
            else:
                b = b.astype(_lib.C128)
        return a, b

    def __add__(self, other):
        if not isinstance(other, ITensorNetworkFunction):
            return NotImplemented
        if not self.s.same_structure(other.s):
            raise ValueError("+ needs functions on the same IndsNetworkMap")
        a, b = self._promote(other)
        h = C.c_void_p()
        self._ctx.call("tnfa_add", a._h, b._h, C.byref(h))
        return self._wrap(h)

    def __mul__(self, other):
        if isinstance(other, ITensorNetworkFunction):
            from .elementary_operators import multiply

            return multiply(self, other)
        c = complex(other)
        out = self.copy() if (c.imag == 0 or self.is_complex) else self.astype(_lib.C128)
        out.scale_vertex(self.s.layout.order[0], c if out.is_complex else c.real)
        return out

    def __rmul__(self, other):
        return self.__mul__(other)

    def __neg__(self):
        return self * -1.0

    def __sub__(self, other):
        return self + (-other)

    def __repr__(self) -> str:
        try:
            _, dt, ne, _ = self.info()
            return (f"ITensorNetworkFunction(nv={self.s.nv()}, dims={self.s.dimensions()}, "
                    f"maxlinkdim={self.maxlinkdim()}, dtype={['f64', 'f32', 'c128'][dt]})")
        except TnfaError:
            return "ITensorNetworkFunction(<invalid>)"


def evaluate(f: ITensorNetworkFunction, xs, dims=None, **kw):
    """evaluate(f, xs, dims) for one point, or for an (n_points x n_dims) array."""
    a = np.asarray(xs)
    if a.ndim == 2:
        return f.evaluate_batch(a, dims, **kw)
    return f.evaluate(xs, dims, **kw)


def inner(f: ITensorNetworkFunction, g: ITensorNetworkFunction):
    """<f|g> over the full grid (conjugating f)."""
    return f.inner(g)


def itensornetwork(f: ITensorNetworkFunction) -> dict:
    """The network inside the function (src/itensornetworkfunction.jl:24), as
    host arrays: vertex name -> tensor [site legs..., parent bond, child bonds]."""
    return f.tensors()


def calculate_fx(f: ITensorNetworkFunction, X, dims=None, **kw) -> np.ndarray:
    """Batched evaluation (the name the GB300 API uses for evaluate over many points)."""
    return f.evaluate_batch(X, dims, **kw)


class EvaluationPlan:
    """A network's evaluation on fixed CUDA buffers, captured as a CUDA graph
    (tnfa_eval_plan_*).  Holds the network, X and out alive."""

    def __init__(self, f, handle, X, out):
        self._f, self._h, self.X, self.out = f, handle, X, out

    def launch(self) -> None:
        """Enqueue one evaluation of the current X on the context's stream."""
        self._f.ctx.call("tnfa_eval_plan_launch", self._h)

    def check(self) -> None:
        """Wait for the stream; raise TnfaError for a bad coordinate."""
        self._f.ctx.call("tnfa_eval_plan_check", self._h)

    def close(self) -> None:
        if self._h is not None and self._h.value:
            _lib.load().tnfa_eval_plan_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

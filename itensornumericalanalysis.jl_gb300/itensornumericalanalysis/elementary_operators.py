"""Finite-difference operators, operator application and products.

Mirrors src/elementary_operators.jl.  An operator is a tree network whose
site legs fuse (out, in) into one leg of dimension base^2 (out = the primed
index of the reference's ITensors).  Operators are built from the
reference's OpSums -- sums of products of the digit operators
D+, D-, Dup, Ddn (src/digit_inds.jl:35-58) -- as a block-diagonal direct sum
of their terms, then compressed on the device by truncation, which is what
ITensorNetworks' ttn(OpSum; cutoff) produces up to gauge.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from .indexmap import IndsNetworkMap
from .network import ITensorNetworkFunction, topology_struct

default_boundary = "Dirichlet"

# Digit operators as matrices M[out, in] (src/digit_inds.jl:35-58: the
# reference writes ITensor(o, s, s') so o[in, out]).
_OPS = {
    "D+": np.array([[0.0, 1.0], [0.0, 0.0]]),
    "D-": np.array([[0.0, 0.0], [1.0, 0.0]]),
    "Ddn": np.array([[1.0, 0.0], [0.0, 0.0]]),
    "Dup": np.array([[0.0, 0.0], [0.0, 1.0]]),
}


def _op_matrix(name, base: int) -> np.ndarray:
    """A digit operator by name, or a base x base matrix M[out, in] given directly."""
    if not isinstance(name, str):
        m = np.asarray(name)
        if m.shape != (base, base):
            raise ValueError(f"a site operator on a base-{base} digit must be {base}x{base}")
        return m
    if name == "I":
        return np.eye(base)
    if base != 2:
        raise ValueError("digit shift operators are defined for base 2")
    if name not in _OPS:
        raise ValueError(f"unknown digit operator {name!r}")
    return _OPS[name]


def operator_legs(s: IndsNetworkMap):
    """Leg arrays of an operator on s: every digit leg becomes (out, in)."""
    nlegs, ldim, lvar, ldig, lkind = s.leg_arrays()
    return nlegs, [d * d for d in ldim], lvar, ldig, [_lib.LEG_OPERATOR] * len(ldim)


class ITensorNetworkOperator(ITensorNetworkFunction):
    """A tree tensor network operator (a TreeTensorNetwork of the reference)."""

    def evaluate_batch(self, *a, **k):
        raise TypeError("an operator is not a function; apply it with operate()")

    def _wrap(self, handle, s=None, legs="same"):
        return ITensorNetworkOperator(s or self.s, handle, self._ctx,
                                      self._legs if legs == "same" else legs)

    def __add__(self, other):
        if not isinstance(other, ITensorNetworkOperator):
            return NotImplemented
        a, b = self._promote(other)
        h = C.c_void_p()
        self._ctx.call("tnfa_add", a._h, b._h, C.byref(h))
        return self._wrap(h)

    def __repr__(self):
        return f"ITensorNetworkOperator(nv={self.s.nv()}, maxlinkdim={self.maxlinkdim()})"


# ------------------------------------------------------------ OpSums ----
class OpSum:
    """Sum of products of digit operators; a term maps (dim, digit) to an op
    name ("D+", "D-", "Dup", "Ddn", "I") or a base x base matrix M[out, in]."""

    def __init__(self, terms=None):
        self.terms: list[tuple[complex, dict]] = list(terms or [])

    def add(self, coef, ops: dict) -> None:
        self.terms.append((coef, dict(ops)))

    def __add__(self, other: "OpSum") -> "OpSum":
        return OpSum(self.terms + other.terms)

    def __rmul__(self, c) -> "OpSum":
        return OpSum([(c * k, ops) for k, ops in self.terms])

    __mul__ = __rmul__


def boundary_term(s: IndsNetworkMap, boundary: str, dim: int, isfwd: bool, n: int = 0) -> OpSum:
    """src/elementary_operators.jl:32-57: Neumann adds Dup.. (fwd) / Ddn.. (bwd)
    on the top L-n digits, Periodic adds D-.. (fwd) / D+.. (bwd)."""
    L = s.ndigits(dim)
    out = OpSum()
    if boundary == "Neumann":
        out.add(1.0, {(dim, j): ("Dup" if isfwd else "Ddn") for j in range(1, L - n + 1)})
    elif boundary == "Periodic":
        out.add(1.0, {(dim, j): ("D-" if isfwd else "D+") for j in range(1, L - n + 1)})
    elif boundary != "Dirichlet":
        raise ValueError(f"unknown boundary {boundary!r}")
    return out


def _shift_opsum(s, dim, boundary, n, up: str, down: str, isfwd: bool) -> OpSum:
    if not s.is_tree():
        raise ValueError("shift operators need a tree")
    if s.base() != 2:
        raise ValueError("shift operators need base 2")
    L = s.ndigits(dim)
    out = OpSum()
    string = {(dim, L - n): up}
    out.add(1.0, string)
    for i in range(L - n, 1, -1):
        string = dict(string)
        string[(dim, i)] = down
        string[(dim, i - 1)] = up
        out.add(1.0, string)
    return out + boundary_term(s, boundary, dim, isfwd, n)


def forward_shift_opsum(s, dim=1, boundary=default_boundary, n: int = 0):
    """f(x + (n+1) delta) with carries (src/elementary_operators.jl:59-80)."""
    return _shift_opsum(s, dim, boundary, n, "D+", "D-", True)


def backward_shift_opsum(s, dim=1, boundary=default_boundary, n: int = 0):
    """f(x - (n+1) delta) with borrows (src/elementary_operators.jl:82-103)."""
    return _shift_opsum(s, dim, boundary, n, "D-", "D+", False)


def no_shift_opsum(s) -> OpSum:
    """Identity (src/elementary_operators.jl:105-110)."""
    return OpSum([(1.0, {})])


def _site_op(s: IndsNetworkMap, v, ops: dict) -> np.ndarray:
    """Fused (out, in) site tensor of one OpSum term at vertex v."""
    t = np.ones(())
    for l in s.legs[v]:
        m = _op_matrix(ops.get((l.dim, l.digit), "I"), l.base)
        t = np.multiply.outer(t, m.reshape(-1))
    return t


# Terms per direct-sum block: an OpSum longer than this is compiled block by
# block, each block compressed, and the blocks summed with a compression
# after every addition, so that no bond before compression exceeds a block
# plus the running sum's rank.
OPSUM_BLOCK = 64


def _native_map(s: IndsNetworkMap) -> bool:
    """Maps the library builds operators for directly (tnfa_op_from_terms /
    tnfa_op_build_stencil): a tree (or forest) of real digit legs."""
    return s.graph.is_forest() and not s.is_complex


def _native_terms(s: IndsNetworkMap, terms, cutoff: float):
    """tnfa_op_from_terms on real terms: None when a coefficient or a site
    matrix is complex (those are assembled here and compressed on the
    device)."""
    if any(np.iscomplexobj(c) and np.imag(c) != 0 for c, _ in terms):
        return None
    lay = s.layout
    legidx, k = {}, 0
    for v in lay.order:
        for l in s.legs[v]:
            legidx[(l.dim, l.digit)] = (k, l.base)
            k += 1
    coefs, nf, fl, fm = [], [], [], []
    for c, ops in terms:
        items = [(key, op) for key, op in ops.items() if not (isinstance(op, str) and op == "I")]
        coefs.append(float(np.real(c)))
        nf.append(len(items))
        for key, op in items:
            if key not in legidx:
                raise ValueError(f"no digit {key} in the index map")
            leg, base = legidx[key]
            m = _op_matrix(op, base)
            if np.iscomplexobj(m) and np.any(np.imag(m) != 0):
                return None
            fl.append(leg)
            fm.extend(np.real(m).astype(np.float64).ravel().tolist())
    t, arrays = topology_struct(s, [1] * lay.n)
    ctx = _lib.default_context()
    h = C.c_void_p()
    cd = (C.c_double * max(1, len(coefs)))(*coefs)
    md = (C.c_double * max(1, len(fm)))(*fm)
    nfa = (C.c_int32 * max(1, len(nf)))(*nf)
    fla = (C.c_int32 * max(1, len(fl)))(*fl)
    ctx.call("tnfa_op_from_terms", C.byref(t), len(coefs), cd, nfa, fla, md, float(cutoff), C.byref(h))
    return ITensorNetworkOperator(s, h, ctx, operator_legs(s))


def opsum_to_operator(s: IndsNetworkMap, opsum: OpSum, cutoff: float = 1e-15,
                      scale_dims: dict | None = None, compress: bool = True):
    """The OpSum as a tree operator (ITensorNetworks' ttn(OpSum; cutoff), used
    by src/elementary_operators.jl:114,119,151): a block-diagonal direct sum
    of the product terms (bond = number of terms), coefficients on the first
    vertex, then compressed on the device by truncation with the relative
    cutoff.  Up to gauge this is the operator ttn(OpSum) returns; the ranks
    are the SVD-minimal ones at that cutoff.  Real terms on a tree go through
    the library's own builder (tnfa_op_from_terms); complex ones are
    assembled here and compressed on the device the same way."""
    terms = opsum.terms
    if not terms:
        raise ValueError("an empty OpSum has no operator")
    if compress and _native_map(s):
        op = _native_terms(s, terms, cutoff)
        if op is not None:
            if scale_dims:
                for v, f in scale_dims.items():
                    op.scale_vertex(v, f)
            return op
    if compress and len(terms) > OPSUM_BLOCK:
        op = None
        for b0 in range(0, len(terms), OPSUM_BLOCK):
            part = _direct_sum(s, terms[b0:b0 + OPSUM_BLOCK])
            part = _compress(part, cutoff) if len(terms[b0:b0 + OPSUM_BLOCK]) > 1 else part
            op = part if op is None else _compress(op + part, cutoff)
        if scale_dims:
            for v, f in scale_dims.items():
                op.scale_vertex(v, f)
        return op
    op = _direct_sum(s, terms)
    if scale_dims:
        for v, f in scale_dims.items():
            op.scale_vertex(v, f)
    if compress and len(terms) > 1:
        op = _compress(op, cutoff)
    return op


def ttn(opsum: OpSum, s: IndsNetworkMap, cutoff: float = 1e-15) -> "ITensorNetworkOperator":
    """ITensorNetworks' ttn(os::OpSum, s; cutoff) as the reference calls it
    (src/elementary_operators.jl:114,119,151)."""
    return opsum_to_operator(s, opsum, cutoff=cutoff)


def _direct_sum(s: IndsNetworkMap, terms) -> "ITensorNetworkOperator":
    lay = s.layout
    T = len(terms)
    real = all(np.isreal(c) and all(isinstance(o, str) or not np.iscomplexobj(o) for o in ops.values())
               for c, ops in terms)
    dtype = float if real else complex
    ts = {}
    for i, v in enumerate(lay.order):
        site = [_site_op(s, v, ops) for _, ops in terms]
        sshape = site[0].shape
        nch = len(lay.children[i])
        root = lay.parent[i] < 0
        out = np.zeros(sshape + ((1,) if root else (T,)) + (T,) * nch, dtype=dtype)
        for t, (coef, _) in enumerate(terms):
            idx = (0 if root else t,) + (t,) * nch
            # += : a lone root (no bonds at all) sums the terms in place
            out[(Ellipsis,) + idx] += site[t] * (coef if i == 0 else 1.0)
        ts[v] = out
    return ITensorNetworkOperator.from_tensors(s, ts, legs=operator_legs(s))


def _compress(op: ITensorNetworkOperator, cutoff: float) -> ITensorNetworkOperator:
    """Recompress the term-by-term direct sum on the device (QR + SVD sweep)."""
    from .truncation import truncate

    return truncate(op, cutoff=cutoff)


def forward_shift_op(s, truncate_kwargs=None, **kw):
    """src/elementary_operators.jl:117-120."""
    return opsum_to_operator(s, forward_shift_opsum(s, **kw), **_tk(truncate_kwargs))


def backward_shift_op(s, truncate_kwargs=None, **kw):
    """src/elementary_operators.jl:112-115."""
    return opsum_to_operator(s, backward_shift_opsum(s, **kw), **_tk(truncate_kwargs))


def _tk(truncate_kwargs):
    tk = dict(truncate_kwargs or {})
    return {"cutoff": tk.get("cutoff", 1e-15)}


def stencil(s: IndsNetworkMap, shifts: Sequence[float], delta_power: int, dim: int = 1,
            left_boundary=default_boundary, right_boundary=default_boundary, scale: bool = True,
            cutoff: float = 1e-15, **_ignored):
    """shifts = [x+2d, x+d, x, x-d, x-2d] weights; scaled by base^power per
    vertex of `dim` (src/elementary_operators.jl:122-160)."""
    if len(shifts) != 5:
        raise ValueError("stencil needs 5 weights")
    b = s.base()
    bcs = {"Dirichlet": _lib.BC_DIRICHLET, "Neumann": _lib.BC_NEUMANN, "Periodic": _lib.BC_PERIODIC}
    for bc in (left_boundary, right_boundary):
        if bc not in bcs:
            raise ValueError(f"unknown boundary {bc!r}")
    if _native_map(s) and b == 2:
        # the library builds the carry-string terms and compresses them
        t, arrays = topology_struct(s, [1] * s.layout.n)
        ctx = _lib.default_context()
        h = C.c_void_p()
        w = (C.c_double * 5)(*[float(x) for x in shifts])
        ctx.call("tnfa_op_build_stencil", C.byref(t), int(dim), w, int(delta_power),
                 bcs[left_boundary], bcs[right_boundary], int(bool(scale)), float(cutoff), C.byref(h))
        return ITensorNetworkOperator(s, h, ctx, operator_legs(s))
    ops = shifts[2] * no_shift_opsum(s)
    for i in (0, 1):
        if shifts[i] != 0:
            ops = ops + shifts[i] * forward_shift_opsum(s, dim, right_boundary, 1 if i == 0 else 0)
    for i in (3, 4):
        if shifts[i] != 0:
            ops = ops + shifts[i] * backward_shift_opsum(s, dim, left_boundary, 1 if i == 4 else 0)
    scale_dims = {v: float(b) ** delta_power for v in s.dimension_vertices(dim)} if scale else None
    return opsum_to_operator(s, ops, cutoff=cutoff, scale_dims=scale_dims)


def first_derivative_operator(s, **kw):
    """(f(x+d) - f(x-d)) / 2d (src/elementary_operators.jl:162-164)."""
    return stencil(s, [0.0, 0.5, 0.0, -0.5, 0.0], 1, **kw)


def second_derivative_operator(s, **kw):
    """(f(x+d) - 2f(x) + f(x-d)) / d^2 (src/elementary_operators.jl:166-168)."""
    return stencil(s, [0.0, 1.0, -2.0, 1.0, 0.0], 2, **kw)


def third_derivative_operator(s, **kw):
    """src/elementary_operators.jl:170-172."""
    return stencil(s, [0.5, -1.0, 0.0, 1.0, -0.5], 3, **kw)


def fourth_derivative_operator(s, **kw):
    """src/elementary_operators.jl:174-176."""
    return stencil(s, [1.0, -4.0, 6.0, -4.0, 1.0], 4, **kw)


def laplacian_operator(s, boundary: str | None = None, dims=None, **kw):
    """Sum of second derivatives over dims (direct sum, not recompressed)
    (src/elementary_operators.jl:178-189)."""
    if boundary is not None:
        kw = dict(kw, left_boundary=boundary, right_boundary=boundary)
    dims = list(dims) if dims is not None else list(range(1, s.dimension() + 1))
    op = second_derivative_operator(s, dim=dims[0], **kw)
    for d in dims[1:]:
        op = op + second_derivative_operator(s, dim=d, **kw)
    return op


def identity_operator(s) -> ITensorNetworkOperator:
    """src/elementary_operators.jl:191-194."""
    return opsum_to_operator(s, no_shift_opsum(s), compress=False)


def operator_proj(f: ITensorNetworkFunction) -> ITensorNetworkOperator:
    """|f> -> diag(f) (src/elementary_operators.jl:247-258)."""
    h = C.c_void_p()
    f.ctx.call("tnfa_operator_proj", f.handle, C.byref(h))
    return ITensorNetworkOperator(f.s, h, f.ctx, operator_legs(f.s))


def multiply(g: ITensorNetworkFunction, f: ITensorNetworkFunction, *more) -> ITensorNetworkFunction:
    """Pointwise product (src/elementary_operators.jl:260-292): bond dims
    multiply on shared vertices; functions on disjoint vertex sets form a
    forest; on partially shared vertex sets the product lives on the union
    tree (legs and edges of both)."""
    if more:
        return multiply(multiply(g, f), *more)
    if g.s.same_structure(f.s):
        a, b = g._promote(f)
        h = C.c_void_p()
        g.ctx.call("tnfa_multiply", a.handle, b.handle, C.byref(h))
        return type(g)(g.s, h, g.ctx)
    if not set(g.s.vertices()) & set(f.s.vertices()):
        a, b = g._promote(f)
        h = C.c_void_p()
        g.ctx.call("tnfa_net_concat", a.handle, b.handle, C.byref(h))
        return type(g)(g.s.union(f.s), h, g.ctx)
    # shared vertices: the union tree, each factor lifted onto it (constant
    # along what it lacks), then the product on one structure
    u = g.s.union(f.s)
    if not u.graph.is_forest():
        raise ValueError("multiply: the union of the two trees has a cycle")
    a, b = g._promote(f)
    la, lb = a.lift(u), b.lift(u)
    h = C.c_void_p()
    g.ctx.call("tnfa_multiply", la.handle, lb.handle, C.byref(h))
    return type(g)(u, h, g.ctx)


def point_to_opsum(s, x, dim: int) -> OpSum:
    """src/elementary_operators.jl:197-206."""
    iv = s.calculate_ind_values([x], [dim])
    out = OpSum()
    out.add(1.0, {(l.dim, l.digit): ("Dup" if val == 1 else "Ddn") for l, val in iv.items()})
    return out


def map_to_zero_operator(s, xs, dims=None, **truncate_kwargs):
    """diag(1 - sum_x delta_x + overlaps) (src/elementary_operators.jl:209-227)."""
    from .elementary_functions import delta_kernel

    xs = [xs] if np.isscalar(xs) else list(xs)
    dims = [1] * len(xs) if dims is None else ([dims] if isinstance(dims, int) else list(dims))
    k = delta_kernel(s, [[x] for x in xs], [[d] for d in dims], remove_overlap=True, coeff=-1.0,
                     include_identity=True)
    return operator_proj(k)


def map_to_zeros(f, xs, dims=None, truncate_kwargs=None, **kw):
    """src/elementary_operators.jl:230-244."""
    from .operate import operate

    op = map_to_zero_operator(f.s, xs, dims, **(truncate_kwargs or {}))
    return operate(op, f, **kw)


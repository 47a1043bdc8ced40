"""Tensor cross interpolation (TCI) of a black-box function into a quantics
tensor network function on a path-shaped map.

The reference exposes this as the TCI package extension
(ext/ITensorNumericalAnalysisTCIExt/tci_util.jl:21-55): a function of n real
variables is sampled on the digit grid through the index map
(input_to_scalars, tci_util.jl:57-66) and ITensorTCI.interpolate builds the
network.  The interpolation algorithm itself lives in ITensorTCI (not part of
the reference); this module restates the standard two-site scheme (TCI2 with
nested pivots): for every bond the matrix
    Pi[(i, s_l), (s_{l+1}, j)] = f(i, s_l, s_{l+1}, j),  i in I_{l-1}, j in J_{l+2}
is sampled in one batch and factorised by cross (ACA with full pivoting) up to
a relative tolerance; its pivots become the new I_l, J_{l+1}.  The result is
the cross form T_1 P_1^-1 T_2 ... T_L turned into site tensors.

Sampling is batched: the callable receives an (N, n_dims) array of points and
returns N values, so an ITensorNetworkFunction (evaluated on the device) or any
vectorised NumPy function can be interpolated.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _aca_full(M: np.ndarray, tol: float, maxrank: int):
    """Cross (adaptive cross approximation with full pivoting) of the sampled
    block M on the device (tnfa_cross): pivot rows and columns, the largest
    entry left in the residual, and max|M|."""
    M = np.ascontiguousarray(np.asarray(M, dtype=np.float64))
    rows, cols = M.shape
    if M.size == 0:
        return [], [], 0.0, 0.0
    k = max(0, min(int(maxrank), rows, cols))
    pr = (C.c_int32 * max(k, 1))()
    pc = (C.c_int32 * max(k, 1))()
    rk = C.c_int32(0)
    err = (C.c_double * 2)()
    _lib.default_context().call("tnfa_cross", M.ctypes.data_as(C.c_void_p), _lib.MEM_HOST, rows, cols,
                                float(tol), int(maxrank), pr, pc, C.byref(rk), err)
    n = rk.value
    return list(pr[:n]), list(pc[:n]), float(err[0]), float(err[1])


class _PathSampler:
    """Maps multi-indices (one digit value per path position) to points."""

    def __init__(self, f, legs, ndims: int):
        self.f = f
        self.legs = legs  # per position: SiteLeg
        self.ndims = ndims

    def __call__(self, idx: np.ndarray) -> np.ndarray:
        # idx: (N, L) digit values
        X = np.zeros((idx.shape[0], self.ndims))
        for pos, l in enumerate(self.legs):
            X[:, l.dim - 1] += idx[:, pos] * float(l.base) ** (-l.digit)
        return np.asarray(self.f(X))


def tci_path(sample, d: list, tol: float = 1e-10, maxbonddim: int = 64, nsweeps: int = 20,
             initial_pivot=None):
    """Two-site TCI on a path with local dimensions d.  sample(idx) evaluates
    the function at an (N, L) array of multi-indices.  Returns (cores, info):
    cores[l] of shape (r_{l-1}, d_l, r_l) with r_0 = r_L = 1."""
    L = len(d)
    if initial_pivot is None:
        # the largest |f| among a few hundred random digit strings
        rng = np.random.default_rng(0)
        cand = np.stack([rng.integers(0, dl, 256) for dl in d], axis=1)
        piv = cand[int(np.argmax(np.abs(sample(cand))))]
    else:
        piv = np.asarray(initial_pivot, dtype=np.int64)
    # I[l]: list of tuples for positions 0..l-1 (I[0] = [()]); J[l]: positions l..L-1 (J[L] = [()])
    I = [[tuple(piv[:l])] for l in range(L + 1)]
    J = [[tuple(piv[l:])] for l in range(L + 1)]
    fmax = abs(float(sample(piv[None, :])[0]))
    rng = np.random.default_rng(1)
    errs, ranks_prev = [], None
    for sweep in range(nsweeps):
        bond_err = []
        bonds = range(L - 1) if sweep % 2 == 0 else range(L - 2, -1, -1)
        for b in bonds:  # bond between positions b and b + 1
            Il, Jr = I[b], J[b + 2]
            rows = [il + (s,) for il in Il for s in range(d[b])]
            cols = [(s,) + jr for s in range(d[b + 1]) for jr in Jr]
            idx = np.array([r + c for r in rows for c in cols], dtype=np.int64).reshape(-1, L)
            Pi = sample(idx).reshape(len(rows), len(cols))
            fmax = max(fmax, float(np.max(np.abs(Pi))))
            pr, pc, err, _ = _aca_full(Pi, tol * fmax / max(np.max(np.abs(Pi)), 1e-300), maxbonddim)
            if not pr:  # an all-zero block: keep the old pivots
                continue
            I[b + 1] = [rows[i] for i in pr]
            J[b + 1] = [cols[j] for j in pc]
            bond_err.append(err / max(fmax, 1e-300))
        # global check: the cross form against f at random digit strings; the
        # worst points join every pivot set (nested: prefixes and suffixes)
        cores = _assemble(sample, d, I, J)
        test = np.stack([rng.integers(0, dl, 512) for dl in d], axis=1)
        miss = np.abs(_mps_values(cores, test) - sample(test))
        bad = np.argsort(miss)[::-1][:4]
        bad = [int(i) for i in bad if miss[i] > tol * fmax]
        for i in bad:
            pt = tuple(int(x) for x in test[i])
            for l in range(1, L):
                if pt[:l] not in I[l] and len(I[l]) < maxbonddim:
                    I[l] = I[l] + [pt[:l]]
                if pt[l:] not in J[l] and len(J[l]) < maxbonddim:
                    J[l] = J[l] + [pt[l:]]
        e = max(bond_err + [float(np.max(miss)) / max(fmax, 1e-300)])
        errs.append(e)
        ranks = [len(I[l]) for l in range(1, L)]
        if sweep >= 1 and e <= tol and not bad and ranks == ranks_prev:
            break
        ranks_prev = ranks
    return _assemble(sample, d, I, J), {"sweeps": len(errs), "errors": errs,
                                        "ranks": [len(I[l]) for l in range(1, L)]}


# ------------------------------------------------------------------ trees --
class _TreeCross:
    """Nested pivot sets of a tree.  Vertices are 0..n-1 with adjacency nbrs;
    for a directed edge (u, v), side[(u, v)] holds the vertices on u's side and
    P[(u, v)] the pivots there: rows of digit values over all n vertices, zero
    off the side, so that pivots of disjoint sides combine by addition."""

    def __init__(self, nbrs, d):
        self.nbrs, self.d, self.n = nbrs, d, len(d)
        self.side = {}
        for u in range(self.n):
            for v in nbrs[u]:
                seen, stack = {u}, [u]
                while stack:
                    x = stack.pop()
                    for y in nbrs[x]:
                        if y not in seen and not (x == u and y == v):
                            seen.add(y)
                            stack.append(y)
                self.side[(u, v)] = np.array(sorted(seen), dtype=np.int64)
        self.P = {}

    def restrict(self, pts, u, v):
        out = np.zeros_like(pts)
        cols = self.side[(u, v)]
        out[:, cols] = pts[:, cols]
        return out

    def block(self, u, exclude):
        """Assignments over side(u, exclude): pivots of u's other neighbours
        combined, then u's own digit (fastest)."""
        rows = np.zeros((1, self.n), dtype=np.int64)
        for w in self.nbrs[u]:
            if w == exclude:
                continue
            A = self.P[(w, u)]
            rows = (rows[:, None, :] + A[None, :, :]).reshape(-1, self.n)
        e = np.zeros(self.n, dtype=np.int64)
        e[u] = 1
        s = np.arange(self.d[u])
        return (rows[:, None, :] + s[None, :, None] * e[None, None, :]).reshape(-1, self.n)

    def add_unique(self, key, new_rows, cap):
        cur = self.P[key]
        have = {tuple(r) for r in cur}
        keep = [r for r in new_rows if tuple(r) not in have]
        if keep:
            self.P[key] = np.concatenate([cur, np.array(keep[: max(0, cap - len(cur))],
                                                        dtype=np.int64).reshape(-1, self.n)])


def _tree_order(nbrs, root):
    parent = {root: -1}
    order = [root]
    for x in order:
        for y in nbrs[x]:
            if y not in parent:
                parent[y] = x
                order.append(y)
    return order, parent


def _tree_assemble(sample, tc: _TreeCross, root: int):
    """Cross form -> one tensor per vertex, axes (digit, neighbours in nbrs
    order).  The bond of edge (child c, parent p) is indexed by P[(c, p)] on
    both ends: the parent's tensor is sampled on it directly and the child's
    absorbs the pivot matrix M[(c, p)]^-1 (least squares)."""
    order, parent = _tree_order(tc.nbrs, root)
    cores = {}
    for v in order:
        parts = [tc.P[(w, v)] for w in tc.nbrs[v]]
        idx = np.zeros((1, tc.n), dtype=np.int64)
        for A in parts:
            idx = (idx[:, None, :] + A[None, :, :]).reshape(-1, tc.n)
        e = np.zeros(tc.n, dtype=np.int64)
        e[v] = 1
        idx = (idx[:, None, :] + np.arange(tc.d[v])[None, :, None] * e[None, None, :]).reshape(-1, tc.n)
        T = np.asarray(sample(idx)).reshape([len(A) for A in parts] + [tc.d[v]])
        T = np.moveaxis(T, -1, 0)  # (digit, neighbours...)
        p = parent[v]
        if p >= 0:
            k = 1 + tc.nbrs[v].index(p)
            Pc, Pp = tc.P[(v, p)], tc.P[(p, v)]
            M = np.asarray(sample((Pc[:, None, :] + Pp[None, :, :]).reshape(-1, tc.n))).reshape(len(Pc), len(Pp))
            Tm = np.moveaxis(T, k, -1)
            sh = Tm.shape
            X = np.linalg.lstsq(M.T, Tm.reshape(-1, sh[-1]).T, rcond=None)[0].T
            T = np.moveaxis(X.reshape(sh[:-1] + (len(Pc),)), -1, k)
        cores[v] = T
    return cores


def _tree_values(cores, nbrs, root, idx):
    """Contract the assembled tree at the rows of idx (N, n)."""
    order, parent = _tree_order(nbrs, root)
    N = idx.shape[0]
    msg = {}
    for v in reversed(order):
        S = cores[v][idx[:, v]]  # (N, neighbours...)
        S = S.astype(np.result_type(S, float))
        # contract the children's messages, last neighbour axis first
        for k in reversed(range(len(nbrs[v]))):
            w = nbrs[v][k]
            if w == parent[v]:
                continue
            S = np.moveaxis(S, 1 + k, -1)
            S = np.einsum("p...k,pk->p...", S, msg[w])
        msg[v] = S.reshape(N, -1)
    return msg[root][:, 0]


def tci_tree(sample, nbrs, d, tol: float = 1e-10, maxbonddim: int = 64, nsweeps: int = 20,
             initial_pivot=None, root: int = 0):
    """Two-site TCI on a tree (the generalisation of tci_path: every edge
    carries nested pivot sets for its two sides; an update samples the block
    [u's side x v's side] built from the neighbours' pivots and re-selects both
    by ACA).  sample(idx) evaluates f at an (N, n) array of digit values,
    column v = vertex v.  Returns (cores, info) with cores[v] of axes (digit,
    neighbours in nbrs[v] order), ready for _tree_values / layout reordering."""
    n = len(d)
    tc = _TreeCross(nbrs, d)
    if initial_pivot is None:
        rng = np.random.default_rng(0)
        cand = np.stack([rng.integers(0, dv, 256) for dv in d], axis=1)
        piv = cand[int(np.argmax(np.abs(sample(cand))))]
    else:
        piv = np.asarray(initial_pivot, dtype=np.int64)
    piv = piv.reshape(1, n)
    for (u, v) in tc.side:
        tc.P[(u, v)] = tc.restrict(piv, u, v)
    fmax = abs(float(np.asarray(sample(piv))[0]))
    order, parent = _tree_order(nbrs, root)
    edges = [(parent[v], v) for v in order if parent[v] >= 0]
    rng = np.random.default_rng(1)
    errs, ranks_prev = [], None
    for sweep in range(nsweeps):
        bond_err = []
        for (u, v) in (edges if sweep % 2 == 0 else edges[::-1]):
            rows, cols = tc.block(u, v), tc.block(v, u)
            Pi = np.asarray(sample((rows[:, None, :] + cols[None, :, :]).reshape(-1, n))).reshape(len(rows), len(cols))
            fmax = max(fmax, float(np.max(np.abs(Pi))))
            pr, pc, err, _ = _aca_full(Pi, tol * fmax / max(np.max(np.abs(Pi)), 1e-300), maxbonddim)
            if not pr:
                continue
            tc.P[(u, v)] = rows[pr]
            tc.P[(v, u)] = cols[pc]
            bond_err.append(err / max(fmax, 1e-300))
        cores = _tree_assemble(sample, tc, root)
        test = np.stack([rng.integers(0, dv, 512) for dv in d], axis=1)
        miss = np.abs(_tree_values(cores, nbrs, root, test) - np.asarray(sample(test)))
        bad = [int(i) for i in np.argsort(miss)[::-1][:4] if miss[i] > tol * fmax]
        for i in bad:
            pt = test[i:i + 1]
            for (u, v) in tc.side:
                tc.add_unique((u, v), tc.restrict(pt, u, v), maxbonddim)
        e = max(bond_err + [float(np.max(miss)) / max(fmax, 1e-300)])
        errs.append(e)
        ranks = [len(tc.P[(v, u)]) for (u, v) in edges]
        if sweep >= 1 and e <= tol and not bad and ranks == ranks_prev:
            break
        ranks_prev = ranks
    cores = _tree_assemble(sample, tc, root)
    return cores, {"sweeps": len(errs), "errors": errs,
                   "ranks": [len(tc.P[(v, u)]) for (u, v) in edges]}


def _mps_values(cores, idx):
    out = np.ones((idx.shape[0], 1))
    for l, A in enumerate(cores):
        out = np.einsum("pa,pab->pb", out, A[:, idx[:, l], :].transpose(1, 0, 2))
    return out[:, 0]


def _assemble(sample, d, I, J):
    """Cross form -> site tensors: A_l = T_l P_l^-1 (l < L - 1), A_{L-1} = T_{L-1}."""
    L = len(d)
    cores = []
    for l in range(L):
        Il, Jr = I[l], J[l + 1]
        idx = np.array([il + (s,) + jr for il in Il for s in range(d[l]) for jr in Jr],
                       dtype=np.int64).reshape(-1, L)
        T = sample(idx).reshape(len(Il), d[l], len(Jr))
        if l < L - 1:
            Ip = I[l + 1]
            idxp = np.array([ip + jr for ip in Ip for jr in Jr], dtype=np.int64).reshape(-1, L)
            P = sample(idxp).reshape(len(Ip), len(Jr))
            A = np.linalg.lstsq(P.T, T.reshape(-1, len(Jr)).T, rcond=None)[0].T.reshape(len(Il), d[l], len(Ip))
        else:
            A = T
        cores.append(A)
    return cores


def interpolate(f, s, tol: float = 1e-10, maxbonddim: int = 64, nsweeps: int = 20,
                initial_pivot=None, dtype=None):
    """Interpolate f (vectorised: (N, n_dims) points -> N values, or an
    ITensorNetworkFunction) into an ITensorNetworkFunction on the map s, a
    tree with one digit leg per vertex (ITensorTCI.interpolate through
    tci_util.jl:21-55, which asserts is_tree(s) and maps each vertex to one
    (dimension, digit)).  Paths (2-D combs included) use tci_path, other trees
    tci_tree."""
    from .network import ITensorNetworkFunction

    lay = s.layout
    g = s.graph
    verts = s.vertices()
    nedges = sum(len(g.neighbors(v)) for v in verts) // 2
    if len(lay.order) < 2 or len(g.components()) != 1 or nedges != len(verts) - 1:
        raise ValueError("interpolate needs a connected tree")
    if any(len(s.legs[v]) != 1 for v in verts):
        raise ValueError("interpolate needs one digit leg per vertex")
    if any(len(g.neighbors(v)) > 2 for v in verts):
        return _interpolate_tree(f, s, tol, maxbonddim, nsweeps, initial_pivot, dtype)
    ends = [v for v in verts if len(g.neighbors(v)) <= 1]
    # walk the path from its first end in vertex order
    path, prev, v = [], None, ends[0]
    while v is not None:
        path.append(v)
        nxt = [w for w in g.neighbors(v) if w != prev]
        prev, v = v, (nxt[0] if nxt else None)
    legs = [s.legs[v][0] for v in path]
    dims = s.dimensions()
    ndims = max(dims)
    if isinstance(f, ITensorNetworkFunction):
        fn = f
        f = lambda X: fn.evaluate_batch(X, list(range(1, ndims + 1)))
    sampler = _PathSampler(f, legs, ndims)
    d = [l.base for l in legs]
    pivot = None
    if initial_pivot is not None:
        iv = s.calculate_ind_values(initial_pivot, list(range(1, ndims + 1)))
        pivot = [iv[l] for l in legs]
    cores, info = tci_path(sampler, d, tol=tol, maxbonddim=maxbonddim, nsweeps=nsweeps,
                           initial_pivot=pivot)
    # path position k -> layout tensor [site, parent, children]
    pos = {v: k for k, v in enumerate(path)}
    ts = {}
    for i, v in enumerate(lay.order):
        A = cores[pos[v]]  # (left, site, right) along the path
        p = lay.parent[i]
        kids = lay.children[i]
        left_nb = path[pos[v] - 1] if pos[v] > 0 else None
        right_nb = path[pos[v] + 1] if pos[v] + 1 < len(path) else None
        axis_of = {}  # neighbour -> axis of A
        if left_nb is not None:
            axis_of[left_nb] = 0
        if right_nb is not None:
            axis_of[right_nb] = 2
        order = [1]
        if p >= 0:
            order.append(axis_of[lay.order[p]])
        order += [axis_of[lay.order[c]] for c in kids]
        # drop the dim-1 outer axes that are not bonds, then reorder
        keep = [1] + [a for a in (0, 2) if a in axis_of.values()]
        B = A.reshape([A.shape[a] for a in sorted(keep)])
        perm = [sorted(keep).index(a) for a in order]
        B = np.transpose(B, perm)
        if p < 0:
            B = B.reshape(B.shape[:1] + (1,) + B.shape[1:])
        ts[v] = B
    out = ITensorNetworkFunction.from_tensors(s, ts, dtype=dtype)
    out.tci_info = info
    return out


def _interpolate_tree(f, s, tol, maxbonddim, nsweeps, initial_pivot, dtype):
    """interpolate() on a tree that is not a path: tci_tree over the layout's
    vertex order (position i = lay.order[i], root 0), then each tensor's axes
    reordered to the layout [site, parent, children...]."""
    from .network import ITensorNetworkFunction

    lay = s.layout
    g = s.graph
    pos = {v: i for i, v in enumerate(lay.order)}
    nbrs = [[pos[w] for w in g.neighbors(v)] for v in lay.order]
    legs = [s.legs[v][0] for v in lay.order]
    ndims = max(s.dimensions())
    if isinstance(f, ITensorNetworkFunction):
        fn = f
        f = lambda X: fn.evaluate_batch(X, list(range(1, ndims + 1)))
    sampler = _PathSampler(f, legs, ndims)
    d = [l.base for l in legs]
    pivot = None
    if initial_pivot is not None:
        iv = s.calculate_ind_values(initial_pivot, list(range(1, ndims + 1)))
        pivot = [iv[l] for l in legs]
    cores, info = tci_tree(sampler, nbrs, d, tol=tol, maxbonddim=maxbonddim, nsweeps=nsweeps,
                           initial_pivot=pivot, root=0)
    ts = {}
    for i, v in enumerate(lay.order):
        A = cores[i]
        p = lay.parent[i]
        perm = [0] + ([1 + nbrs[i].index(p)] if p >= 0 else []) + [1 + nbrs[i].index(c) for c in lay.children[i]]
        B = np.transpose(A, perm)
        if p < 0:
            B = B.reshape(B.shape[:1] + (1,) + B.shape[1:])
        ts[v] = B
    out = ITensorNetworkFunction.from_tensors(s, ts, dtype=dtype)
    out.tci_info = info
    return out

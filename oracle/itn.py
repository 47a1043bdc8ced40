"""Labelled-tensor restatement of ITensorNumericalAnalysis.jl (test oracle).

Tensors carry Index objects (dimension + identity) and contract over shared
indices, as ITensors.jl does.  Networks are dicts vertex -> Tensor over a
named graph.  Functions follow the reference file:line cited in each
docstring.  Pure numpy; FP64 / complex128 throughout.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field
from math import comb

import numpy as np

__all__ = [
    "Index", "Tensor", "contract", "SiteMap", "Net",
    "grid_graph", "comb_tree_graph", "path_graph", "binary_tree_graph",
    "siteinds", "complex_siteinds", "digits_greedy", "calculate_ind_values", "calculate_p",
    "const_itn", "exp_itn", "cosh_itn", "sinh_itn", "tanh_itn", "cos_itn", "sin_itn", "poly_itn",
    "delta_p", "random_net", "net_add", "net_multiply", "net_scale",
    "evaluate", "evaluate_batch", "integrate", "dense", "dense_grid_1d",
    "forward_shift_terms", "backward_shift_terms", "stencil_terms", "apply_terms_dense",
    "bond_spectrum", "gradient", "aca_full",
]

_next_id = itertools.count()


class Index:
    __slots__ = ("dim", "tag", "uid")

    def __init__(self, dim: int, tag: str = ""):
        self.dim, self.tag, self.uid = int(dim), tag, next(_next_id)

    def __repr__(self):
        return f"Index({self.dim},{self.tag!r})"


class Tensor:
    def __init__(self, arr, inds):
        self.arr = np.asarray(arr)
        self.inds = list(inds)
        assert self.arr.ndim == len(self.inds), (self.arr.shape, self.inds)

    def __mul__(self, other):
        if np.isscalar(other):
            return Tensor(self.arr * other, self.inds)
        common = [i for i in self.inds if i in other.inds]
        ax_a = [self.inds.index(i) for i in common]
        ax_b = [other.inds.index(i) for i in common]
        arr = np.tensordot(self.arr, other.arr, axes=(ax_a, ax_b))
        inds = [i for i in self.inds if i not in common] + [i for i in other.inds if i not in common]
        return Tensor(arr, inds)

    __rmul__ = __mul__

    def permute(self, inds):
        return Tensor(np.transpose(self.arr, [self.inds.index(i) for i in inds]), inds)

    def scalar(self):
        assert not self.inds
        return self.arr[()]


def onehot(ind: Index, val: int) -> Tensor:
    v = np.zeros(ind.dim)
    v[val] = 1.0
    return Tensor(v, [ind])


def delta(inds) -> Tensor:
    """ITensors delta: 1 where all indices agree (all ones for one index)."""
    inds = list(inds)
    if not inds:
        return Tensor(np.ones(()), [])
    d = inds[0].dim
    a = np.zeros([i.dim for i in inds])
    for x in range(d):
        a[(x,) * len(inds)] = 1.0
    return Tensor(a, inds)


def contract(tensors) -> Tensor:
    """Greedy pairwise contraction (smallest result first); exact."""
    ts = list(tensors)
    if not ts:
        return Tensor(np.ones(()), [])
    while len(ts) > 1:
        best = None
        for a in range(len(ts)):
            for b in range(a + 1, len(ts)):
                common = set(ts[a].inds) & set(ts[b].inds)
                if not common and best is not None:
                    continue
                size = 1
                for i in set(ts[a].inds) ^ set(ts[b].inds):
                    size *= i.dim
                key = (0 if common else 1, size)
                if best is None or key < best[0]:
                    best = (key, a, b)
        _, a, b = best
        t = ts[a] * ts[b]
        ts = [x for k, x in enumerate(ts) if k not in (a, b)] + [t]
    return ts[0]


# ---------------------------------------------------------------- graphs ----
def grid_graph(dims):
    """NamedGraphs named_grid: CartesianIndices vertex order."""
    ranges = [range(1, d + 1) for d in dims]
    verts = [tuple(reversed(t)) for t in itertools.product(*reversed(ranges))]
    edges = []
    for v in verts:
        for ax in range(len(dims)):
            if v[ax] < dims[ax]:
                w = list(v)
                w[ax] += 1
                edges.append((v, tuple(w)))
    return verts, edges


def path_graph(L):
    return grid_graph((L, 1))


def comb_tree_graph(dims):
    """NamedGraphs named_comb_tree((nx, ny)): backbone (i,1)-(i+1,1), teeth (i,j)-(i,j+1)."""
    nx, ny = dims
    verts = [(i, j) for j in range(1, ny + 1) for i in range(1, nx + 1)]
    edges = [((i, 1), (i + 1, 1)) for i in range(1, nx)]
    edges += [((i, j - 1), (i, j)) for i in range(1, nx + 1) for j in range(2, ny + 1)]
    return verts, edges


def binary_tree_graph(n):
    verts = list(range(1, n + 1))
    edges = [(i, c) for i in verts for c in (2 * i, 2 * i + 1) if c <= n]
    return verts, edges


# ------------------------------------------------------------ index maps ----
@dataclass
class SiteMap:
    """IndsNetworkMap: vertices, edges, site indices per vertex and the
    index -> (dimension, digit, is_real) map (src/indsnetworkmap.jl:9-13)."""

    verts: list
    edges: list
    site: dict                 # vertex -> [Index]
    info: dict                 # Index -> (dim, digit, is_real)
    base: int = 2
    is_complex: bool = False

    def neighbors(self, v):
        return [b for a, b in self.edges if a == v] + [a for a, b in self.edges if b == v]

    def dims(self):
        out = []
        for v in self.verts:
            for i in self.site[v]:
                d = self.info[i][0]
                if d not in out:
                    out.append(d)
        return sorted(out)

    def dimension_vertices(self, dim):
        return [v for v in self.verts if any(self.info[i][0] == dim for i in self.site[v])]

    def vertex(self, dim, digit):
        (v,) = [v for v in self.verts for i in self.site[v]
                if self.info[i][0] == dim and self.info[i][1] == digit and self.info[i][2]]
        return v

    def ind(self, dim, digit, real=True):
        (i,) = [i for v in self.verts for i in self.site[v]
                if self.info[i][:2] == (dim, digit) and self.info[i][2] == real]
        return i

    def scalar(self, ind, value):
        """index_value_to_scalar (src/IndexMaps/realindexmap.jl:13-15,
        src/IndexMaps/complexindexmap.jl:25-32)."""
        d, k, real = self.info[ind]
        w = value * float(ind.dim) ** (-k)
        return w if real else 1j * w

    def path(self, a, b):
        prev = {a: None}
        q = [a]
        for v in q:
            for w in self.neighbors(v):
                if w not in prev:
                    prev[w] = v
                    q.append(w)
        out = [b]
        while out[-1] != a:
            out.append(prev[out[-1]])
        return out[::-1]


def _default_dv(verts, map_dimension):
    """src/digit_inds.jl:17-21."""
    return [verts[i::map_dimension] for i in range(map_dimension)]


def siteinds(graph, dimension_vertices=None, base=2, map_dimension=1) -> SiteMap:
    """continuous_siteinds (src/digit_inds.jl:72-86 + src/IndexMaps/realindexmap.jl:53-72)."""
    verts, edges = graph
    dv = dimension_vertices or _default_dv(verts, map_dimension)
    site = {v: [] for v in verts}
    info = {}
    for d, vs in enumerate(dv, start=1):
        for k, v in enumerate(vs, start=1):
            i = Index(base, f"V{v} Dim{d} Dig{k}")
            site[v].append(i)
            info[i] = (d, k, True)
    return SiteMap(list(verts), list(edges), site, info, base, False)


def complex_siteinds(graph, real_dv=None, imag_dv=None, base=2, map_dimension=1) -> SiteMap:
    """complex_continuous_siteinds (src/digit_inds.jl:88-115, complexindexmap.jl:75-114)."""
    verts, edges = graph
    rdv = real_dv or _default_dv(verts, map_dimension)
    idv = imag_dv or _default_dv(verts, map_dimension)
    site = {v: [] for v in verts}
    info = {}
    for real, dv in ((True, rdv), (False, idv)):
        for d, vs in enumerate(dv, start=1):
            for k, v in enumerate(vs, start=1):
                i = Index(base, f"{'Re' if real else 'Im'} V{v} Dim{d} Dig{k}")
                site[v].append(i)
                info[i] = (d, k, real)
    return SiteMap(list(verts), list(edges), site, info, base, True)


def digits_greedy(x: float, base: int, L: int) -> list[int]:
    """set_ind_values! (src/IndexMaps/abstractindexmap.jl:121-138): for digit
    k = 1..L pick the largest v with x_rn >= v * base^-k and subtract it."""
    out, rem = [], float(x)
    for k in range(1, L + 1):
        invb = 1.0 / float(base) ** k
        val = base - 1
        while True:
            if rem >= abs(val * invb):
                rem -= abs(val * invb)
                break
            val -= 1
        out.append(val)
    return out


def calculate_ind_values(s: SiteMap, xs, dims) -> dict:
    """src/IndexMaps/realindexmap.jl:67-76 and complexindexmap.jl:116-132."""
    out = {}
    for x, d in zip(xs, dims):
        for real in ((True, False) if s.is_complex else (True,)):
            part = float(np.real(x)) if real else float(np.imag(x))
            inds = sorted((i for i, (dd, k, r) in s.info.items() if dd == d and r == real),
                          key=lambda i: s.info[i][1])
            if not inds:
                continue
            vals = digits_greedy(part, inds[0].dim, len(inds))
            for i, v in zip(inds, vals):
                out[i] = v
    return out


def calculate_p(s: SiteMap, ivmap: dict, dims):
    """src/IndexMaps/abstractindexmap.jl:103-119."""
    return [sum(s.scalar(i, v) for i, v in ivmap.items() if s.info[i][0] == d) for d in dims]


# -------------------------------------------------------------- networks ----
@dataclass
class Net:
    """ITensorNetworkFunction: tensors per vertex + link index per edge."""

    s: SiteMap
    T: dict
    link: dict = field(default_factory=dict)  # frozenset({u, v}) -> Index

    def copy(self):
        return Net(self.s, dict(self.T), dict(self.link))

    def linkdims(self):
        return {k: i.dim for k, i in self.link.items()}


def _new_links(s: SiteMap, dim: int) -> dict:
    return {frozenset(e): Index(dim, f"L{e}") for e in s.edges}


def _vertex_links(net: Net, v):
    return [net.link[frozenset((v, w))] for w in net.s.neighbors(v)]


def random_net(s: SiteMap, link_space=1, rng=None, normalize=False) -> Net:
    """random_tensornetwork (src/elementary_functions.jl:209-221), numpy Gaussian."""
    rng = np.random.default_rng(rng)
    link = _new_links(s, link_space)
    net = Net(s, {}, link)
    for v in s.verts:
        inds = s.site[v] + _vertex_links(net, v)
        a = rng.standard_normal([i.dim for i in inds])
        if normalize:
            a = a / np.linalg.norm(a)
        net.T[v] = Tensor(a, inds)
    return net


def const_itn(s: SiteMap, c=1.0, linkdim=1) -> Net:
    """src/elementary_functions.jl:16-26 with c_tensor src/utils.jl:42-47."""
    V = len(s.verts)
    if np.isreal(c) and np.real(c) < 0:
        cp = (complex(c) / linkdim) ** (1.0 / V)
    else:
        cp = (c / linkdim) ** (1.0 / V)
    net = Net(s, {}, _new_links(s, linkdim))
    for v in s.verts:
        t = delta(_vertex_links(net, v))
        for i in s.site[v]:
            t = t * Tensor(np.ones(i.dim), [i])
        net.T[v] = t * cp
    return net


def exp_itn(s: SiteMap, k=1.0, a=0.0, c=1.0, dim=1) -> Net:
    """src/elementary_functions.jl:30-53."""
    net = const_itn(s)
    dv = s.dimension_vertices(dim)
    Lx = len(dv)
    for v in dv:
        t = Tensor(np.ones(()), [])
        for i in s.site[v]:
            if s.info[i][0] == dim:
                vals = np.array([s.scalar(i, x) for x in range(i.dim)])
                t = t * Tensor(np.exp(k * vals), [i])
            else:
                t = t * Tensor(np.ones(i.dim), [i])
        t = t * np.exp(a / Lx)
        t = t * delta(_vertex_links(net, v))
        net.T[v] = t
    net.T[dv[0]] = net.T[dv[0]] * c
    return net


def net_add(f: Net, g: Net) -> Net:
    """ITensorNetworks add (direct sum on every link; semantics as src/fixes.jl:39-91)."""
    s = f.s
    link = {e: Index(f.link[e].dim + g.link[e].dim, "sum") for e in f.link}
    out = Net(s, {}, link)
    for v in s.verts:
        nb = s.neighbors(v)
        lf = [f.link[frozenset((v, w))] for w in nb]
        lg = [g.link[frozenset((v, w))] for w in nb]
        lo = [link[frozenset((v, w))] for w in nb]
        site = s.site[v]
        A = f.T[v].permute(site + lf).arr
        B = g.T[v].permute(site + lg).arr
        dt = np.result_type(A, B)
        if not nb:
            out.T[v] = Tensor(A + B, site)
            continue
        O = np.zeros([i.dim for i in site] + [i.dim for i in lo], dtype=dt)
        ns = len(site)
        O[(slice(None),) * ns + tuple(slice(0, i.dim) for i in lf)] = A
        O[(slice(None),) * ns + tuple(slice(a.dim, a.dim + b.dim) for a, b in zip(lf, lg))] = B
        out.T[v] = Tensor(O, site + lo)
    return out


def net_scale(f: Net, v, c) -> Net:
    out = f.copy()
    out.T[v] = out.T[v] * c
    return out


def net_multiply(f: Net, g: Net) -> Net:
    """Hadamard product on shared vertices (src/elementary_operators.jl:260-292)."""
    s = f.s
    link = {e: Index(f.link[e].dim * g.link[e].dim, "prod") for e in f.link}
    out = Net(s, {}, link)
    for v in s.verts:
        nb = s.neighbors(v)
        lf = [f.link[frozenset((v, w))] for w in nb]
        lg = [g.link[frozenset((v, w))] for w in nb]
        site = s.site[v]
        A = f.T[v].permute(site + lf).arr
        B = g.T[v].permute(site + lg).arr
        ns, nl = len(site), len(nb)
        # out[s, (a1 b1), (a2 b2)...] = A[s, a...] B[s, b...]
        letters = "abcdefghijklmnopqrstuvwxyz"
        sl = letters[:ns]
        al = letters[ns:ns + nl]
        bl = letters[ns + nl:ns + 2 * nl]
        outl = sl + "".join(x + y for x, y in zip(al, bl))
        C = np.einsum(f"{sl}{al},{sl}{bl}->{outl}", A, B)
        C = C.reshape([i.dim for i in site] + [x.dim * y.dim for x, y in zip(lf, lg)])
        out.T[v] = Tensor(C, site + [link[frozenset((v, w))] for w in nb])
    return out


def cosh_itn(s, k=1.0, a=0.0, c=1.0, dim=1):
    """src/elementary_functions.jl:57-68."""
    return net_add(exp_itn(s, k, a, 0.5 * c, dim), exp_itn(s, -k, -a, 0.5 * c, dim))


def sinh_itn(s, k=1.0, a=0.0, c=1.0, dim=1):
    """src/elementary_functions.jl:72-83."""
    return net_add(exp_itn(s, k, a, 0.5 * c, dim), exp_itn(s, -k, -a, -0.5 * c, dim))


def tanh_itn(s, k=1.0, a=0.0, c=1.0, nterms=20, dim=1):
    """src/elementary_functions.jl:87-105."""
    first = s.dimension_vertices(dim)[0]
    psi = const_itn(s)
    for n in range(1, nterms + 1):
        t = exp_itn(s, -2 * k * n, -2 * n * a, 1.0, dim)
        t = net_scale(t, first, 2 * (-1) ** n)
        psi = net_add(psi, t)
    return net_scale(psi, first, c)


def cos_itn(s, k=1.0, a=0.0, c=1.0, dim=1):
    """src/elementary_functions.jl:109-120 (complex exponentials)."""
    return net_add(exp_itn(s, 1j * k, 1j * a, 0.5 * c, dim), exp_itn(s, -1j * k, -1j * a, 0.5 * c, dim))


def sin_itn(s, k=1.0, a=0.0, c=1.0, dim=1):
    """src/elementary_functions.jl:124-135 (complex exponentials)."""
    return net_add(exp_itn(s, 1j * k, 1j * a, -0.5j * c, dim),
                   exp_itn(s, -1j * k, -1j * a, 0.5j * c, dim))


def _f_alpha_beta(alpha, beta):
    """src/polynomialutils.jl:4-6."""
    return max(0, beta - sum(alpha)) if len(alpha) else max(0, beta)


def _coeff(N, alpha, beta):
    """src/polynomialutils.jl:9-16."""
    if N == 1:
        return 1
    return int(np.prod([comb(_f_alpha_beta(alpha[: N - 1 - i], beta), alpha[N - 1 - i])
                        for i in range(1, N)]))


def _q_n_tensor(N, sinds, alphas, beta, xivals):
    """Q_N_tensor (src/polynomialutils.jl:19-41); ComplexF64 as in the reference."""
    n = beta.dim - 1
    arr = np.zeros([i.dim for i in sinds] + [n + 1] * N, dtype=complex)
    for si in itertools.product(*[range(i.dim) for i in sinds]):
        xi = sum(xivals[j][k] for j, k in enumerate(si))
        for li in itertools.product(range(n + 1), repeat=N):
            al, be = li[: N - 1], li[N - 1]
            f = _f_alpha_beta(al, be)
            arr[si + li] = _coeff(N, al, be) * (xi ** f)
    return Tensor(arr, list(sinds) + list(alphas) + [beta])


def _transfer_tensor(phys, beta, alphas):
    """src/polynomialutils.jl:45-68."""
    dims = [i.dim for i in phys]
    vd = beta.dim
    N = len(alphas)
    arr = np.zeros(dims + [vd] + [vd] * N)
    for si in itertools.product(*[range(d) for d in dims]):
        for j in range(vd):
            if N:
                for ks in itertools.product(range(vd), repeat=N):
                    if sum(ks) == j:
                        arr[si + (j,) + ks] = 1.0
            else:
                arr[si + (j,)] = 1.0 if j == 0 else 0.0
    return Tensor(arr, list(phys) + [beta] + list(alphas))


def poly_itn(s: SiteMap, coeffs, dim=1, k=1.0, c=1.0) -> Net:
    """src/elementary_functions.jl:139-207 on a tree (the BFS tree is the tree)."""
    n = len(coeffs)
    if n == 1:
        return const_itn(s, c=coeffs[0])
    coeffs = [cf * k ** i for i, cf in enumerate(coeffs)]
    psi = const_itn(s, linkdim=n)
    dv = s.dimension_vertices(dim)
    src = dv[0]
    for v in dv:
        sinds = s.site[v]
        sd = [i for i in sinds if s.info[i][0] == dim]
        snd = [i for i in sinds if s.info[i][0] != dim]
        xivals = [[s.scalar(i, x) for x in range(i.dim)] for i in sd]
        nb = s.neighbors(v)
        if v != src:
            toward = s.path(v, src)[1]
            beta = psi.link[frozenset((v, toward))]
            alphas = [psi.link[frozenset((v, w))] for w in nb if w != toward]
            t = _q_n_tensor(len(nb), sd, alphas, beta, xivals)
        else:
            beta = Index(n, "Dummy")
            alphas = [psi.link[frozenset((v, w))] for w in nb]
            t = _q_n_tensor(len(nb) + 1, sd, alphas, beta, xivals) * Tensor(np.array(coeffs), [beta])
        for i in snd:
            t = t * Tensor(np.ones(i.dim), [i])
        psi.T[v] = t
    psi.T[src] = psi.T[src] * c
    for v in s.verts:
        if v in dv:
            continue
        toward = s.path(v, src)[1]
        beta = psi.link[frozenset((v, toward))]
        alphas = [psi.link[frozenset((v, w))] for w in s.neighbors(v) if w != toward]
        psi.T[v] = _transfer_tensor(s.site[v], beta, alphas)
    return psi


def delta_p(s: SiteMap, xs, dims=None) -> Net:
    """src/elementary_functions.jl:224-241."""
    dims = dims or list(range(1, len(xs) + 1))
    iv = calculate_ind_values(s, xs, dims)
    net = Net(s, {}, _new_links(s, 1))
    for v in s.verts:
        t = Tensor(np.ones(()), [])
        for i in s.site[v]:
            t = t * (onehot(i, iv[i]) if i in iv else Tensor(np.ones(i.dim), [i]))
        net.T[v] = t * delta(_vertex_links(net, v))
    return net


# ------------------------------------------------------------ contraction ----
def evaluate(f: Net, xs, dims=None):
    """evaluate = project + full contraction (src/itensornetworkfunction.jl:84-112)."""
    dims = dims or list(range(1, len(xs) + 1))
    iv = calculate_ind_values(f.s, xs, dims)
    ts = []
    for v in f.s.verts:
        t = f.T[v]
        for i in f.s.site[v]:
            t = t * onehot(i, iv[i])
        ts.append(t)
    return contract(ts).scalar()


def evaluate_batch(f: Net, X, dims=None) -> np.ndarray:
    """evaluate (src/itensornetworkfunction.jl:96-106) at every row of X.

    The same project + contraction as :func:`evaluate`, organised for many
    points: on a tree the contraction is the leaf-to-root message pass that
    scalar(tn; alg="bp") reduces to on trees, with the points that share a
    vertex's digit values contracted against one slice of its tensor.  Digits
    come from the greedy map (:func:`calculate_ind_values`).  Graphs with a
    cycle fall back to :func:`evaluate` point by point."""
    X = np.asarray(X, dtype=complex if f.s.is_complex else float)
    if X.ndim == 1:
        X = X.reshape(-1, 1)
    P = len(X)
    dims = dims or list(range(1, X.shape[1] + 1))
    verts, edges = f.s.verts, f.s.edges
    seen, comps = set(), []
    for r in verts:
        if r in seen:
            continue
        order, parent = [r], {r: None}
        seen.add(r)
        for v in order:
            for w in f.s.neighbors(v):
                if w not in seen:
                    seen.add(w)
                    parent[w] = v
                    order.append(w)
        comps.append((order, parent))
    if len(edges) != len(verts) - len(comps):
        return np.array([evaluate(f, list(x), dims) for x in X])
    digit = {}  # site Index -> digit value of every point
    for p_, x in enumerate(X):
        for ind, val in calculate_ind_values(f.s, list(x), dims).items():
            digit.setdefault(ind, np.zeros(P, dtype=np.int64))[p_] = val
    link = {}
    for v in verts:
        for w in f.s.neighbors(v):
            common = [i for i in f.T[v].inds if i in f.T[w].inds]
            link[(v, w)] = common[0]
    result = np.ones(P, dtype=complex if f.s.is_complex else float)
    for order, parent in comps:
        msg = {}
        for v in reversed(order):
            t = f.T[v]
            sites = [i for i in t.inds if i in digit]
            children = [w for w in f.s.neighbors(v) if parent.get(w) == v]
            keys = np.stack([digit[i] for i in sites], axis=1) if sites else np.zeros((P, 0), int)
            out_ind = link[(v, parent[v])] if parent[v] is not None else None
            out = np.zeros((P, out_ind.dim) if out_ind else (P,), dtype=np.result_type(t.arr, result))
            for key in np.unique(keys, axis=0):
                idx = np.nonzero(np.all(keys == key, axis=1))[0]
                sl = t.permute(sites + [i for i in t.inds if i not in sites]).arr[tuple(key)]
                axes = [i for i in t.inds if i not in sites]
                if not children:  # a leaf: the slice itself, for every point of the group
                    arr = np.broadcast_to(sl, (len(idx),) + sl.shape)
                else:
                    # the first child through one matrix product with the slice,
                    # the others as products batched over the points
                    c0 = link[(v, children[0])]
                    arr = np.tensordot(msg[children[0]][idx], sl, axes=([1], [axes.index(c0)]))
                    axes = [i for i in axes if i is not c0]
                    for c in children[1:]:
                        ax = axes.index(link[(v, c)])
                        a2 = np.moveaxis(arr, ax + 1, -1)
                        shp = a2.shape
                        a2 = np.matmul(a2.reshape(len(idx), -1, shp[-1]), msg[c][idx][:, :, None])
                        arr = a2.reshape(shp[:-1])
                        axes = [i for i in axes if i is not link[(v, c)]]
                out[idx] = arr.reshape(out[idx].shape)
            msg[v] = out
            for c in children:
                del msg[c]
        result = result * msg[order[0]]
    return result


def integrate(f: Net, take_sum=False):
    """src/integration.jl:6-17."""
    c = 1.0 if take_sum else 1.0 / f.s.base
    ts = []
    for v in f.s.verts:
        t = f.T[v]
        for i in f.s.site[v]:
            t = t * Tensor(np.full(i.dim, c), [i])
        ts.append(t)
    return contract(ts).scalar()


def dense(f: Net, order) -> np.ndarray:
    """The full tensor of f over the site indices `order` (small networks)."""
    return contract(list(f.T.values())).permute(list(order)).arr


def dense_grid_1d(f: Net, dim=1) -> tuple[np.ndarray, list]:
    """f on every grid point of a one-variable network, index order digit 1..L."""
    inds = sorted((i for i, (d, k, r) in f.s.info.items() if d == dim and r),
                  key=lambda i: f.s.info[i][1])
    return dense(f, inds).reshape(-1), inds


# -------------------------------------------------------------- operators ----
# Digit operators as [out, in] (src/digit_inds.jl:35-58 writes ITensor(o, s, s')).
OPS = {
    "D+": np.array([[0.0, 1.0], [0.0, 0.0]]),
    "D-": np.array([[0.0, 0.0], [1.0, 0.0]]),
    "Ddn": np.array([[1.0, 0.0], [0.0, 0.0]]),
    "Dup": np.array([[0.0, 0.0], [0.0, 1.0]]),
}


def _boundary_terms(L, boundary, dim, isfwd, n):
    """src/elementary_operators.jl:32-57."""
    if boundary == "Neumann":
        return [(1.0, {(dim, j): ("Dup" if isfwd else "Ddn") for j in range(1, L - n + 1)})]
    if boundary == "Periodic":
        return [(1.0, {(dim, j): ("D-" if isfwd else "D+") for j in range(1, L - n + 1)})]
    return []


def forward_shift_terms(L, dim=1, boundary="Dirichlet", n=0):
    """src/elementary_operators.jl:59-80: D+ at digit L-n, then carry strings."""
    terms = [(1.0, {(dim, L - n): "D+"})]
    string = [((dim, L - n), "D+")]
    for i in range(L - n, 1, -1):
        string.pop()
        string.append(((dim, i), "D-"))
        string.append(((dim, i - 1), "D+"))
        terms.append((1.0, dict(string)))
    return terms + _boundary_terms(L, boundary, dim, True, n)


def backward_shift_terms(L, dim=1, boundary="Dirichlet", n=0):
    """src/elementary_operators.jl:82-103."""
    terms = [(1.0, {(dim, L - n): "D-"})]
    string = [((dim, L - n), "D-")]
    for i in range(L - n, 1, -1):
        string.pop()
        string.append(((dim, i), "D+"))
        string.append(((dim, i - 1), "D-"))
        terms.append((1.0, dict(string)))
    return terms + _boundary_terms(L, boundary, dim, False, n)


def stencil_terms(L, shifts, delta_power, dim=1, left="Dirichlet", right="Dirichlet", scale=True,
                  base=2, nverts=None):
    """src/elementary_operators.jl:122-160 as a list of (coef, ops) terms."""
    terms = [(shifts[2], {})]
    for i, n in ((0, 1), (1, 0)):
        if shifts[i] != 0:
            terms += [(shifts[i] * c, o) for c, o in forward_shift_terms(L, dim, right, n)]
    for i, n in ((3, 0), (4, 1)):
        if shifts[i] != 0:
            terms += [(shifts[i] * c, o) for c, o in backward_shift_terms(L, dim, left, n)]
    if scale:
        f = float(base) ** (delta_power * (nverts if nverts is not None else L))
        terms = [(c * f, o) for c, o in terms]
    return terms


def apply_terms_dense(terms, F: np.ndarray, axis_of: dict) -> np.ndarray:
    """sum_t coef_t (prod of digit ops) F on a dense tensor; axis_of maps
    (dim, digit) -> axis of F."""
    out = np.zeros_like(F, dtype=np.result_type(F, float))
    for coef, ops in terms:
        G = F
        for key, name in ops.items():
            ax = axis_of[key]
            G = np.moveaxis(np.tensordot(OPS[name], G, axes=([1], [ax])), 0, ax)
        out = out + coef * G
    return out


def bond_spectrum(F: np.ndarray, left_axes) -> np.ndarray:
    """Singular values of F across the bipartition (left_axes | rest)."""
    left = list(left_axes)
    rest = [a for a in range(F.ndim) if a not in left]
    M = np.transpose(F, left + rest).reshape(int(np.prod([F.shape[a] for a in left])), -1)
    return np.linalg.svd(M, compute_uv=False)


def gradient(f: Net, X, dims, dout) -> dict:
    """sum_p dout_p d f(x_p) / d T_v for every vertex: f is linear in each
    T_v, so the derivative at a point is the environment of v (every other
    tensor sliced at the point's digits and contracted), placed at the slice
    of v's own site value.  Arrays use the order site inds + links of f.T[v]."""
    out = {v: np.zeros(f.T[v].arr.shape, dtype=np.result_type(f.T[v].arr, float)) for v in f.s.verts}
    for x, w in zip(X, dout):
        iv = calculate_ind_values(f.s, list(x), dims)
        sliced = {}
        for v in f.s.verts:
            t = f.T[v]
            for i in f.s.site[v]:
                t = t * onehot(i, iv[i])
            sliced[v] = t
        for v in f.s.verts:
            env = contract([sliced[u] for u in f.s.verts if u != v])
            links = [i for i in f.T[v].inds if i not in f.s.site[v]]
            env = env.permute(links) if links else env
            idx = tuple(iv[i] for i in f.s.site[v])
            out[v][idx] += w * env.arr
    return out


def aca_full(M: np.ndarray, tol: float, maxrank: int):
    """Cross of a sampled block by adaptive cross approximation with full
    pivoting (the factorisation step of the two-site TCI that ITensorTCI runs
    for the reference's TCI extension, ext/ITensorNumericalAnalysisTCIExt/
    tci_util.jl:21-55; ITensorTCI is not part of the reference, so this
    restates the published algorithm): the entry of largest magnitude of the
    residual (first in row-major order among equal ones) becomes a pivot
    unless it is at most tol * max|M|, and the residual loses its rank-one
    cross R[:, j] R[i, :] / R[i, j].  Returns pivot rows, pivot columns, the
    largest residual entry left and max|M|."""
    R = np.array(M, dtype=np.result_type(M, float), copy=True)
    scale = np.max(np.abs(M)) if M.size else 0.0
    rows, cols = [], []
    err = scale
    while len(rows) < min(maxrank, *M.shape):
        k = int(np.argmax(np.abs(R)))
        i, j = divmod(k, R.shape[1])
        piv = R[i, j]
        err = abs(piv)
        if scale == 0.0 or err <= tol * scale:
            break
        rows.append(i)
        cols.append(j)
        R = R - np.outer(R[:, j], R[i, :]) / piv
    if len(rows) == min(maxrank, *M.shape):
        err = float(np.max(np.abs(R))) if R.size else 0.0
    return rows, cols, float(err), float(scale)

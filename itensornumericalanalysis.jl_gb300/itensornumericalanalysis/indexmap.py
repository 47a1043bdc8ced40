"""Digit site legs and their map to continuous coordinates.

Mirrors src/digit_inds.jl (digit legs on graph vertices),
src/IndexMaps/{abstract,real,complex}indexmap.jl (digit k of variable d has
weight value * base^-k, digit 1 most significant) and src/indsnetworkmap.jl
(IndsNetworkMap = graph + legs + map).  Legs are plain records here; the
device never sees names, only the layout built in :class:`TreeLayout`.
"""
from __future__ import annotations

from dataclasses import dataclass
from functools import cached_property
from typing import Hashable

import numpy as np

from .graphs import NamedGraph

REAL, IMAG = "real", "imag"


@dataclass(frozen=True)
class SiteLeg:
    """One digit index: variable `dim` (1-based), digit (1 = most significant)."""

    vertex: Hashable
    dim: int
    digit: int
    base: int = 2
    kind: str = REAL  # REAL or IMAG (complex index maps)

    def value_to_scalar(self, value: int):
        """index_value_to_scalar (src/IndexMaps/realindexmap.jl:13-15,
        src/IndexMaps/complexindexmap.jl:25-32)."""
        w = value * float(self.base) ** (-self.digit)
        return 1j * w if self.kind == IMAG else w

    def values_to_scalars(self) -> list:
        return [self.value_to_scalar(i) for i in range(self.base)]


def default_dimension_vertices(g: NamedGraph, map_dimension: int = 1) -> list[list]:
    """Round-robin assignment of the graph's vertices to dimensions
    (src/digit_inds.jl:17-21)."""
    vs = g.vertices()
    return [vs[i::map_dimension] for i in range(map_dimension)]


class TreeLayout:
    """Device order of a forest: roots are the first vertex (graph order) of
    each component; vertices are numbered breadth first so that
    parent[v] < v and the children of a vertex have increasing numbers."""

    def __init__(self, g: NamedGraph):
        if not g.is_forest():
            raise ValueError(
                "tensor network functions on this engine live on trees (or forests); "
                "the graph has a cycle"
            )
        self.order: list = []
        self.parent: list[int] = []
        pos: dict = {}
        for comp in g.components():
            root = comp[0]
            pos[root] = len(self.order)
            self.order.append(root)
            self.parent.append(-1)
            head = pos[root]
            while head < len(self.order):
                v = self.order[head]
                for w in g.neighbors(v):
                    if w not in pos:
                        pos[w] = len(self.order)
                        self.order.append(w)
                        self.parent.append(head)
                head += 1
        self.pos = pos
        self.children: list[list[int]] = [[] for _ in self.order]
        for i, p in enumerate(self.parent):
            if p >= 0:
                self.children[p].append(i)

    @property
    def n(self) -> int:
        return len(self.order)

    def neighbours_in_layout_order(self, i: int) -> list[int]:
        """[parent (if any), children...] of layout vertex i."""
        return ([self.parent[i]] if self.parent[i] >= 0 else []) + self.children[i]


def _quotient_is_forest(g: NamedGraph, groups: list[list]) -> tuple[bool, int]:
    """Whether the groups' quotient graph is a forest, and the most edges
    that cross between any two groups."""
    gid = {v: k for k, gr in enumerate(groups) for v in gr}
    cross: dict = {}
    for u, w in g.edges():
        a, b = gid[u], gid[w]
        if a != b:
            key = (min(a, b), max(a, b))
            cross[key] = cross.get(key, 0) + 1
    q = NamedGraph(range(len(groups)), cross.keys())
    return q.is_forest(), max(cross.values(), default=0)


def tree_groups(g: NamedGraph) -> list[list]:
    """Vertex groups of a graph whose quotient graph is a forest (each group in
    graph vertex order, groups ordered by their first vertex).  Candidates:
    for grid-like names (tuples of one length) the slices of constant
    coordinate k and the lines along coordinate k; always the breadth-first
    layers from the first vertex.  The forest candidate crossed by the fewest
    edges between two groups wins (then the one with the smallest groups)."""
    verts = g.vertices()
    pos = {v: i for i, v in enumerate(verts)}
    cands = []
    if verts and all(isinstance(v, tuple) for v in verts) and len({len(v) for v in verts}) == 1:
        for k in range(len(verts[0])):
            for key in (lambda v, k=k: v[k], lambda v, k=k: v[:k] + v[k + 1:]):
                grp: dict = {}
                for v in verts:
                    grp.setdefault(key(v), []).append(v)
                cands.append(list(grp.values()))
    layers, seen = [], set()
    for r in verts:  # breadth-first layers per component
        if r in seen:
            continue
        frontier = [r]
        seen.add(r)
        while frontier:
            layers.append(frontier)
            nxt = []
            for v in frontier:
                for w in g.neighbors(v):
                    if w not in seen:
                        seen.add(w)
                        nxt.append(w)
            frontier = nxt
    cands.append(layers)
    best = None
    for groups in cands:
        groups = [sorted(gr, key=pos.get) for gr in groups]
        groups.sort(key=lambda gr: pos[gr[0]])
        ok, cross = _quotient_is_forest(g, groups)
        if not ok:
            continue
        score = (cross, max(len(gr) for gr in groups))
        if best is None or score < best[0]:
            best = (score, groups)
    return best[1]


class IndsNetworkMap:
    """A graph whose vertices carry digit legs, plus the digit -> coordinate map."""

    def __init__(self, graph: NamedGraph, legs: dict, is_complex: bool = False):
        self.graph = graph
        self.legs = {v: list(legs.get(v, [])) for v in graph.vertices()}
        self.is_complex = is_complex

    # -- structure ----------------------------------------------------------
    @cached_property
    def layout(self) -> TreeLayout:
        return TreeLayout(self.graph)

    @cached_property
    def tree_image(self) -> "IndsNetworkMap":
        """The map itself on a forest.  On a graph with cycles (e.g.
        named_grid((3, 3)), which the reference evaluates with
        scalar(alg="bp"/"exact")) the map of a tree of vertex groups: grid
        rows or columns (the grouping whose tree is crossed by the fewest
        edges), else breadth-first layers.  A group carries its members' legs
        in member order; a bond between two groups stands for all the edges
        between them.  Functions on this map are represented exactly on the
        image (merge_to_tree_image for given tensors); the constructors build
        directly on it, where sums keep the bonds of a tree."""
        if self.graph.is_forest():
            return self
        groups = tree_groups(self.graph)
        names = [tuple(gr) for gr in groups]
        gid = {v: n for n, gr in zip(names, groups) for v in gr}
        q = NamedGraph(names)
        for u, w in self.graph.edges():
            if gid[u] != gid[w]:
                q.add_edge(gid[u], gid[w])
        legs = {n: [l for v in gr for l in self.legs[v]] for n, gr in zip(names, groups)}
        img = IndsNetworkMap(q, legs, self.is_complex)
        img.merged_from = self
        img.groups = dict(zip(names, groups))
        return img

    def vertices(self) -> list:
        return self.graph.vertices()

    def nv(self) -> int:
        return self.graph.nv()

    def inds(self, v=None) -> list[SiteLeg]:
        if v is None:
            return [l for w in self.vertices() for l in self.legs[w]]
        return list(self.legs[v])

    def __getitem__(self, v) -> list[SiteLeg]:
        return self.inds(v)

    def base(self) -> int:
        bases = {l.base for l in self.inds()}
        if len(bases) != 1:
            raise ValueError("site legs have different bases")
        return bases.pop()

    def is_tree(self) -> bool:
        return self.graph.is_tree()

    # -- dimensions ---------------------------------------------------------
    def dimensions(self) -> list[int]:
        seen = []
        for l in self.inds():
            if l.dim not in seen:
                seen.append(l.dim)
        return seen

    def dimension(self, leg: SiteLeg | None = None) -> int:
        if leg is not None:
            return leg.dim
        return max(self.dimensions())

    def dimension_inds(self, dims) -> list[SiteLeg]:
        dims = [dims] if isinstance(dims, int) else list(dims)
        return [l for l in self.inds() if l.dim in dims]

    def dimension_vertices(self, dims) -> list:
        dims = [dims] if isinstance(dims, int) else list(dims)
        return [v for v in self.vertices() if any(l.dim in dims for l in self.legs[v])]

    def vertex(self, dim: int, digit: int, kind: str = REAL):
        hits = [
            v for v in self.vertices()
            for l in self.legs[v] if l.dim == dim and l.digit == digit and l.kind == kind
        ]
        if len(hits) != 1:
            raise KeyError(f"no unique vertex for dim={dim} digit={digit}")
        return hits[0]

    def vertex_dimension(self, v) -> int:
        (leg,) = self.legs[v]
        return leg.dim

    def vertex_digit(self, v) -> int:
        (leg,) = self.legs[v]
        return leg.digit

    def vertices_dimensions(self, verts) -> list[int]:
        return [l.dim for v in verts for l in self.legs[v]]

    def vertices_digits(self, verts) -> list[int]:
        return [l.digit for v in verts for l in self.legs[v]]

    def ndigits(self, dim: int, kind: str = REAL) -> int:
        return sum(1 for l in self.inds() if l.dim == dim and l.kind == kind)

    # -- digit map ----------------------------------------------------------
    def calculate_ind_values(self, xs, dims=None) -> dict:
        """Digits of the point xs (src/IndexMaps/realindexmap.jl:67-76 with the
        greedy subtraction of src/IndexMaps/abstractindexmap.jl:121-138)."""
        xs = [xs] if np.isscalar(xs) else list(xs)
        if dims is None:
            dims = list(range(1, len(xs) + 1))
        dims = [dims] if isinstance(dims, int) else list(dims)
        if len(xs) != len(dims):
            raise ValueError("xs and dims differ in length")
        out = {}
        parts = [(REAL, lambda z: float(np.real(z)))]
        if self.is_complex:
            parts.append((IMAG, lambda z: float(np.imag(z))))
        for d, x in zip(dims, xs):
            for kind, part in parts:
                legs = sorted(
                    (l for l in self.inds() if l.dim == d and l.kind == kind), key=lambda l: l.digit
                )
                rem = part(x)
                if not (rem >= 0.0 and np.isfinite(rem)):
                    raise ValueError(f"coordinate {x} outside the digit map's domain [0, inf)")
                for l in legs:
                    invb = 1.0 / float(l.base) ** l.digit
                    val = 0
                    for cand in range(l.base - 1, 0, -1):
                        t = cand * invb
                        if rem >= t:
                            val, rem = cand, rem - t
                            break
                    out[l] = val
        return out

    def calculate_p(self, ind_values: dict, dims=None) -> list:
        """Coordinates from digit values (src/IndexMaps/abstractindexmap.jl:103-119)."""
        dims = self.dimensions() if dims is None else ([dims] if isinstance(dims, int) else dims)
        return [sum(l.value_to_scalar(v) for l, v in ind_values.items() if l.dim == d) for d in dims]

    def grid_points(self, N: int, d: int) -> list:
        """N uniform grid points of dimension d (src/IndexMaps/realindexmap.jl:78-86);
        for a complex map the N x N points of the real and imaginary grids
        (src/IndexMaps/complexindexmap.jl:134-144)."""
        re = [l for l in self.inds() if l.dim == d and l.kind == REAL]
        base = float(re[0].base)
        L = len(re)
        a = round(base**L / N)
        if not self.is_complex:
            pts = [i * (a / base**L) for i in range(N + 2)]
            return [x for x in pts if x < 1]
        Li = sum(1 for l in self.inds() if l.dim == d and l.kind == IMAG)
        ai = round(base**Li / N)
        pts = [i * (a / base**L) + 1j * j * (ai / base**Li) for i in range(N + 2) for j in range(N + 2)]
        return [z for z in pts if z.real < 1 and z.imag < 1]

    # -- derived maps -------------------------------------------------------
    def reduced(self, dims) -> "IndsNetworkMap":
        """reduced_indsnetworkmap (src/indsnetworkmap.jl:29-46)."""
        dims = [dims] if isinstance(dims, int) else list(dims)
        legs = {v: [l for l in self.legs[v] if l.dim in dims] for v in self.vertices()}
        keep = [v for v in self.vertices() if legs[v]]
        return IndsNetworkMap(self.graph.induced_subgraph(keep), legs, self.is_complex)

    def union(self, other: "IndsNetworkMap") -> "IndsNetworkMap":
        g = self.graph.copy()
        for v in other.vertices():
            g.add_vertex(v)
        for u, w in other.graph.edges():
            g.add_edge(u, w)
        legs = {v: list(ls) for v, ls in self.legs.items()}
        for v in other.vertices():
            mine = legs.setdefault(v, [])
            have = {(l.dim, l.digit, l.kind) for l in mine}
            mine.extend(l for l in other.legs[v] if (l.dim, l.digit, l.kind) not in have)
        return IndsNetworkMap(g, legs, self.is_complex or other.is_complex)

    def same_structure(self, other: "IndsNetworkMap") -> bool:
        return (
            self.graph.vertices() == other.graph.vertices()
            and set(self.graph.edges()) == set(other.graph.edges())
            and all(self.legs[v] == other.legs[v] for v in self.vertices())
        )

    # -- device topology ------------------------------------------------------
    def leg_arrays(self):
        """Per layout vertex: n_legs, and flattened leg dim/var/digit/kind."""
        lay = self.layout
        nlegs, ldim, lvar, ldig, lkind = [], [], [], [], []
        for v in lay.order:
            legs = self.legs[v]
            nlegs.append(len(legs))
            for l in legs:
                ldim.append(l.base)
                lvar.append(l.dim)
                ldig.append(l.digit)
                lkind.append(1 if l.kind == IMAG else 0)
        return nlegs, ldim, lvar, ldig, lkind

    def __repr__(self) -> str:
        return f"IndsNetworkMap(nv={self.nv()}, dims={self.dimensions()}, complex={self.is_complex})"


def merge_to_tree_image(s: IndsNetworkMap, tensors: dict) -> dict:
    """Exact tensors of a function on s.tree_image, from per-vertex tensors on
    the graph of s with axes [site legs..., bonds to the neighbours in graph
    neighbour order]: the tensors of each group contracted over the group's
    inner edges; the edges from one group to another (in graph edge order)
    fused into one bond.  The result is in the image's canonical layout
    [site legs..., parent bond, child bonds...]."""
    img = s.tree_image
    if img is s:
        raise ValueError("the map's graph is a forest: give canonical-layout tensors")
    g = s.graph
    edges = g.edges()
    eid = {}
    for k, (u, w) in enumerate(edges):
        eid[(u, w)] = eid[(w, u)] = k
    gid = {v: n for n, gr in img.groups.items() for v in gr}
    lay = img.layout
    out = {}
    for i, name in enumerate(lay.order):
        members = img.groups[name]
        ops, nsym = [], len(edges)
        site_syms = []
        for v in members:
            t = np.asarray(tensors[v])
            nl = len(s.legs[v])
            sub = list(range(nsym, nsym + nl))
            nsym += nl
            site_syms += sub
            sub += [eid[(v, w)] for w in g.neighbors(v)]
            if t.ndim != len(sub):
                raise ValueError(f"tensor of vertex {v!r} has {t.ndim} axes, expected {len(sub)}")
            ops += [t, sub]
        out_syms, bond_dims = list(site_syms), []
        for j in lay.neighbours_in_layout_order(i):
            other = lay.order[j]
            es = sorted(k for k, (u, w) in enumerate(edges)
                        if {gid[u], gid[w]} == {name, other})
            out_syms += es
            bond_dims.append(es)
        # compact labels (einsum takes at most 52 distinct ones per call)
        relabel: dict = {}
        for k in range(1, len(ops), 2):
            ops[k] = [relabel.setdefault(x, len(relabel)) for x in ops[k]]
        out_lab = [relabel[x] for x in out_syms]
        arr = np.einsum(*ops, out_lab, optimize=True)
        site_shape = arr.shape[: len(site_syms)]
        shape, ax = list(site_shape), len(site_syms)
        for es in bond_dims:
            d = 1
            for _ in es:
                d *= arr.shape[ax]
                ax += 1
            shape.append(d)
        if lay.parent[i] < 0:  # a root's parent bond of dimension 1
            shape.insert(len(site_shape), 1)
        out[name] = arr.reshape(shape)
    return out


def digit_siteinds(g: NamedGraph, dimension_vertices=None, base: int = 2, map_dimension: int = 1):
    """Legs of a real map (src/digit_inds.jl:72-86)."""
    if not dimension_vertices or not dimension_vertices[0]:
        dimension_vertices = default_dimension_vertices(g, map_dimension)
    legs: dict = {v: [] for v in g.vertices()}
    for d, verts in enumerate(dimension_vertices, start=1):
        for k, v in enumerate(verts, start=1):
            legs[v].append(SiteLeg(v, d, k, base, REAL))
    return legs


def continuous_siteinds(
    g: NamedGraph, dimension_vertices=None, *, base: int = 2, map_dimension: int = 1
) -> IndsNetworkMap:
    """RealIndsNetworkMap (src/indsnetworkmap.jl:53-64, alias :83)."""
    return IndsNetworkMap(g, digit_siteinds(g, dimension_vertices, base, map_dimension), False)


real_continuous_siteinds = continuous_siteinds


def complex_continuous_siteinds(
    g: NamedGraph,
    real_dimension_vertices=None,
    imag_dimension_vertices=None,
    *,
    base: int = 2,
    map_dimension: int = 1,
) -> IndsNetworkMap:
    """ComplexIndsNetworkMap (src/indsnetworkmap.jl:66-81)."""
    legs = complex_digit_siteinds(g, real_dimension_vertices, imag_dimension_vertices, base, map_dimension)
    return IndsNetworkMap(g, legs, True)


def complex_digit_siteinds(g: NamedGraph, real_dimension_vertices=None, imag_dimension_vertices=None,
                           base: int = 2, map_dimension: int = 1):
    """Legs of a complex map: every vertex's real digit legs, then its
    imaginary ones (src/digit_inds.jl:88-115)."""
    if not real_dimension_vertices or not real_dimension_vertices[0]:
        real_dimension_vertices = default_dimension_vertices(g, map_dimension)
    if not imag_dimension_vertices or not imag_dimension_vertices[0]:
        imag_dimension_vertices = default_dimension_vertices(g, map_dimension)
    legs: dict = {v: [] for v in g.vertices()}
    for d, verts in enumerate(real_dimension_vertices, start=1):
        for k, v in enumerate(verts, start=1):
            legs[v].append(SiteLeg(v, d, k, base, REAL))
    for d, verts in enumerate(imag_dimension_vertices, start=1):
        for k, v in enumerate(verts, start=1):
            legs[v].append(SiteLeg(v, d, k, base, IMAG))
    return legs


RealIndsNetworkMap = continuous_siteinds
ComplexIndsNetworkMap = complex_continuous_siteinds


def reduced_indsnetworkmap(s: IndsNetworkMap, dims) -> IndsNetworkMap:
    return s.reduced(dims)


def grid_points(s: IndsNetworkMap, *args) -> list:
    """grid_points(s, N, d): N uniform points of variable d; grid_points(s, d):
    N = base^L with L the number of digit legs of d, i.e. every grid point of
    a real variable (src/IndexMaps/abstractindexmap.jl:149-155)."""
    s = _map(s)
    if len(args) == 1:
        (d,) = args
        legs = [l for l in s.inds() if l.dim == d]
        return s.grid_points(legs[0].base ** len(legs), d)
    N, d = args
    return s.grid_points(N, d)


# ---------------------------------------------------------------------------
# Free functions with the reference's exported names.  Each takes an
# IndsNetworkMap or anything holding one in `.s` (an ITensorNetworkFunction),
# as the reference forwards them from the function to its map
# (src/itensornetworkfunction.jl:60-76).
def _map(x) -> IndsNetworkMap:
    return x if isinstance(x, IndsNetworkMap) else x.s


def dimension(x, leg: SiteLeg | None = None) -> int:
    """Number of variables, or the variable of one leg (abstractindexmap.jl)."""
    return _map(x).dimension(leg)


def dimensions(x) -> list[int]:
    return _map(x).dimensions()


def dimension_inds(x, dims) -> list[SiteLeg]:
    """The legs of one or several variables (abstractindexmap.jl:83-89)."""
    return _map(x).dimension_inds(dims)


def dimension_vertices(x, dims) -> list:
    """Vertices carrying digits of the given variable(s) (indsnetworkmap.jl:139-145)."""
    return _map(x).dimension_vertices(dims)


def vertex_dimension(x, v) -> int:
    """The variable of the one leg of v (indsnetworkmap.jl:123-125)."""
    return _map(x).vertex_dimension(v)


def vertex_digit(x, v) -> int:
    """The digit of the one leg of v (indsnetworkmap.jl:135-137)."""
    return _map(x).vertex_digit(v)


def vertices_dimensions(x, verts) -> list[int]:
    return _map(x).vertices_dimensions(verts)


def vertices_digits(x, verts) -> list[int]:
    return _map(x).vertices_digits(verts)


def vertex_dimensions(x, v) -> list[int]:
    """The variables of every leg of v (indsnetworkmap.jl:127-129)."""
    return [l.dim for l in _map(x).legs[v]]


def vertex_digits(x, v) -> list[int]:
    """The digits of every leg of v (indsnetworkmap.jl:131-133)."""
    return [l.digit for l in _map(x).legs[v]]


def vertex(x, dim: int, digit: int):
    """The vertex holding the real leg of (dim, digit) (indsnetworkmap.jl:147-150)."""
    (v,) = [v for v, ls in _map(x).legs.items() for l in ls
            if l.dim == dim and l.digit == digit and l.kind == REAL]
    return v


def digit(x, leg: SiteLeg) -> int:
    """The digit of a leg (abstractindexmap.jl:76)."""
    return leg.digit


def base(x) -> int:
    """The base of the map's digits (indsnetworkmap.jl:113)."""
    legs = _map(x).inds()
    return legs[0].base if legs else 2


def index_value_to_scalar(x, leg: SiteLeg, value: int):
    """The contribution of one digit value to its coordinate (realindexmap.jl:13-15,
    complexindexmap.jl:25-32)."""
    return leg.value_to_scalar(value)


def indsnetworkmap(f) -> IndsNetworkMap:
    """The map of a function (itensornetworkfunction.jl:25)."""
    return _map(f)


def calculate_ind_values(x, xs, dims=None) -> dict:
    """Digits of a point: leg -> value (abstractindexmap.jl:121-160)."""
    return _map(x).calculate_ind_values(xs, dims)


def calculate_p(x, ind_values: dict, dims=None) -> list:
    """The point a digit assignment stands for (abstractindexmap.jl:103-119)."""
    return _map(x).calculate_p(ind_values, dims)


def indsnetwork(x):
    """The graph and its site legs (indsnetworkmap.jl:15): (graph, {v: [legs]})."""
    m = _map(x)
    return m.graph, {v: list(m.legs[v]) for v in m.vertices()}


class AbstractIndexMap(dict):
    """An index map: site leg -> (variable, digit) (src/IndexMaps/abstractindexmap.jl)."""


class RealIndexMap(AbstractIndexMap):
    """The index map of real variables (src/IndexMaps/realindexmap.jl:6-9)."""


class ComplexIndexMap(AbstractIndexMap):
    """The index map of complex variables, real and imaginary digit legs
    (src/IndexMaps/complexindexmap.jl)."""


def indexmap(x) -> AbstractIndexMap:
    """The index map (indsnetworkmap.jl:16): leg -> (variable, digit)."""
    m = _map(x)
    cls = ComplexIndexMap if m.is_complex else RealIndexMap
    return cls({l: (l.dim, l.digit) for v in m.vertices() for l in m.legs[v]})


def indexmaptype(x) -> type:
    """RealIndexMap or ComplexIndexMap (indsnetworkmap.jl:20)."""
    return ComplexIndexMap if _map(x).is_complex else RealIndexMap

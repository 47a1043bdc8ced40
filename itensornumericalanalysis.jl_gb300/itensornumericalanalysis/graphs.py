"""Named graphs: the vertex naming and ordering of NamedGraphs.jl generators.

Vertex order matters because the reference assigns digits to vertices in
graph order (src/digit_inds.jl:17-21).  The generators below reproduce the
NamedGraphs.jl orders: `named_grid` enumerates CartesianIndices (first
coordinate fastest); `named_comb_tree((nx, ny))` has the same vertices with
a backbone (j, 1) - (j+1, 1) and teeth (j, k) - (j, k+1).
"""
from __future__ import annotations

import itertools
from typing import Hashable, Iterable, Sequence

import numpy as np


class NamedGraph:
    """An undirected simple graph with hashable vertex names and a fixed vertex order."""

    def __init__(self, vertices: Iterable[Hashable] = (), edges: Iterable[tuple] = ()):
        self._vertices: list = []
        self._adj: dict = {}
        for v in vertices:
            self.add_vertex(v)
        for u, w in edges:
            self.add_edge(u, w)

    # -- construction --------------------------------------------------
    def add_vertex(self, v) -> None:
        if v not in self._adj:
            self._vertices.append(v)
            self._adj[v] = []

    def add_edge(self, u, w) -> None:
        if u == w:
            raise ValueError("self loops are not allowed")
        self.add_vertex(u)
        self.add_vertex(w)
        if w not in self._adj[u]:
            self._adj[u].append(w)
            self._adj[w].append(u)

    def rem_vertex(self, v) -> None:
        for w in self._adj.pop(v):
            self._adj[w].remove(v)
        self._vertices.remove(v)

    def copy(self) -> "NamedGraph":
        g = NamedGraph(self._vertices)
        for u, w in self.edges():
            g.add_edge(u, w)
        return g

    def induced_subgraph(self, verts: Iterable) -> "NamedGraph":
        keep = set(verts)
        g = NamedGraph([v for v in self._vertices if v in keep])
        for u, w in self.edges():
            if u in keep and w in keep:
                g.add_edge(u, w)
        return g

    def rename_vertices(self, f) -> "NamedGraph":
        g = NamedGraph([f(v) for v in self._vertices])
        for u, w in self.edges():
            g.add_edge(f(u), f(w))
        return g

    # -- queries ------------------------------------------------------
    def vertices(self) -> list:
        return list(self._vertices)

    def nv(self) -> int:
        return len(self._vertices)

    def ne(self) -> int:
        return sum(len(a) for a in self._adj.values()) // 2

    def neighbors(self, v) -> list:
        return list(self._adj[v])

    def has_vertex(self, v) -> bool:
        return v in self._adj

    def edges(self) -> list[tuple]:
        pos = {v: i for i, v in enumerate(self._vertices)}
        out = []
        for u in self._vertices:
            for w in self._adj[u]:
                if pos[u] < pos[w]:
                    out.append((u, w))
        return out

    def components(self) -> list[list]:
        seen, comps = set(), []
        for r in self._vertices:
            if r in seen:
                continue
            comp, stack = [], [r]
            seen.add(r)
            while stack:
                v = stack.pop()
                comp.append(v)
                for w in self._adj[v]:
                    if w not in seen:
                        seen.add(w)
                        stack.append(w)
            comps.append(comp)
        return comps

    def is_forest(self) -> bool:
        return self.ne() == self.nv() - len(self.components())

    def is_tree(self) -> bool:
        return self.is_forest() and len(self.components()) == 1

    def path(self, a, b) -> list:
        """Vertices on the tree path a -> b."""
        prev = {a: None}
        queue = [a]
        for v in queue:
            if v == b:
                break
            for w in self._adj[v]:
                if w not in prev:
                    prev[w] = v
                    queue.append(w)
        if b not in prev:
            raise ValueError("vertices are not connected")
        out = [b]
        while out[-1] != a:
            out.append(prev[out[-1]])
        return out[::-1]

    def __repr__(self) -> str:
        return f"NamedGraph(nv={self.nv()}, ne={self.ne()})"


def named_grid(dims: Sequence[int]) -> NamedGraph:
    """Grid graph; vertices are coordinate tuples in CartesianIndices order."""
    dims = tuple(int(d) for d in dims)
    ranges = [range(1, d + 1) for d in dims]
    verts = [tuple(reversed(t)) for t in itertools.product(*reversed(ranges))]
    g = NamedGraph(verts)
    for v in verts:
        for ax in range(len(dims)):
            if v[ax] < dims[ax]:
                w = list(v)
                w[ax] += 1
                g.add_edge(v, tuple(w))
    return g


def named_path_graph(L: int) -> NamedGraph:
    """Path of L vertices named (i, 1), i.e. named_grid((L, 1))."""
    return named_grid((L, 1))


def named_comb_tree(dims: Sequence[int]) -> NamedGraph:
    """Comb tree of NamedGraphs.jl: backbone along the first coordinate at
    second coordinate 1, one tooth per backbone vertex."""
    nx, ny = (int(d) for d in dims)
    verts = [(i, j) for j in range(1, ny + 1) for i in range(1, nx + 1)]
    g = NamedGraph(verts)
    for i in range(1, nx):
        g.add_edge((i, 1), (i + 1, 1))
    for i in range(1, nx + 1):
        for j in range(2, ny + 1):
            g.add_edge((i, j - 1), (i, j))
    return g


def named_binary_tree(n: int) -> NamedGraph:
    """Heap-ordered binary tree on vertices 1..n: children of i are 2i, 2i+1."""
    g = NamedGraph(range(1, n + 1))
    for i in range(1, n + 1):
        for c in (2 * i, 2 * i + 1):
            if c <= n:
                g.add_edge(i, c)
    return g


def uniform_tree(n: int, rng: np.random.Generator | int | None = None) -> NamedGraph:
    """Uniformly random labelled tree on vertices (1, 1) .. (n, 1) (Pruefer code).

    Same distribution as Graphs.uniform_tree, not the same random stream."""
    rng = np.random.default_rng(rng)
    g = NamedGraph([(i, 1) for i in range(1, n + 1)])
    if n <= 1:
        return g
    if n == 2:
        g.add_edge((1, 1), (2, 1))
        return g
    code = list(rng.integers(1, n + 1, size=n - 2))
    degree = [1] * (n + 1)
    for x in code:
        degree[x] += 1
    for x in code:
        leaf = next(i for i in range(1, n + 1) if degree[i] == 1)
        g.add_edge((leaf, 1), (int(x), 1))
        degree[leaf] -= 1
        degree[x] -= 1
    u, w = [i for i in range(1, n + 1) if degree[i] == 1]
    g.add_edge((u, 1), (w, 1))
    return g

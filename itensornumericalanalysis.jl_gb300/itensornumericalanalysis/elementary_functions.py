"""Closed-form constructors of tensor network functions.

Mirrors src/elementary_functions.jl and src/polynomialutils.jl.  Tensors are
written in the canonical device layout [site legs..., parent bond, child
bonds...] of `s.layout` and uploaded; sums of networks (cosh, sinh, tanh,
delta_p of several points) are formed on the device by the direct sum
(tnfa_add), exactly like the reference's `+`.

Element types: the reference builds cos/sin from complex exponentials and
makes every polynomial ComplexF64 (src/elementary_functions.jl:116-117,
131-132, 156).  For real k, a, c on a real map this module builds the same
functions with real tensors of the same bond dimension instead (cos/sin as a
bond-2 rotation network, polynomials with real Q_N tensors); complex
parameters or complex maps give complex networks built as the reference does.
"""
from __future__ import annotations

from math import comb
from typing import Sequence

import numpy as np

from . import _lib
from .indexmap import IndsNetworkMap
from .network import ITensorNetworkFunction

default_c_value = 1.0
default_a_value = 0.0
default_k_value = 1.0
default_nterms = 20
default_dim = 1


def _on_tree_image(fn):
    """Build on the map's tree image: on a graph with cycles the function is
    represented on a tree of vertex groups (IndsNetworkMap.tree_image)."""
    import functools

    @functools.wraps(fn)
    def wrapped(s, *args, **kw):
        return fn(s.tree_image, *args, **kw)

    return wrapped


def _is_real(*xs) -> bool:
    return all(np.isreal(x) for x in xs)


def _ones_sites(s: IndsNetworkMap, v):
    return np.ones(tuple(l.base for l in s.legs[v]))


def _site_factor(s: IndsNetworkMap, v, dim: int, fn, dtype=float):
    """Outer product over the legs of v: fn(leg) (a length-base vector) on the
    legs of `dim`, ones on the others."""
    t = np.ones((), dtype=dtype)
    for l in s.legs[v]:
        vec = np.asarray(fn(l), dtype=dtype) if l.dim == dim else np.ones(l.base, dtype=dtype)
        t = np.multiply.outer(t, vec)
    return t


def _bond_shape(s: IndsNetworkMap, i: int, chi: int):
    lay = s.layout
    return (chi if lay.parent[i] >= 0 else 1,) + (chi,) * len(lay.children[i])


def _product_network(s: IndsNetworkMap, site_tensors: dict) -> ITensorNetworkFunction:
    """Bond-1 network from per-vertex site tensors."""
    lay = s.layout
    ts = {}
    for i, v in enumerate(lay.order):
        st = np.asarray(site_tensors[v])
        ts[v] = st.reshape(st.shape + _bond_shape(s, i, 1))
    return ITensorNetworkFunction.from_tensors(s, ts)


@_on_tree_image
def const_itensornetwork(s: IndsNetworkMap, c=default_c_value, linkdim: int = 1):
    """f = c with every bond of dimension `linkdim` (src/elementary_functions.jl:16-26):
    each tensor is c' * delta(bonds) (x) ones(sites), c'^nv * linkdim = c."""
    lay = s.layout
    V, L = lay.n, int(linkdim)
    if _is_real(c):
        c = float(np.real(c))
        cp = (abs(c) / L) ** (1.0 / V)
        dtype = float
    else:
        cp = (complex(c) / L) ** (1.0 / V)
        dtype = complex
    ts = {}
    for i, v in enumerate(lay.order):
        bshape = _bond_shape(s, i, L)
        core = np.zeros(bshape, dtype=dtype)
        nb = len(lay.children[i]) + (1 if lay.parent[i] >= 0 else 0)
        if nb == 0:
            core[...] = cp
        else:
            for x in range(L):
                idx = (x if lay.parent[i] >= 0 else 0,) + (x,) * len(lay.children[i])
                core[idx] = cp
        ts[v] = np.multiply.outer(_ones_sites(s, v).astype(dtype), core)
    if dtype is float and c < 0:
        r = lay.order[0]
        ts[r] = -ts[r]
    return ITensorNetworkFunction.from_tensors(s, ts)


@_on_tree_image
def exp_itensornetwork(s: IndsNetworkMap, k=default_k_value, a=default_a_value,
                       c=default_c_value, dim: int = default_dim):
    """exp(k x_dim + a) * c as a bond-1 product network (src/elementary_functions.jl:30-53)."""
    dverts = s.dimension_vertices(dim)
    if not dverts:
        raise ValueError(f"dimension {dim} has no vertices")
    Lx = len(dverts)
    real = _is_real(k, a, c) and not s.is_complex
    dtype = float if real else complex
    cast = (lambda z: float(np.real(z))) if real else complex
    site = {}
    for v in s.vertices():
        if v in dverts:
            t = _site_factor(
                s, v, dim,
                lambda l: [np.exp(cast(k) * l.value_to_scalar(i)) for i in range(l.base)],
                dtype,
            )
            site[v] = t * np.exp(cast(a) / Lx)
        else:
            site[v] = _ones_sites(s, v).astype(dtype)
    site[dverts[0]] = site[dverts[0]] * cast(c)
    return _product_network(s, site)


@_on_tree_image
def cosh_itensornetwork(s, k=default_k_value, a=default_a_value, c=default_c_value, dim=default_dim):
    """cosh(kx+a)*c, bond 2 (src/elementary_functions.jl:57-68)."""
    return exp_itensornetwork(s, k, a, 0.5 * c, dim) + exp_itensornetwork(s, -k, -a, 0.5 * c, dim)


@_on_tree_image
def sinh_itensornetwork(s, k=default_k_value, a=default_a_value, c=default_c_value, dim=default_dim):
    """sinh(kx+a)*c, bond 2 (src/elementary_functions.jl:72-83)."""
    return exp_itensornetwork(s, k, a, 0.5 * c, dim) + exp_itensornetwork(s, -k, -a, -0.5 * c, dim)


@_on_tree_image
def tanh_itensornetwork(s, k=default_k_value, a=default_a_value, c=default_c_value,
                        nterms: int = default_nterms, dim=default_dim):
    """tanh(kx+a)*c ~ 1 + 2 sum_n (-1)^n exp(-2n(kx+a)), bond 1+nterms
    (src/elementary_functions.jl:87-105)."""
    first = s.dimension_vertices(dim)[0]
    psi = const_itensornetwork(s)
    for n in range(1, nterms + 1):
        t = exp_itensornetwork(s, -2 * k * n, -2 * n * a, 1.0, dim)
        t.scale_vertex(first, 2.0 * (-1) ** n)
        psi = psi + t
    if _is_real(c) and not psi.is_complex:
        psi.scale_vertex(first, float(np.real(c)))
    else:
        if not psi.is_complex:
            psi = psi.astype(_lib.C128)
        psi.scale_vertex(first, complex(c))
    return psi


def _rotation_network(s: IndsNetworkMap, k: float, a: float, c: float, dim: int, part: str):
    """c * Re/Im(exp(i(k x_dim + a))) as a real bond-2 tree network: every
    message is the (Re, Im) pair of exp(i * phase of its subtree)."""
    lay = s.layout
    if len(lay.children) and lay.parent.count(-1) != 1:
        raise ValueError("rotation form needs a tree")
    ts = {}
    for i, v in enumerate(lay.order):
        legs = s.legs[v]
        shape = tuple(l.base for l in legs)
        theta = np.zeros(shape)
        for idx in np.ndindex(*shape) if shape else [()]:
            theta[idx] = k * sum(
                float(np.real(l.value_to_scalar(x))) for l, x in zip(legs, idx) if l.dim == dim
            )
        nch = len(lay.children[i])
        is_root = lay.parent[i] < 0
        out = np.zeros(shape + ((1,) if is_root else (2,)) + (2,) * nch)
        for bidx in np.ndindex(*((2,) * nch)) if nch else [()]:
            ph = 1j ** sum(bidx)
            for sidx in np.ndindex(*shape) if shape else [()]:
                z = np.exp(1j * (theta[sidx] + (a if is_root else 0.0))) * ph
                if is_root:
                    out[sidx + (0,) + bidx] = c * (z.real if part == "re" else z.imag)
                else:
                    out[sidx + (0,) + bidx] = z.real
                    out[sidx + (1,) + bidx] = z.imag
        ts[v] = out
    return ITensorNetworkFunction.from_tensors(s, ts)


@_on_tree_image
def cos_itensornetwork(s, k=default_k_value, a=default_a_value, c=default_c_value, dim=default_dim):
    """cos(kx+a)*c, bond 2 (src/elementary_functions.jl:109-120)."""
    if _is_real(k, a, c) and not s.is_complex and s.is_tree():
        return _rotation_network(s, float(np.real(k)), float(np.real(a)), float(np.real(c)), dim, "re")
    return (exp_itensornetwork(s, 1j * k, 1j * a, 0.5 * c, dim)
            + exp_itensornetwork(s, -1j * k, -1j * a, 0.5 * c, dim))


@_on_tree_image
def sin_itensornetwork(s, k=default_k_value, a=default_a_value, c=default_c_value, dim=default_dim):
    """sin(kx+a)*c, bond 2 (src/elementary_functions.jl:124-135)."""
    if _is_real(k, a, c) and not s.is_complex and s.is_tree():
        return _rotation_network(s, float(np.real(k)), float(np.real(a)), float(np.real(c)), dim, "im")
    return (exp_itensornetwork(s, 1j * k, 1j * a, -0.5j * c, dim)
            + exp_itensornetwork(s, -1j * k, -1j * a, 0.5j * c, dim))


# ------------------------------------------------------------- polynomials --
def _f_alpha_beta(alpha: Sequence[int], beta: int) -> int:
    """Exponent of x_v in Q_N (src/polynomialutils.jl:4-6)."""
    return max(0, beta - sum(alpha)) if alpha else max(0, beta)


def _coeff(N: int, alpha: Sequence[int], beta: int) -> int:
    """Multinomial weight of Q_N (src/polynomialutils.jl:9-16)."""
    if N == 1:
        return 1
    out = 1
    for i in range(1, N):
        f = _f_alpha_beta(alpha[: N - 1 - i], beta)
        out *= comb(f, alpha[N - 1 - i]) if f >= 0 else 0
    return out


@_on_tree_image
def polynomial_itensornetwork(s: IndsNetworkMap, coeffs: Sequence, dim: int = default_dim,
                              k=default_k_value, c=default_c_value):
    """sum_i coeffs[i] (k x)^i * c as a bond-n tree network (Q_N tensors on the
    vertices of `dim`, transfer tensors elsewhere; src/elementary_functions.jl:139-207,
    src/polynomialutils.jl:19-79)."""
    coeffs = list(coeffs)
    n = len(coeffs)
    if n == 1:
        return const_itensornetwork(s, c=coeffs[0])
    coeffs = [cf * k**i for i, cf in enumerate(coeffs)]
    real = _is_real(*coeffs, c) and not s.is_complex
    dtype = float if real else complex
    lay = s.layout
    dverts = s.dimension_vertices(dim)
    source = dverts[0]
    g = s.graph
    ts = {}
    for i, v in enumerate(lay.order):
        nbrs = lay.neighbours_in_layout_order(i)  # [parent?, children...] as layout ids
        if v == source:
            beta_axis = None
        else:
            toward = g.path(v, source)[1]
            beta_axis = nbrs.index(lay.pos[toward])
        legs = s.legs[v]
        site_shape = tuple(l.base for l in legs)
        alpha_axes = [ax for ax in range(len(nbrs)) if ax != beta_axis]
        if v in dverts:
            # x_v per site configuration (sum over this vertex's digits of `dim`)
            xv = np.zeros(site_shape, dtype=dtype)
            for sidx in np.ndindex(*site_shape) if site_shape else [()]:
                xv[sidx] = sum(l.value_to_scalar(x) for l, x in zip(legs, sidx) if l.dim == dim)
            N = len(nbrs) + (1 if v == source else 0)
            out = np.zeros(site_shape + (n,) * len(nbrs), dtype=dtype)
            for bonds in np.ndindex(*((n,) * len(nbrs))) if nbrs else [()]:
                alpha = [bonds[ax] for ax in alpha_axes]
                betas = range(n) if v == source else [bonds[beta_axis]]
                acc = np.zeros(site_shape, dtype=dtype)
                for beta in betas:
                    w = _coeff(N, alpha, beta)
                    if w == 0:
                        continue
                    term = w * xv ** _f_alpha_beta(alpha, beta)
                    acc = acc + (coeffs[beta] * term if v == source else term)
                out[(Ellipsis,) + tuple(bonds)] = acc
            if v == source:
                out = out * c
        else:
            out = np.zeros(site_shape + (n,) * len(nbrs), dtype=dtype)
            for bonds in np.ndindex(*((n,) * len(nbrs))):
                beta = bonds[beta_axis]
                alpha = [bonds[ax] for ax in alpha_axes]
                if (sum(alpha) == beta) if alpha else (beta == 0):
                    out[(Ellipsis,) + tuple(bonds)] = 1.0
        if lay.parent[i] < 0:
            out = out.reshape(site_shape + (1,) + out.shape[len(site_shape):])
        ts[v] = out
    return ITensorNetworkFunction.from_tensors(s, ts)


@_on_tree_image
def random_itensornetwork(s: IndsNetworkMap, link_space: int = 1, rng=None, dtype=float,
                          normalize: bool = False):
    """Gaussian random tensors with bonds of dimension link_space
    (src/elementary_functions.jl:209-221).  normalize: unit Frobenius norm per tensor."""
    rng = np.random.default_rng(rng)
    lay = s.layout
    ts = {}
    for i, v in enumerate(lay.order):
        shape = tuple(l.base for l in s.legs[v]) + _bond_shape(s, i, link_space)
        t = rng.standard_normal(shape)
        if dtype is complex:
            t = t + 1j * rng.standard_normal(shape)
        if normalize:
            t = t / np.linalg.norm(t)
        ts[v] = t
    return ITensorNetworkFunction.from_tensors(s, ts)


@_on_tree_image
def delta_p(s: IndsNetworkMap, xs, dims=None):
    """Product state that is 1 on the digits of xs (a plane if some dims are
    left out); a list of points gives their sum (src/elementary_functions.jl:224-261)."""
    if len(xs) and isinstance(xs[0], (list, tuple, np.ndarray)):
        points = [list(p) for p in xs]
        pdims = dims if dims is not None else [list(range(1, len(p) + 1)) for p in points]
        if not points:
            raise ValueError("delta_p needs at least one point")
        psi = None
        for p, d in zip(points, pdims):
            t = delta_p(s, p, d)
            psi = t if psi is None else psi + t
        return psi
    xs = [xs] if np.isscalar(xs) else list(xs)
    dims = list(range(1, len(xs) + 1)) if dims is None else ([dims] if isinstance(dims, int) else list(dims))
    ivmap = s.calculate_ind_values(xs, dims)
    site = {}
    for v in s.vertices():
        t = np.ones(())
        for l in s.legs[v]:
            vec = np.zeros(l.base)
            if l in ivmap:
                vec[ivmap[l]] = 1.0
            else:
                vec[:] = 1.0
            t = np.multiply.outer(t, vec)
        site[v] = t
    return _product_network(s, site)


def _delta_overlaps(points, points_dims):
    """The intersections delta_kernel subtracts once (src/elementary_functions.jl
    :264-324): for every pair of (point, dims) sets that are not two distinct
    points on the same dims, the union of their coordinates, unless the two
    fix one dimension at different values (no intersection).  Returns
    (points, dims) lists."""
    over_p, over_d = [], []
    for i in range(len(points)):
        p1, d1 = list(points[i]), list(points_dims[i])
        for j in range(i + 1, len(points)):
            p2, d2 = list(points[j]), list(points_dims[j])
            if len(d1) == len(d2) and np.allclose(d1, d2) and not (
                len(p1) == len(p2) and np.allclose(p1, p2)
            ):
                continue
            ps_, ds_ = p1 + p2, d1 + d2
            order = sorted(range(len(ds_)), key=lambda q: ds_[q])
            ps, ds = [ps_[order[0]]], [ds_[order[0]]]
            for q in range(1, len(ds_)):
                if ds_[order[q]] != ds_[order[q - 1]]:
                    ps.append(ps_[order[q]])
                    ds.append(ds_[order[q]])
                    continue
                # same dimension twice: the reference compares ps_[q] and
                # ps_[q-1] (unsorted positions) here
                if np.isclose(ps_[q], ps_[q - 1]):
                    continue
                ps, ds = [], []
                break
            if not ds:
                continue
            over_p.append(ps)
            over_d.append(ds)
    return over_p, over_d


@_on_tree_image
def delta_kernel(s: IndsNetworkMap, points, points_dims=None, remove_overlap: bool = True,
                 coeff=-1.0, include_identity: bool = True):
    """const + coeff * sum of delta_p over points, minus the double-counted
    intersections (src/elementary_functions.jl:264-324)."""
    if points_dims is None:
        points_dims = [list(range(1, len(p) + 1)) for p in points]
    psi = coeff * delta_p(s, points, points_dims)
    if include_identity:
        psi = const_itensornetwork(s) + psi
    if remove_overlap and len(points) > 1:
        over_p, over_d = _delta_overlaps(points, points_dims)
        if over_p:
            psi = psi + (-coeff) * delta_p(s, over_p, over_d)
    return psi


const_itn = const_itensornetwork
exp_itn = exp_itensornetwork
cosh_itn = cosh_itensornetwork
sinh_itn = sinh_itensornetwork
tanh_itn = tanh_itensornetwork
cos_itn = cos_itensornetwork
sin_itn = sin_itensornetwork
poly_itn = polynomial_itensornetwork
rand_itn = random_itensornetwork

"""Synthetic workloads of the benchmark configurations (seeded)."""
from __future__ import annotations

import numpy as np

from .graphs import named_grid
from .indexmap import continuous_siteinds
from .network import ITensorNetworkFunction


def uneven_mps_batch(n: int = 512, seed: int = 3, lmin: int = 10, lmax: int = 30,
                     chimin: int = 8, chimax: int = 128):
    """n one-variable quantics MPS: L ~ U{lmin..lmax}; chi = round(exp(U[ln chimin,
    ln chimax])), capped per bond at min(chi, 2^k, 2^(L-k)); Gaussian tensors,
    each scaled to unit Frobenius norm.  Returns [(s, tensors dict)]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        L = int(rng.integers(lmin, lmax + 1))
        chi = int(round(np.exp(rng.uniform(np.log(chimin), np.log(chimax)))))
        s = continuous_siteinds(named_grid((L, 1)))
        lay = s.layout
        # bond k joins vertex k-1 and k (k = 1..L-1)
        bond = [1] + [min(chi, 2**k, 2 ** (L - k)) for k in range(1, L)]
        ts = {}
        for i, v in enumerate(lay.order):
            shape = (2, bond[i]) + ((bond[i + 1],) if i + 1 < L else ())
            t = rng.standard_normal(shape)
            ts[v] = t / np.linalg.norm(t)
        out.append((s, ts))
    return out


def upload_batch(batch, ctx=None):
    return [ITensorNetworkFunction.from_tensors(s, ts, ctx=ctx) for s, ts in batch]


def mps_apply_truncate_cost(s, ts, D: int = 3) -> float:
    """Flop estimate of applying a bond-D operator to the MPS (s, ts) and
    truncating it, per site at the actual shapes: the exact apply
    2·d²·D²·χl·χr, Householder QR of the (d·D·χl) x (D·χr) core
    (2mn² - 2n³/3 with m >= n) and a Jacobi SVD of its n x n factor (~12 n³)."""
    lay = s.layout
    total = 0.0
    for i, v in enumerate(lay.order):
        shape = np.shape(ts[v])
        d = shape[0]
        chil = shape[1] if len(shape) > 1 else 1
        chir = shape[2] if len(shape) > 2 else 1
        total += 2.0 * d * d * D * D * chil * chir
        m, n = d * D * chil, D * chir
        m, n = max(m, n), min(m, n)
        total += 2.0 * m * n * n - 2.0 * n ** 3 / 3.0 + 12.0 * n ** 3
    return total


def lpt_shards(costs, n: int) -> list:
    """Longest-processing-time-first split of items with the given costs over
    n workers (each item to the least loaded worker, largest items first; the
    heaviest load is within 4/3 of the best split).  Returns n lists of item
    indices, each in ascending order."""
    import heapq

    loads = [(0.0, r) for r in range(n)]
    heapq.heapify(loads)
    out = [[] for _ in range(n)]
    for i in sorted(range(len(costs)), key=lambda j: (-costs[j], j)):
        load, r = heapq.heappop(loads)
        out[r].append(i)
        heapq.heappush(loads, (load + costs[i], r))
    return [sorted(x) for x in out]

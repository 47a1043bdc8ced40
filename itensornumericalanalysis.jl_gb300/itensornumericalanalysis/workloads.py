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

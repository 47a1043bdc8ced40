"""tnfa_evaluate_noalloc: batched evaluation for callers that cannot allocate
device memory during the call (their GPU memory is owned by another runtime's
caching allocator, or they run latency-bound loops that must not block on the
allocator).  The entry point takes all scratch from a fixed device array in
the library; it must agree with tnfa_evaluate call after call, and reject a
request whose scratch does not fit.

This file is collected last so that a failure here stops a `-x` run only
after every other test has run."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from _helpers import upload_oracle

pytestmark = pytest.mark.gpu

TOL_F64 = 1e-12
TOL_F32 = 2e-5


def _device(a, dtype):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).cuda()


def _evaluate(ina, f, Xd, n, dims, out, kind, prec, noalloc):
    import torch

    torch.cuda.synchronize()
    lib = f.ctx.lib
    d = (C.c_int32 * len(dims))(*dims)
    if noalloc:
        st = lib.tnfa_evaluate_noalloc(f.ctx.handle, f.handle, Xd.data_ptr(), n, len(dims), d,
                                       out.data_ptr(), kind, prec)
    else:
        st = lib.tnfa_evaluate(f.ctx.handle, f.handle, Xd.data_ptr(), n, len(dims), d,
                               ina._lib.MEM_DEVICE, out.data_ptr(), kind, ina._lib.MEM_DEVICE,
                               prec)
    f.ctx.check(st)
    return out.cpu().numpy()


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_noalloc_matches_evaluate_twice(ina, dtype):
    import torch

    L = ina._lib
    graph = O.binary_tree_graph(31)
    rng = np.random.default_rng(40)
    s_or = O.siteinds(graph, map_dimension=3)
    net = O.random_net(s_or, 16, rng, normalize=True)
    f, _ = upload_oracle(ina, graph, net, dtype=L.F64 if dtype == "f64" else L.F32)
    prec = L.PREC_F64 if dtype == "f64" else L.PREC_F32
    for call in range(2):  # two calls in a row share (and must clear) the scratch
        X = rng.random((3000 + 517 * call, 3))
        Xd = _device(X, torch.float64)
        n = len(X)
        if dtype == "f64":
            a = _evaluate(ina, f, Xd, n, [1, 2, 3], torch.empty(n, dtype=torch.float64, device="cuda"),
                          L.OUT_F64, prec, True)
            b = _evaluate(ina, f, Xd, n, [1, 2, 3], torch.empty(n, dtype=torch.float64, device="cuda"),
                          L.OUT_F64, prec, False)
            assert np.max(np.abs(a - b)) <= TOL_F64 * np.max(np.abs(b))
        else:
            a = _evaluate(ina, f, Xd, n, [1, 2, 3], torch.empty(2 * n, dtype=torch.float32, device="cuda"),
                          L.OUT_F32_SCALED, prec, True)
            b = _evaluate(ina, f, Xd, n, [1, 2, 3], torch.empty(2 * n, dtype=torch.float32, device="cuda"),
                          L.OUT_F32_SCALED, prec, False)
            va = np.ldexp(a[:n].astype(np.float64), a[n:].view(np.int32))
            vb = np.ldexp(b[:n].astype(np.float64), b[n:].view(np.int32))
            assert np.max(np.abs(va - vb) / np.abs(vb)) <= TOL_F32


@pytest.mark.parametrize("case", ["fused_f64", "fused_f32", "complex"])
def test_noalloc_other_branches_twice(ina, case):
    """The small-bond branch (every bond <= 8: the whole tree per thread in
    one launch, only the digit program and its schedule in the array) in FP64
    and FP32, and a complex network (complex128 messages, (re, im) output),
    each against tnfa_evaluate on two calls in a row."""
    import torch

    L = ina._lib
    rng = np.random.default_rng(42)
    if case == "complex":
        graph = O.binary_tree_graph(15)
        s_or = O.siteinds(graph, map_dimension=3)
        net = O.random_net(s_or, 12, rng, normalize=True)
        f, _ = upload_oracle(ina, graph, net)
        f = f.astype(L.C128)
        f.scale_vertex(f.s.layout.order[0], 0.6 - 0.8j)
        nd, prec, kind = 3, L.PREC_F64, L.OUT_C128
    else:
        graph = O.path_graph(12)
        s_or = O.siteinds(graph)
        net = O.random_net(s_or, 6, rng, normalize=True)
        f, _ = upload_oracle(ina, graph, net, dtype=L.F64 if case == "fused_f64" else L.F32)
        nd = 1
        prec = L.PREC_F64 if case == "fused_f64" else L.PREC_F32
        kind = L.OUT_F64
    dims = list(range(1, nd + 1))
    for call in range(2):
        X = rng.random((2500 + 301 * call, nd))
        Xd = _device(X, torch.float64)
        n = len(X)
        odt = torch.complex128 if case == "complex" else torch.float64
        if case != "complex":
            f.ctx.kernel_stats(reset=True)
        a = _evaluate(ina, f, Xd, n, dims, torch.empty(n, dtype=odt, device="cuda"), kind, prec, True)
        if case != "complex":
            st = f.ctx.kernel_stats(reset=True)
            assert st.get("eval_fused", {}).get("launches", 0) >= 1, st
        b = _evaluate(ina, f, Xd, n, dims, torch.empty(n, dtype=odt, device="cuda"), kind, prec, False)
        tol = TOL_F32 if case == "fused_f32" else TOL_F64
        assert np.max(np.abs(a - b)) <= tol * np.max(np.abs(b))


def test_noalloc_rejects_oversize_requests(ina):
    import torch

    L = ina._lib
    graph = O.binary_tree_graph(15)
    rng = np.random.default_rng(41)
    s_or = O.siteinds(graph, map_dimension=3)
    net = O.random_net(s_or, 64, rng, normalize=True)
    f, _ = upload_oracle(ina, graph, net)
    n = 400_000  # ~3 message slots x 64 doubles per point: far above 32 MiB
    Xd = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    with pytest.raises(ina.TnfaError) as e:
        _evaluate(ina, f, Xd, n, [1, 2, 3], out, L.OUT_F64, L.PREC_F64, True)
    assert e.value.status == L.ERR_INVALID_ARGUMENT
    assert "points per call" in str(e.value)
    # a mismatched precision is refused rather than converted (that would allocate)
    with pytest.raises(ina.TnfaError):
        _evaluate(ina, f, Xd, 10, [1, 2, 3], out, L.OUT_F64, L.PREC_F32, True)

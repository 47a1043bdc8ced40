"""Benchmark of the hot path: batched point evaluation of a quantics tree
tensor network (60-vertex balanced binary tree, 3 variables x 20 bits,
chi = 128, Gaussian tensors of unit Frobenius norm, 10^7 points in [0,1)^3).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--points P]
                    [--precision mixed|mixed_fast|f32|f64] [--impl ours|reference]

Prints one JSON line.  `value` is points/s over all ranks with inputs already
in device memory; `e2e` is the same through the public C-ABI call with host
buffers (host->device and device->host copies inside the timed region).
The headline precision "mixed" is gated: every point of a 32768-point sample
must lie within 1e-8 (relative) of the plain FP64 path, else the line carries
"accuracy_gate": {"passed": false} and the process exits with status 3.
Under torchrun every rank evaluates its own share of points (weak scaling:
the per-GPU point count is fixed), no collective on the data path.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "itensornumericalanalysis.jl_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "MPO-apply+truncate/s & point evals/s, mixed vs FP64 plain, rel.err<=1e-8"
WORKLOAD = "batched_evaluate: binary tree 60 vertices, 3 vars x 20 bits, chi=128, fp32 tensors"
N_VERT, CHI, NDIM = 60, 128, 3
# DRAM traffic per point of one two-child chi-128 vertex launch, from ncu
# captures of this workload (dram__bytes_read.sum + dram__bytes_write.sum):
# k_contract_tc2 read 2.108 GB + wrote 1.000 GB for 2e6 points
TC2_DRAM_BYTES_PER_POINT = (2.108e9 + 1.000e9) / 2.0e6
# k_contract_oz read 61.8 MB + wrote 91.6 MB for 131072 points (capture of a
# two-child vertex of this workload at 131072 points)
OZ_DRAM_BYTES_PER_POINT = (61.8e6 + 91.6e6) / 131072
# tensor-core passes per algorithmic product
MMA_PASSES = {"contract_oz": 26, "contract_tc": 3}


# ------------------------------------------------------------- workload --
def config3_tensors(seed: int = 1):
    """Tensors of the 60-vertex heap-ordered binary tree in the device layout
    [site, parent, children...], Gaussian, unit Frobenius norm, float32."""
    import itensornumericalanalysis as ina

    g = ina.named_binary_tree(N_VERT)
    s = ina.continuous_siteinds(g, map_dimension=NDIM)
    lay = s.layout
    rng = np.random.default_rng(seed)
    ts = {}
    for i, v in enumerate(lay.order):
        shape = (2, CHI if lay.parent[i] >= 0 else 1) + (CHI,) * len(lay.children[i])
        t = rng.standard_normal(shape, dtype=np.float32)
        ts[v] = t / np.linalg.norm(t)
    return s, ts


def config3_points(n: int, seed: int = 1, offset: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    if offset:
        rng.random((offset, NDIM))  # advance to this rank's share
    return rng.random((n, NDIM))


def oracle_net(s, ts):
    """The same network in the oracle's labelled-tensor form."""
    import oracle as O

    so = O.siteinds(O.binary_tree_graph(N_VERT), map_dimension=NDIM)
    link = {frozenset(e): O.Index(CHI, "L") for e in so.edges}
    net = O.Net(so, {}, link)
    lay = s.layout
    for i, v in enumerate(lay.order):
        nb = lay.neighbours_in_layout_order(i)
        arr = ts[v].astype(np.float64)
        if lay.parent[i] < 0:
            arr = arr[:, 0]
        inds = so.site[v] + [link[frozenset((v, lay.order[j]))] for j in nb]
        net.T[v] = O.Tensor(arr, inds)
    return net


_WORKER_NET = {}


def _oracle_batch_worker(args):
    seed, pts = args
    import itensornumericalanalysis.indexmap  # noqa: F401  (host layout only)
    import oracle as O

    if seed not in _WORKER_NET:  # the network is built once per worker process
        s, ts = config3_tensors(seed)
        _WORKER_NET[seed] = oracle_net(s, ts)
        O.evaluate_batch(_WORKER_NET[seed], pts[:16], [1, 2, 3])  # warm the BLAS threads
    net = _WORKER_NET[seed]
    t0 = time.perf_counter()
    vals = O.evaluate_batch(net, pts, [1, 2, 3])
    return time.perf_counter() - t0, vals


_CPU_POOL = {}


def cpu_baseline(n_points: int, cores: int, seed: int = 1, offset: int = 0):
    """The oracle's batched FP64 evaluation (the reference's project +
    contraction, points sharing a digit contracted against one tensor slice
    through BLAS) on `cores` host threads, in a separate process whose BLAS
    is limited to that many threads (kept for later calls)."""
    import multiprocessing as mp

    pts = config3_points(n_points, seed, offset=offset)
    if cores not in _CPU_POOL:
        keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
        saved = {k: os.environ.get(k) for k in keys}
        for k in keys:
            os.environ[k] = str(cores)
        try:
            _CPU_POOL[cores] = mp.get_context("spawn").Pool(1)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
    busy, vals = _CPU_POOL[cores].apply(_oracle_batch_worker, ((seed, pts),))
    return n_points / busy, busy, pts, vals


# ----------------------------------------------------------------- clocks --
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, flag in zip(names, parts[4:8]):
                if flag.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- main --
def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "fallback": True}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if _cuda() else "gloo")
    return ws, rank, local


def _cuda() -> bool:
    import torch

    return torch.cuda.is_available()


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if _cuda() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, ws, rank):
    """The reference's CPU path as restated by the oracle (the reference
    itself is Julia, absent here and on the GPU hosts): its FP64 batched
    evaluation on all host threads, one bounded sample of the workload per
    step."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    n = args.cpu_points
    times = []
    for _ in range(args.warmup):
        cpu_baseline(max(16, n // 8), cores)
    for _ in range(args.steps):
        rate, busy, _, _ = cpu_baseline(n, cores)
        times.append(busy)
    rate = n / float(np.mean(times))
    sample = f"{n} points of the workload per step, oracle batched FP64 evaluation, {cores} BLAS threads"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "points/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * float(np.mean(times)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "points_per_step": n},
        "cpu_baseline": {"value": rate, "unit": "points/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": rate, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


def _timed(fn, reps=1):
    import torch

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        out = fn()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps, out


def integrate_rates(f32net, f64net, peaks) -> dict:
    """integrate() over [0,1)^3 of the benchmark network: the HBM-bound member
    of the path (one persistent k_integrate launch reads every tensor byte
    once), FP32 and FP64 copies.  Per call: CUDA events on the current stream
    around 5 calls (host set-up and the read-back included); per kernel: the
    library's own CUDA events around each k_integrate launch (on its
    stream)."""
    import torch

    out = {}
    for name, nt in (("f32", f32net), ("f64", f64net)):
        nt.integrate()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record()
        reps = 5
        for _ in range(reps):
            nt.integrate()
        ev1.record()
        torch.cuda.synchronize()
        ti = ev0.elapsed_time(ev1) / 1e3 / reps
        nbytes = nt.info()[2] * (4 if name == "f32" else 8)
        nt.ctx.kernel_stats(reset=True)
        nt.ctx.set_timing(True)
        for _ in range(reps):
            nt.integrate()
        nt.ctx.set_timing(False)
        st = nt.ctx.kernel_stats(reset=True).get("integrate", {})
        tk = st["ms"] / st["launches"] / 1e3 if st.get("launches") else float("nan")
        out[name] = {"ms": ti * 1e3, "tensor_bytes": nbytes, "GBps": nbytes / ti / 1e9,
                     "frac_of_hbm": nbytes / ti / 1e9 / peaks["hbm_gbs"],
                     "kernel_ms": tk * 1e3, "kernel_GBps": nbytes / tk / 1e9,
                     "kernel_frac_of_hbm": nbytes / tk / 1e9 / peaks["hbm_gbs"]}
    return out


def secondary_measurements(ctx, ws, rank, args, f32net=None, f64net=None, Xd=None,
                           ref64=None) -> dict:
    """The other configurations of the metric, one timed repetition each after
    a warm-up: batched MPO apply + truncate (512 uneven MPS, first derivative,
    cutoff 1e-10; FP64 plain and mixed), the 2-D Laplace solve (comb 2 x 16),
    the reference's CPU case end to end (L = 20), and the gradient of batched
    evaluation (comb 2 x 12, chi 32, FP32, 2^20 points)."""
    import itensornumericalanalysis as ina
    from itensornumericalanalysis.workloads import (lpt_shards, mps_apply_truncate_cost,
                                                    uneven_mps_batch, upload_batch)

    only = set(args.only.split(",")) if args.only else None

    def want(name):
        return only is None or name in only

    out = {}
    if want("mixed_fast"):
        # the split-BF16 tensor-core path (3 passes, FP32 messages) on the
        # headline workload: faster, about 1e-5 relative
        import torch

        if f32net is None:
            s3, ts3 = config3_tensors(1)
            f32net = ina.ITensorNetworkFunction.from_tensors(s3, ts3, ctx=ctx, dtype=ina._lib.F32)
            f64net = f32net.astype(ina._lib.F64)
        P = args.points
        if Xd is None:
            Xd = torch.from_numpy(config3_points(P, 1, offset=rank * P)).cuda()
        o = torch.empty(2 * P, dtype=torch.float32, device="cuda")
        d3 = (ctypes.c_int32 * 3)(1, 2, 3)

        def fast():
            ctx.call("tnfa_evaluate", f32net.handle, Xd.data_ptr(), P, 3, d3, ina._lib.MEM_DEVICE,
                     o.data_ptr(), ina._lib.OUT_F32_SCALED, ina._lib.MEM_DEVICE,
                     ina._lib.PREC_MIXED_FAST)

        fast()
        ctx.kernel_stats(reset=True)
        ctx.set_timing(True)
        tf, _ = _timed(fast, 1)
        ctx.set_timing(False)
        stf = ctx.kernel_stats(reset=True)
        tf = max_over_ranks(tf, ws)
        nf = min(args.f64_points, P)
        if ref64 is None:
            o64 = torch.empty(nf, dtype=torch.float64, device="cuda")
            ctx.call("tnfa_evaluate", f64net.handle, Xd.data_ptr(), nf, 3, d3, ina._lib.MEM_DEVICE,
                     o64.data_ptr(), ina._lib.OUT_F64, ina._lib.MEM_DEVICE, ina._lib.PREC_F64)
            ref64 = o64.cpu().numpy()
        oh = o.cpu().numpy()
        gf = np.ldexp(oh[:nf].astype(np.float64), oh[P:P + nf].view(np.int32))
        rf = np.abs(gf - ref64[:nf]) / np.abs(ref64[:nf])
        out["mixed_fast"] = {
            "value": ws * P / tf, "unit": "points/s", "points": P,
            "rel_err_vs_fp64": {"median": float(np.median(rf)), "max": float(np.max(rf)),
                                "normwise": float(np.linalg.norm(gf - ref64[:nf]) /
                                                  np.linalg.norm(ref64[:nf]))},
            "roofline": roofline(stf, max(stf, key=lambda k: stf[k]["ms"]) if stf else None,
                                 measured_peaks()),
            "what": "precision mixed_fast: tcgen05 split-BF16 (hi/lo, 3 passes), FP32 messages; "
                    "misses the 1e-8 gate, reported beside the headline"}
    if only is not None and "integrate" in only:
        s3, ts3 = config3_tensors(1)
        n32 = ina.ITensorNetworkFunction.from_tensors(s3, ts3, ctx=ctx, dtype=ina._lib.F32)
        out["integrate"] = integrate_rates(n32, n32.astype(ina._lib.F64), measured_peaks())
        del n32
    if want("apply_truncate"):
        # --- config 5: MPO apply + truncate of an uneven batch -------------------
        batch = uneven_mps_batch(n=args.mps, seed=3)
        if ws > 1:  # strong scaling: the batch split by LPT on flop estimates
            shards = lpt_shards([mps_apply_truncate_cost(s_, t_) for s_, t_ in batch], ws)
            batch = [batch[i] for i in shards[rank]]
        fs = upload_batch(batch, ctx=ctx)
        ops = {}
        for s, _ in batch:
            if s.nv() not in ops:
                ops[s.nv()] = ina.first_derivative_operator(s)
        oplist = [ops[s.nv()] for s, _ in batch]
        Xc5 = np.random.default_rng(0).random(256)
        c5 = {}
        for prec in ("f64", "mixed"):
            ina.operate_batched(oplist[:8], fs[:8], cutoff=1e-10, precision=prec)  # warm-up
            ctx.kernel_stats(reset=True)
            ctx.set_timing(True)
            t, res = _timed(lambda: ina.operate_batched(oplist, fs, cutoff=1e-10, precision=prec))
            ctx.set_timing(False)
            st = ctx.kernel_stats(reset=True)
            t = max_over_ranks(t, ws)
            c5[prec] = {
                "value": args.mps / t, "unit": "MPS/s", "s_per_batch": t,
                "max_bond_after": max(r.maxlinkdim() for r in res),
                "kernel_ms": {k: round(v["ms"], 2) for k, v in sorted(st.items(), key=lambda kv: -kv[1]["ms"])[:6]},
                "vals": [r.evaluate_batch(Xc5) for r in res[:64]],
            }
            del res
        va, vb = c5["f64"].pop("vals"), c5["mixed"].pop("vals")
        err = max(float(np.max(np.abs(a - b)) / max(np.max(np.abs(a)), 1e-300)) for a, b in zip(va, vb))
        # the plain FP64 path: one operate() per MPS (the reference's own call
        # pattern), FP64 throughout, on every 8th MPS of the batch (a uniform
        # sample of its lengths and bond dimensions)
        sub = list(range(0, len(fs), 8))
        ina.operate(oplist[0], fs[0], cutoff=1e-10, precision="f64")  # warm-up
        tp, resp = _timed(lambda: [ina.operate(oplist[i], fs[i], cutoff=1e-10, precision="f64") for i in sub])
        tp = max_over_ranks(tp, ws)
        vp = [r.evaluate_batch(Xc5) for r in resp[:8]]
        errp = max(float(np.max(np.abs(a - b)) / max(np.max(np.abs(a)), 1e-300))
                   for a, b in zip(vp, [vb[i] for i in sub[:8] if i < len(vb)]))
        plain = {"value": ws * len(sub) / tp, "unit": "MPS/s", "mps": len(sub), "s": tp,
                 "what": "one operate() per MPS (apply, then QR orthogonalisation and SVD sweep of "
                         "the exact product), FP64, every 8th MPS of the batch"}
        out["mpo_apply_truncate"] = {
            "value": c5["mixed"]["value"], "unit": "MPS/s", "batch": args.mps,
            "scaling": "strong (LPT split of the batch over the ranks)" if ws > 1 else None,
            "precision": "mixed (FP32-preconditioned Jacobi, double-float polish, FP64 rank-revealing QR)",
            "mixed": c5["mixed"], "fp64_batched": c5["f64"], "fp64_plain": plain,
            "mixed_over_fp64_plain": c5["mixed"]["value"] / plain["value"],
            "mixed_over_fp64_batched": c5["mixed"]["value"] / c5["f64"]["value"],
            "rel_err_mixed_vs_fp64": err,
            "rel_err_mixed_vs_fp64_plain": errp,
            "rel_err_what": "max over 64 MPS (8 for the plain path) of max|g_mixed - g_f64| / max|g_f64| "
                            "at 256 points",
        }
        if max(err, errp) > 1e-8:
            raise SystemExit(f"mixed apply+truncate misses the 1e-8 gate: {err:.3g} / {errp:.3g}")
        del fs
    if want("laplace"):
        # --- config 2: 2-D Laplace solve on a comb, 2 x 16 bits ---------------------
        L2 = 16
        s2 = ina.continuous_siteinds(ina.named_comb_tree((2, L2)),
                                     [[(1, j) for j in range(L2, 0, -1)], [(2, j) for j in range(1, L2 + 1)]])
        b2 = ina.sin_itn(s2, k=np.pi, dim=1) * ina.sin_itn(s2, k=np.pi, dim=2)
        A2 = ina.laplacian_operator(s2)

        def solve2():
            return ina.linsolve(A2, b2, nsweeps=2, maxdim=40, cutoff=1e-20, tol=1e-8, refinements=2)

        solve2()
        t2, x2 = _timed(solve2)
        X2 = np.random.default_rng(2).random((4096, 2))
        exact2 = -np.sin(np.pi * X2[:, 0]) * np.sin(np.pi * X2[:, 1]) / (2 * np.pi**2)
        got2 = x2.evaluate_batch(X2, [1, 2])
        # the FP64 floor of any stored solution: each value of x carries a
        # rounding of up to eps |x|, which the operator turns into a residual
        # of eps || |A| |x| || / ||b|| (|A| = the stencil with absolute
        # weights; x is one-signed here, so |A| |x| = |A| x up to sign)
        absA = None
        for d in (1, 2):
            op = ina.stencil(s2, [0.0, 1.0, 2.0, 1.0, 0.0], 2, dim=d)
            absA = op if absA is None else absA + op
        floor2 = 2.0**-53 * ina.operate(absA, x2, cutoff=0.0).norm() / b2.norm()
        out["laplace_linsolve"] = {
            "value": t2, "unit": "s", "what": "linsolve(laplacian, sin(pi x) sin(pi y)), 2 sweeps, maxdim 40, cutoff 1e-20, 2 refinement steps",
            "rel_residual": x2.rel_residual, "rel_residual_fp64_floor": floor2,
            "floor_what": "eps_64 * || |A| |x| || / ||b||: the residual that rounding x to FP64 alone can cause",
            "maxlinkdim": x2.maxlinkdim(),
            "max_err_vs_continuum": float(np.max(np.abs(got2 - exact2)) / np.max(np.abs(exact2))),
        }
    if want("config1"):
        # --- config 1: the reference's CPU case on the GPU ---------------------------
        L = 20
        s = ina.continuous_siteinds(ina.named_grid((L, 1)))
        X = np.random.default_rng(0).random((4096, 1))

        def cfg1():
            f = ina.exp_itn(s, k=-1.0) + ina.sin_itn(s, k=2 * np.pi)
            g = ina.operate(ina.second_derivative_operator(s), f, cutoff=1e-12, maxdim=32)
            return g.evaluate_batch(X), g.integrate()

        cfg1()
        t1, _ = _timed(cfg1)
        out["config1_latency"] = {"value": t1, "unit": "s",
                                  "what": "build f, build d2/dx2, apply+truncate (1e-12, 32), 4096 evals, integrate"}
        # small-batch evaluation latency: eager calls vs the captured plan (CUDA graph)
        import torch

        g1 = ina.operate(ina.second_derivative_operator(s), ina.exp_itn(s, k=-1.0) + ina.sin_itn(s, k=2 * np.pi),
                         cutoff=1e-12, maxdim=32)
        Xd1 = torch.tensor(X, dtype=torch.float64, device="cuda")
        cplx1 = g1.is_complex
        o1 = torch.empty(len(X), dtype=torch.complex128 if cplx1 else torch.float64, device="cuda")
        kind1 = ina._lib.OUT_C128 if cplx1 else ina._lib.OUT_F64
        d1 = (ctypes.c_int32 * 1)(1)

        def eager():
            g1.ctx.call("tnfa_evaluate", g1.handle, Xd1.data_ptr(), len(X), 1, d1, ina._lib.MEM_DEVICE,
                        o1.data_ptr(), kind1, ina._lib.MEM_DEVICE, ina._lib.PREC_F64)

        plan = g1.evaluation_plan(Xd1, o1)
        eager()
        te, _ = _timed(eager, 200)
        plan.launch()
        tg, _ = _timed(plan.launch, 200)
        plan.check()
        plan.close()
        out["small_batch_eval_latency"] = {
            "value": tg * 1e6, "unit": "us per call", "eager_us": te * 1e6, "points": len(X),
            "what": "config-1 network (path 20, FP64, bond <= 32) at 4096 device points: "
                    "captured plan replay (one graph launch) vs eager tnfa_evaluate"}
        # the same low-rank network at 10^7 device points: the fused small-bond
        # kernel (one launch, the tree walked per point on chip) in FP64 and FP32
        nbig = 10_000_000
        Xbig = torch.tensor(np.random.default_rng(5).random((nbig, 1)), dtype=torch.float64, device="cuda")
        obig = torch.empty(nbig, dtype=torch.float64, device="cuda")
        low = {}
        for name, net, pr in (("f64", g1, ina._lib.PREC_F64),
                              ("f32", g1.astype(ina._lib.F32), ina._lib.PREC_F32)):
            def big(net=net, pr=pr):
                net.ctx.call("tnfa_evaluate", net.handle, Xbig.data_ptr(), nbig, 1, d1, ina._lib.MEM_DEVICE,
                             obig.data_ptr(), ina._lib.OUT_F64, ina._lib.MEM_DEVICE, pr)
            big()
            tb, _ = _timed(big, 5)
            low[name] = {"value": nbig / tb, "unit": "points/s", "ms": tb * 1e3,
                         "compulsory_GBps": nbig * 16 / tb / 1e9}
        out["lowrank_eval"] = {
            "value": low["f64"]["value"], "unit": "points/s", "points": nbig, "f64": low["f64"],
            "f32": low["f32"], "maxlinkdim": g1.maxlinkdim(),
            "what": "config-1 network at 10^7 device points through the fused small-bond kernel; "
                    "compulsory traffic 16 B/point (x in, value out)"}
    if want("gradient"):
        # --- config 4: gradient of batched evaluation --------------------------------
        import torch

        L4 = 12
        s4 = ina.continuous_siteinds(ina.named_comb_tree((2, L4)),
                                     [[(1, j) for j in range(1, L4 + 1)], [(2, j) for j in range(1, L4 + 1)]])
        rng = np.random.default_rng(2)
        lay = s4.layout
        ts = {}
        for i, v in enumerate(lay.order):
            shape = (2, 32 if lay.parent[i] >= 0 else 1) + (32,) * len(lay.children[i])
            ts[v] = 0.1 * rng.standard_normal(shape)
        f4 = ina.ITensorNetworkFunction.from_tensors(s4, ts, ctx=ctx, dtype=ina._lib.F32)
        P4 = 1 << 20
        X4 = torch.tensor(rng.random((P4, 2)), device="cuda")
        dout = torch.tensor(rng.standard_normal(P4), device="cuda")
        g4 = torch.zeros(f4.info()[2], dtype=torch.float32, device="cuda")
        dims = (ctypes.c_int32 * 2)(1, 2)

        def grad():
            ctx.call("tnfa_evaluate_vjp", f4.handle, X4.data_ptr(), P4, 2, dims, 1, dout.data_ptr(), 1,
                     g4.data_ptr(), 1)

        grad()
        t4, _ = _timed(grad, 3)
        out["gradient"] = {"value": P4 / t4, "unit": "points/s", "points": P4,
                           "what": "tnfa_evaluate_vjp, comb 2x12 chi 32 FP32 (forward + outside messages + accumulation)"}
    return out


def roofline(stats: dict, fam: str | None, peaks: dict) -> dict | None:
    """Roofline of the dominant kernel family: algorithmic flops (one pass per
    product) over its CUDA-event time, against the sustained bf16 peak (the
    kernel runs back to back for the whole step, under the power cap); the
    executed tensor work counts every slice / split pass."""
    if not fam:
        return None
    st = stats[fam]
    achieved = st["flops"] / (st["ms"] / 1e3) / 1e12
    peak = peaks["bf16_tflops_sustained"]
    passes = MMA_PASSES.get(fam, 1)
    traffic, src = None, None
    per_point = {"contract_tc": TC2_DRAM_BYTES_PER_POINT,
                 "contract_oz": OZ_DRAM_BYTES_PER_POINT}.get(fam)
    if per_point and st["launches"]:
        # traffic grows with the points (their messages): scale to this run's
        # average points per launch of the family
        pts_per_launch = st["flops"] / st["launches"] / (2.0 * CHI ** 3)
        traffic = per_point * pts_per_launch
        src = "ncu dram__bytes_read+write of a smaller capture, scaled by points per launch"
    return {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic, "traffic_source": src,
            "kernel": fam,
            "kernel_share": st["ms"] / sum(v["ms"] for v in stats.values()),
            "peak_source": ("MEASURED_PEAKS.json bf16 sustained (kernel timed inside a long step)"
                            if "fallback" not in peaks else "fallback"),
            "frac_of_burst_peak": achieved / peaks["bf16_tflops"],
            "mma_passes": passes,
            "tensor_work_executed": achieved * passes,
            "frac_executed": achieved * passes / peak}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--points", type=int, default=10_000_000)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "mixed_fast", "f32", "f64"])
    ap.add_argument("--f64-points", type=int, default=1 << 15)
    ap.add_argument("--cpu-points", type=int, default=2048)
    ap.add_argument("--e2e-steps", type=int, default=2,
                    help="end-to-end repetitions (at most --steps)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--mps", type=int, default=512, help="config-5 batch size")
    ap.add_argument("--only", default="",
                    help="run only these secondary measurements (comma list of apply_truncate, "
                         "laplace, config1, gradient, integrate, mixed_fast) and print them; "
                         "no headline step")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch

    import itensornumericalanalysis as ina
    from itensornumericalanalysis import _build, _lib

    if not _build.LIB_PATH.exists():
        _build.build()
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    ctx = _lib.Context(local, stream.cuda_stream)
    if args.only:
        sec = secondary_measurements(ctx, ws, rank, args)
        if rank == 0:
            print(json.dumps({"secondary": sec}))
        return
    ina.set_default_context(ctx)

    s, ts = config3_tensors(1)
    f32net = ina.ITensorNetworkFunction.from_tensors(s, ts, ctx=ctx, dtype=_lib.F32)
    f64net = f32net.astype(_lib.F64)
    P = args.points
    Xh = config3_points(P, 1, offset=rank * P)
    Xd = torch.from_numpy(Xh).cuda()
    scaled = args.precision in ("mixed_fast", "f32")  # FP32 messages: mantissa + exponent out
    out_kind = _lib.OUT_F32_SCALED if scaled else _lib.OUT_F64
    out = (torch.empty(2 * P, dtype=torch.float32, device="cuda") if scaled
           else torch.empty(P, dtype=torch.float64, device="cuda"))
    dims = (ctypes.c_int32 * 3)(1, 2, 3)
    prec = {"mixed": _lib.PREC_MIXED, "mixed_fast": _lib.PREC_MIXED_FAST, "f32": _lib.PREC_F32,
            "f64": _lib.PREC_F64}[args.precision]
    net = f64net if args.precision == "f64" else f32net

    def step_device(n=P, x=Xd, o=out, which=net, pr=prec):
        ctx.call("tnfa_evaluate", which.handle, x.data_ptr(), n, 3, dims, _lib.MEM_DEVICE,
                 o.data_ptr(), out_kind, _lib.MEM_DEVICE, pr)

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    ctx.kernel_stats(reset=True)
    ctx.set_timing(True)
    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step_device()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    clk = clocks.stop()
    ctx.set_timing(False)
    t_dev = e0.elapsed_time(e1) / 1e3 / args.steps
    t_dev = max_over_ranks(t_dev, ws)
    stats = ctx.kernel_stats(reset=True)
    value = ws * P / t_dev
    if scaled:
        oh = out.cpu().numpy()
        got_all = np.ldexp(oh[:P].astype(np.float64), oh[P:].view(np.int32))
    else:
        got_all = out.cpu().numpy()

    # dominant kernel: live CUDA-event time and algorithmic flops
    fam = max(stats, key=lambda k: stats[k]["ms"]) if stats else None
    peaks = measured_peaks()
    roof = roofline(stats, fam, peaks)
    launches = sum(v["launches"] for v in stats.values()) // args.steps

    # end to end: pinned host X -> device -> result back, through the C ABI
    Xpin = torch.from_numpy(Xh).pin_memory()
    outpin = torch.empty(out.numel(), dtype=out.dtype).pin_memory()

    def step_e2e():
        ctx.call("tnfa_evaluate", net.handle, Xpin.data_ptr(), P, 3, dims, _lib.MEM_HOST,
                 outpin.data_ptr(), out_kind, _lib.MEM_HOST, prec)

    n_e2e = max(1, min(args.e2e_steps, args.steps))
    step_e2e()
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        step_e2e()
    torch.cuda.synchronize()
    t_e2e = max_over_ranks((time.perf_counter() - t0) / n_e2e, ws)

    # accuracy against the FP64 plain path on the first points, and its rate
    nf = min(args.f64_points, P)
    o64 = torch.empty(nf, dtype=torch.float64, device="cuda")

    def step_f64():
        ctx.call("tnfa_evaluate", f64net.handle, Xd.data_ptr(), nf, 3, dims, _lib.MEM_DEVICE,
                 o64.data_ptr(), _lib.OUT_F64, _lib.MEM_DEVICE, _lib.PREC_F64)

    step_f64()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    step_f64()
    torch.cuda.synchronize()
    f64_rate = nf / (time.perf_counter() - t0)
    ref64 = o64.cpu().numpy()
    got = got_all[:nf]
    rel = np.abs(got - ref64) / np.abs(ref64)
    gate = {"limit": 1e-8, "max_rel": float(np.max(rel)), "points": nf,
            "passed": bool(np.max(rel) <= 1e-8)}

    integ = integrate_rates(f32net, f64net, peaks)
    dtype = {"mixed": "bf16 integer slices (26 passes, exact fp32 accumulation), fp64 messages",
             "mixed_fast": "bf16 hi/lo (3 passes), fp32 messages", "f32": "f32", "f64": "f64"}
    result = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_dev * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": dtype[args.precision],
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "points_per_gpu": P, "vertices": N_VERT, "chi": CHI,
                   "precision": args.precision,
                   "output": "f32 mantissa + i32 exponent" if scaled else "f64",
                   "l2": "inputs larger than L2 (X 240 MB/rank at 1e7 points, tensors 470 MB)"},
        "roofline": roof,
        "e2e": {"value": ws * P / t_e2e, "unit": "points/s", "h2d_bytes_per_step": P * 3 * 8,
                "d2h_bytes_per_step": out.numel() * out.element_size(), "steps": n_e2e},
        "gpu_launches": int(launches),
        "clocks": clk,
        "fp64_plain": {"value": f64_rate, "unit": "points/s", "sample_points": nf,
                       "speedup_of_value": value / ws / f64_rate},
        "rel_err_vs_fp64": {"median": float(np.median(rel)), "max": float(np.max(rel)),
                            "normwise": float(np.linalg.norm(got - ref64) / np.linalg.norm(ref64)),
                            "points": nf, "what": "per point |v - v_f64| / |v_f64|"},
        "accuracy_gate": gate,
        "kernels": {k: {"launches_per_step": v["launches"] // args.steps,
                        "ms_per_step": v["ms"] / args.steps} for k, v in stats.items()},
        "integrate": dict(integ, what="integrate() of the benchmark network; bytes = tensor bytes "
                                      "(read once), time per call incl. the final readback",
                          peak_source="MEASURED_PEAKS.json hbm_gbs"),
    }
    del Xpin, outpin
    if not args.no_secondary:
        result["secondary"] = secondary_measurements(ctx, ws, rank, args, f32net=f32net,
                                                     f64net=f64net, Xd=Xd, ref64=ref64)
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        rate, busy, pts, vals = cpu_baseline(args.cpu_points, cores)
        # the oracle's values against the device paths on the same points
        chk = f64net.evaluate_batch(pts, [1, 2, 3], precision="f64")
        n_or = min(len(pts), nf)
        result["cpu_baseline"] = {
            "value": rate, "unit": "points/s", "cores": cores, "kind": "port",
            "sample": f"{args.cpu_points} points of the workload, oracle batched FP64 evaluation "
                      f"(numpy + BLAS), {cores} threads, {busy:.2f} s",
            "rel_err_device_f64_vs_oracle": float(np.max(np.abs(chk - vals) / np.abs(vals))),
            "rel_err_headline_vs_oracle": float(np.max(np.abs(got_all[:n_or] - vals[:n_or]) /
                                                       np.abs(vals[:n_or]))),
        }
    if rank == 0:
        print(json.dumps(result), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    if args.precision == "mixed" and not gate["passed"]:
        print(f"accuracy gate failed: max per-point relative error {gate['max_rel']:.3e} > 1e-8",
              file=sys.stderr, flush=True)
        sys.exit(3)


if __name__ == "__main__":
    main()

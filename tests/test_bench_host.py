"""bench.py's host-side arithmetic (no device): the roofline object of the
dominant kernel family, from the library's per-family CUDA-event stats."""
import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import bench  # noqa: E402


PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 2000.0, "bf16_tflops_sustained": 1700.0}


def test_roofline_of_the_sliced_kernel():
    pts = 131072
    fl = 2.0 * bench.CHI**3 * pts * 28  # 28 two-child vertices, one launch each
    stats = {"contract_oz": {"launches": 28, "ms": 10.0, "flops": fl, "bytes": 0.0},
             "digitize": {"launches": 1, "ms": 0.5, "flops": 0.0, "bytes": 0.0}}
    r = bench.roofline(stats, "contract_oz", PEAKS)
    assert r["achieved"] == pytest.approx(fl / 1e-2 / 1e12)
    assert r["frac"] == pytest.approx(r["achieved"] / 1700.0)
    assert r["frac_of_burst_peak"] == pytest.approx(r["achieved"] / 2000.0)
    assert r["mma_passes"] == bench.MMA_PASSES["contract_oz"] == 26
    assert r["frac_executed"] == pytest.approx(26 * r["frac"])
    # DRAM traffic per launch: the captured bytes per point times the points one launch covers
    assert r["traffic"] == pytest.approx(bench.OZ_DRAM_BYTES_PER_POINT * pts)
    assert r["kernel_share"] == pytest.approx(10.0 / 10.5)
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"


def test_roofline_without_a_family():
    assert bench.roofline({}, None, PEAKS) is None


class _Proc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_sampler_parses_nvidia_smi_lines():
    """The clocks object of the JSON line: median SM clock under load, the
    maximum, and every throttle reason seen Active."""
    c = bench.ClockSampler(0)
    c.proc = _Proc()
    c.lines = ["1965, 2070, 900.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
               "2070, 2070, 1000.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
               "2010, 2070, 950.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
               "garbage line"]
    r = c.stop()
    assert r["sm_mhz"] == 2010.0 and r["sm_max_mhz"] == 2070.0 and r["samples"] == 3
    assert r["reasons"] == ["sw_power_cap"]


def test_clock_sampler_without_nvidia_smi():
    assert bench.ClockSampler(0).stop()["reasons"] == ["nvidia-smi unavailable"]


def test_uneven_mps_batch_follows_the_config():
    """512 MPS, L in 10..30, chi in 8..128 capped per bond at min(chi, 2^k,
    2^(L-k)), unit-Frobenius Gaussian tensors, the same batch for the same seed."""
    import numpy as np

    from itensornumericalanalysis.workloads import uneven_mps_batch

    batch = uneven_mps_batch(n=512, seed=3)
    again = uneven_mps_batch(n=4, seed=3)
    assert len(batch) == 512
    Ls, chis = [], []
    for (s, ts) in batch:
        order = s.layout.order
        L = len(order)
        Ls.append(L)
        assert 10 <= L <= 30
        bonds = [np.shape(ts[v])[2] for v in order[:-1]]
        chi = max(bonds)
        chis.append(chi)
        # chi is the largest bond: either the drawn chi or, when every bond is
        # capped, the largest cap; either way every bond is min(chi, caps)
        assert bonds == [min(chi, 2**k, 2 ** (L - k)) for k in range(1, L)]
        for v in order:
            assert abs(np.linalg.norm(ts[v]) - 1.0) < 1e-12
    assert min(Ls) == 10 and max(Ls) == 30
    assert 8 <= min(chis) and max(chis) <= 128 and max(chis) >= 100
    for (s, ts), (s2, ts2) in zip(batch[:4], again):
        assert all(np.array_equal(ts[v], ts2[w]) for v, w in zip(s.layout.order, s2.layout.order))


def test_config3_workload_shapes():
    """60-vertex heap binary tree, 3 variables x 20 digits, chi = 128: 29
    vertices with two children (the root among them), one with one child, 30
    leaves; FP32 tensors of unit Frobenius norm; 470 MB in all."""
    import numpy as np

    s, ts = bench.config3_tensors(1)
    lay = s.layout
    nch = [len(c) for c in lay.children]
    assert len(lay.order) == 60 and nch.count(0) == 30 and nch.count(2) == 29 and nch.count(1) == 1
    assert sorted(s.ndigits(d) for d in (1, 2, 3)) == [20, 20, 20]
    nbytes = sum(t.nbytes for t in ts.values())
    assert abs(nbytes / 1e6 - 470) < 10
    assert all(t.dtype == np.float32 and abs(float(np.linalg.norm(t)) - 1) < 1e-5 for t in ts.values())
    X = bench.config3_points(1000, 1)
    assert X.shape == (1000, 3) and X.min() >= 0 and X.max() < 1

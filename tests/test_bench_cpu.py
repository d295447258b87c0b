"""Host-side pieces of bench.py, on CPU: the kernel names it reports, the
DRAM traffic it reads from the committed ncu summaries, the count of agents
the reference's dispatch updates, and the seeded synthetic agents."""
import os
import sys

import numpy as np
import pytest

import oracle
from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_every_agent_shape_has_a_kernel_name():
    # shape-table indices 0..14: 9-11 and 13-14 run the persistent kernel
    names = [bench.agents_kernel_name(s) for s in range(15)]
    assert names.count("agents_persistent_kernel") == 5
    assert set(names) == {"agents_kernel", "agents_persistent_kernel"}
    assert bench.trail_kernel_name(7, 1) == bench.trail_kernel_name(9, 0) == "trail_stream_kernel"
    assert bench.trail_kernel_name(10, 1) == "trail_tma_kernel"
    assert bench.trail_kernel_name(3, 1) == "trail_gauss_kernel"
    assert bench.trail_kernel_name(3, 0) == "trail_box3_kernel"


@pytest.mark.parametrize("key", sorted(bench.TRAFFIC_PROFILES))
def test_profiled_traffic_is_read_from_the_committed_summary(key):
    workload, kernel = key
    traffic, source = bench.profiled_traffic(workload, kernel)
    assert source is not None and os.path.exists(os.path.join(ROOT, source)), key
    W, H, n = bench.CONFIGS[workload][:3]
    algorithmic = 32.0 * n if kernel.startswith("agents") else 8.0 * W * H
    # the summaries hold one launch's DRAM bytes: near the algorithmic bytes,
    # above them only by the sensor and deposit traffic that reaches DRAM
    assert 0.5 * algorithmic < traffic < 3.0 * algorithmic, (key, traffic, algorithmic)


def test_profiled_traffic_needs_a_matching_capture():
    assert bench.profiled_traffic("plain-4096", "agents_kernel") == (None, None)
    assert bench.profiled_traffic("plain-512", "trail_stream_kernel") == (None, None)


@pytest.mark.parametrize("n", [1, 63, 64, 65, 4_194_240, 4_194_241, 4_194_304, 10_000_000, 16_777_216,
                               67_108_864])
def test_reference_dispatch_visited_matches_the_visit_counts(n):
    """bench's closed form for the agents the reference's dispatch updates
    is the first index with no visit (every lower index has one)."""
    k = bench.reference_dispatch_visited(n)
    assert 0 < k <= n
    probe = np.unique(np.clip(np.array([0, 1, k // 2, k - 2, k - 1, k, k + 1, n - 1], np.int64), 0, n - 1))
    visits = oracle.dispatch_visits(n, probe.astype(np.uint64))
    assert np.all(visits[probe < k] >= 1), (n, k)
    assert np.all(visits[probe >= k] == 0), (n, k)
    if n <= 4_194_240:
        assert k == n


def test_synthetic_agents_are_seeded_and_in_range():
    W, H = 64, 48
    a = bench.make_agents(10_000, W, H, 1.0, 2.0, seed=3)
    b = bench.make_agents(10_000, W, H, 1.0, 2.0, seed=3)
    assert a.dtype == np.float32 and a.shape == (10_000, 4)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert (a[:, 0] >= 0).all() and (a[:, 0] < W).all()
    assert (a[:, 1] >= 0).all() and (a[:, 1] < H).all()
    assert (a[:, 2] >= 0).all() and (a[:, 2] <= np.float32(2 * np.pi)).all()
    assert (a[:, 3] >= 1.0).all() and (a[:, 3] <= 2.0).all()


def test_clock_sampler_names_the_process_gpu(monkeypatch):
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES", raising=False)
    assert bench.ClockSampler.smi_id(0) == "0"
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "5,GPU-1234")
    assert bench.ClockSampler.smi_id(0) == "5"
    assert bench.ClockSampler.smi_id(1) == "GPU-1234"
    assert bench.ClockSampler.smi_id(2) == "2"


def test_clock_summary_reads_reasons():
    s = bench.ClockSampler(0)
    s.lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 2040, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
               "garbage"]
    out = s.summary()
    assert out["sm_mhz"] == 2055.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"] and out["samples"] == 2

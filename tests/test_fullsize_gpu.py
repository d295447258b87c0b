"""Checks at the benchmark sizes: 4096x4096 with 16,777,216 agents and
8192x8192 with 67,108,864 agents.

  * one and two steps from an identical state, bit-exact against the oracle
    (agents, the step's deposit counts and the trail), with Morton reordering on;
  * properties of a 200-step run that hold at any size: the deposit counts are
    exactly the histogram of the agents' cells, the trail stays in [0, 1],
    headings stay in [0, 2pi), and the run is bit-identical whatever the
    reorder schedule and graph chunking;
  * long-run statistics (trail mass, value histogram, radially averaged power
    spectrum) of a 1000-step 512x512 run against the oracle's.
"""
import numpy as np
import pytest

import oracle
from conftest import agents_uniform, config0_params
from test_parity_gpu import assert_bitexact, make_sim

pytestmark = pytest.mark.gpu

SIZES = {
    "4096": (4096, 4096, 16_777_216, 1.0, 2.0, 9.0),
    "8192": (8192, 8192, 67_108_864, 1.5, 3.0, 18.0),
}


def bench_params(W, H, lo, hi, dist, sensor_mode=0):
    return config0_params(W, H, decay_mode=1, blur_mode=1, agent_speed_min=lo, agent_speed_max=hi,
                          agent_sensor_distance=dist, sensor_mode=sensor_mode)


def expected_counts(agents, W, H):
    """The deposit cells of compute.wgsl:135-141 from the agents' new
    positions: i32(x), i32(y), skipped outside the grid."""
    cx = agents[:, 0].astype(np.int64)  # x >= 0 after the wrap: truncation
    cy = agents[:, 1].astype(np.int64)
    ok = (cx >= 0) & (cx < W) & (cy >= 0) & (cy < H)
    return np.bincount(cy[ok] * W + cx[ok], minlength=W * H).astype(np.uint32).reshape(H, W)


@pytest.mark.parametrize("size,sensor_mode", [("4096", 0), ("8192", 0), ("4096", 1)])
def test_full_size_steps_bitexact(gpu, size, sensor_mode):
    W, H, n, lo, hi, dist = SIZES[size]
    p = bench_params(W, H, lo, hi, dist, sensor_mode)
    agents = agents_uniform(n, W, H, lo, hi, seed=11)
    trail = np.random.default_rng(12).random((H, W), dtype=np.float32)
    sim = make_sim(W, H, n, p, agents, trail)
    # Morton order before every step; counts kept for the comparison
    sim.set_options(reorder_every=1, exact_counts=1)
    ca, ct = agents.copy(), trail.copy()
    del agents, trail
    for step in range(2):
        sim.step(1)
        counts = oracle.run(p, W, H, ca, ct, 1, record_counts=True)
        assert_bitexact(sim.download_deposit_counts(), counts[0], f"counts step {step}")
        assert_bitexact(sim.download_agents(), ca, f"agents step {step}")
        assert_bitexact(sim.download_trail(), ct, f"trail step {step}")
    sim.close()


def test_full_size_run_properties(gpu):
    W, H, n, lo, hi, dist = SIZES["4096"]
    p = bench_params(W, H, lo, hi, dist)
    agents = agents_uniform(n, W, H, lo, hi, seed=13)
    a = make_sim(W, H, n, p, agents)
    a.set_options(reorder_every=50, graph_chunk=50, exact_counts=1)
    a.step(200)
    got = a.download_agents()
    counts = a.download_deposit_counts()
    trail = a.download_trail()
    a.close()
    # the last step's counts are the histogram of the agents' cells
    assert_bitexact(counts, expected_counts(got, W, H), "counts vs agent cells")
    assert int(counts.sum()) <= n
    # state ranges
    assert np.isfinite(trail).all() and trail.min() >= 0.0 and trail.max() <= 1.0
    assert (got[:, 2] >= 0).all() and (got[:, 2] < np.float32(2 * np.pi) + np.float32(1e-6)).all()
    assert (got[:, 0] >= 0).all() and (got[:, 0] <= W).all() and (got[:, 1] >= 0).all() and (got[:, 1] <= H).all()
    # invariance: no reordering, no graphs, a different chunking, the
    # streaming trail kernel with deposit marks -> the same bits
    b = make_sim(W, H, n, p, agents)
    b.set_options(reorder_every=0, use_graphs=0, trail_tile=8)
    b.step(73)
    b.set_options(use_graphs=1, graph_chunk=31)
    b.step(127)
    assert_bitexact(b.download_agents(), got, "agents, other schedule")
    assert_bitexact(b.download_trail(), trail, "trail, other schedule")
    b.close()


def radial_spectrum(t, nbins=32):
    f = np.abs(np.fft.fft2(t - t.mean())) ** 2
    H, W = t.shape
    ky = np.fft.fftfreq(H)[:, None]
    kx = np.fft.fftfreq(W)[None, :]
    k = np.sqrt(kx * kx + ky * ky)
    bins = np.minimum((k / k.max() * nbins).astype(int), nbins - 1)
    return np.bincount(bins.ravel(), weights=f.ravel(), minlength=nbins) / np.bincount(bins.ravel(), minlength=nbins)


def test_long_run_statistics_match_oracle(gpu):
    """1000 steps of the 512x512 / 65,536-agent configuration: the dynamics
    are chaotic, so the run is compared through its statistics (and, since
    every operation is pinned, also bit for bit)."""
    W = H = 512
    n = 65_536
    p = config0_params(W, H)
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=0)
    sim = make_sim(W, H, n, p, agents)
    sim.set_options(reorder_every=100)
    sim.step(1000)
    gt, ga = sim.download_trail(), sim.download_agents()
    sim.close()
    ca, ct = agents.copy(), np.zeros((H, W), np.float32)
    oracle.run(p, W, H, ca, ct, 1000)
    g64, c64 = gt.astype(np.float64), ct.astype(np.float64)
    assert abs(g64.sum() - c64.sum()) <= 1e-6 * max(1.0, abs(c64.sum()))
    hg, _ = np.histogram(gt, bins=64, range=(0.0, 1.0))
    hc, _ = np.histogram(ct, bins=64, range=(0.0, 1.0))
    assert np.array_equal(hg, hc)
    sg, sc = radial_spectrum(g64), radial_spectrum(c64)
    assert np.allclose(sg, sc, rtol=1e-6, atol=0.0)
    assert_bitexact(gt, ct, "trail after 1000 steps")
    assert_bitexact(ga, ca, "agents after 1000 steps")

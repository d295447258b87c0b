"""slime_step_noalloc: the step for callers that may not allocate device
memory while they run (their device memory is all reserved up front, or an
allocation's device synchronisation would stall them).  It takes the agents
and both trails as device pointers and keeps its deposit counts in a fixed
array inside the library.  Checked bit for bit against slime_step on the same
state, over two calls in a row (the second reads what the first wrote, and
finds the shared count array cleared again).  This file is collected last on
purpose."""
import ctypes as C

import numpy as np
import pytest

from conftest import agents_uniform, config0_params

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_step_noalloc_matches_slime_step_twice(gpu):
    import torch

    import slime_gb300 as sg
    L = sg.lib()
    W, H, n = 320, 200, 30001
    for decay_mode, blur_mode in ((1, 1), (0, 0)):
        p = config0_params(W, H, decay_mode=decay_mode, blur_mode=blur_mode, agent_speed_min=30.0,
                           agent_speed_max=50.0, agent_jitter=0.3, decay_factor=0.97 if decay_mode else 10.0)
        agents = agents_uniform(n, W, H, 30.0, 50.0, seed=5)
        trail = np.random.default_rng(6).random((H, W), dtype=np.float32)

        # the existing entry point
        with sg.Simulation(W, H, n, p) as sim:
            sim.upload_agents(agents)
            sim.upload_trail(trail)
            sim.step(1)
            a1, t1 = sim.download_agents(), sim.download_trail()
            sim.step(1)
            a2, t2 = sim.download_agents(), sim.download_trail()

        # the allocation-free entry point on caller-owned device buffers
        dev = torch.device("cuda", 0)
        cols = [torch.tensor(np.ascontiguousarray(agents[:, j]), device=dev) for j in range(4)]
        ta = torch.tensor(trail, device=dev)
        tb = torch.empty_like(ta)
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        for (src, dst), (aw, tw) in zip(((ta, tb), (tb, ta)), ((a1, t1), (a2, t2))):
            rc = L.slime_step_noalloc(C.byref(p), W, H, n, *[_ptr(c) for c in cols], _ptr(src), _ptr(dst), stream)
            assert rc == 0
            torch.cuda.synchronize()
            got = np.stack([c.cpu().numpy() for c in cols], axis=1)
            assert np.array_equal(got.view(np.uint32), aw.view(np.uint32))
            assert np.array_equal(dst.cpu().numpy().view(np.uint32), tw.view(np.uint32))


def test_step_noalloc_scratch_beyond_the_array_and_overlapping(gpu):
    """The caller-owned count array: a 2048x1024 trail (twice the fixed
    array) matches slime_step bit for bit, and two colonies stepped on two
    streams at once, each with its own count array, match their sequential
    runs."""
    import torch

    import slime_gb300 as sg
    L = sg.lib()
    W, H, n = 2048, 1024, 200_000
    p = config0_params(W, H, agent_speed_min=30.0, agent_speed_max=50.0, agent_jitter=0.3)
    dev = torch.device("cuda", 0)
    runs = []
    for seed in (11, 12):
        agents = agents_uniform(n, W, H, 30.0, 50.0, seed=seed)
        trail = np.random.default_rng(seed).random((H, W), dtype=np.float32)
        with sg.Simulation(W, H, n, p) as sim:
            sim.upload_agents(agents)
            sim.upload_trail(trail)
            sim.step(2)
            want = sim.download_agents(), sim.download_trail()
        cols = [torch.tensor(np.ascontiguousarray(agents[:, j]), device=dev) for j in range(4)]
        ta = torch.tensor(trail, device=dev)
        tb = torch.empty_like(ta)
        counts = torch.full((H * W,), 7, dtype=torch.int32, device=dev)  # cleared by each call
        runs.append((cols, ta, tb, counts, torch.cuda.Stream(), want))
    torch.cuda.synchronize()
    for src_dst in ((1, 2), (2, 1)):
        for cols, ta, tb, counts, st, _ in runs:  # both colonies in flight at once
            src, dst = (ta, tb) if src_dst == (1, 2) else (tb, ta)
            rc = L.slime_step_noalloc_scratch(C.byref(p), W, H, n, *[_ptr(c) for c in cols], _ptr(src), _ptr(dst),
                                              _ptr(counts), C.c_void_p(st.cuda_stream))
            assert rc == 0
    torch.cuda.synchronize()
    for cols, ta, tb, counts, st, (wa, wt) in runs:
        got = np.stack([c.cpu().numpy() for c in cols], axis=1)
        assert np.array_equal(got.view(np.uint32), wa.view(np.uint32))
        assert np.array_equal(ta.cpu().numpy().view(np.uint32), wt.view(np.uint32))
    cols, ta, tb, counts, st, _ = runs[0]
    rc = L.slime_step_noalloc_scratch(C.byref(p), W, H, n, *[_ptr(c) for c in cols], _ptr(ta), _ptr(tb), None, None)
    assert rc == -1


def test_step_noalloc_rejects_sizes_beyond_its_array(gpu):
    import torch

    import slime_gb300 as sg
    L = sg.lib()
    dev = torch.device("cuda", 0)
    big = torch.zeros(2048 * 1024, device=dev)
    out = torch.zeros_like(big)
    x = torch.zeros(4, device=dev)
    p = config0_params(2048, 1024)
    rc = L.slime_step_noalloc(C.byref(p), 2048, 1024, 4, _ptr(x), _ptr(x), _ptr(x), _ptr(x), _ptr(big), _ptr(out),
                              None)
    assert rc == -1
    p = config0_params(1, 64)
    rc = L.slime_step_noalloc(C.byref(p), 1, 64, 4, _ptr(x), _ptr(x), _ptr(x), _ptr(x), _ptr(big), _ptr(out), None)
    assert rc == -1


def test_step_noalloc_in_the_reference_dispatch(gpu):
    """4,264,240 agents in the reference's dispatch (4,465 never updated,
    most of the rest visited twice) at deposition 0.3, so every extra visit's
    deposit shows in the trail: two calls against the oracle."""
    import torch

    import oracle
    import slime_gb300 as sg
    L = sg.lib()
    W, H, n = 320, 200, 4_264_240
    p = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=10.0, pheromone_deposition_amount=0.3,
                       agent_speed_min=30.0, agent_speed_max=50.0, dispatch_mode=1)
    agents = agents_uniform(n, W, H, 0.5, 80.0, seed=7)
    trail = np.random.default_rng(8).random((H, W), dtype=np.float32)
    dev = torch.device("cuda", 0)
    cols = [torch.tensor(np.ascontiguousarray(agents[:, j]), device=dev) for j in range(4)]
    ta = torch.tensor(trail, device=dev)
    tb = torch.empty_like(ta)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ca, ct = agents.copy(), trail.copy()
    for src, dst in ((ta, tb), (tb, ta)):
        rc = L.slime_step_noalloc(C.byref(p), W, H, n, *[_ptr(c) for c in cols], _ptr(src), _ptr(dst), stream)
        assert rc == 0
        torch.cuda.synchronize()
        oracle.run(p, W, H, ca, ct, 1)
        got = np.stack([c.cpu().numpy() for c in cols], axis=1)
        assert np.array_equal(got.view(np.uint32), ca.view(np.uint32))
        assert np.array_equal(dst.cpu().numpy().view(np.uint32), ct.view(np.uint32))

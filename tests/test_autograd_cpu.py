"""The torch.autograd.Function role (slime_gb300.autograd.TrailChain) on
CPU, over a stand-in for the simulation whose backward returns known
gradients: the wiring, not the adjoint (the adjoint itself is compared with
the FP64 oracle in test_adjoint_gpu.py)."""
import numpy as np
import torch

from slime_gb300.autograd import trail_chain


class FakeSim:
    W, H = 6, 4

    def __init__(self):
        from slime_gb300 import SlimeParams
        self.p = SlimeParams()
        self.calls = []

    def params(self):
        return self.p

    def set_params(self, p):
        self.p = p

    def upload_agents(self, a):
        self.calls.append(("agents", a.shape))

    def upload_trail(self, t):
        self.trail = t.copy()

    def forward_record(self, n, k):
        self.calls.append(("record", n, k))

    def download_trail(self):
        return 2.0 * self.trail

    def backward(self, g, want_trail_grad=True):
        from slime_gb300 import SlimeGrads
        self.g = g.copy()
        out = SlimeGrads()
        out.d_decay_factor, out.d_diffusion_rate, out.d_deposition_amount = 1.5, -2.0, 0.25
        return out, (3.0 * g).reshape(self.H, self.W) if want_trail_grad else None


def test_gradients_reach_tensor_parameters_in_their_dtype():
    sim = FakeSim()
    t0 = torch.rand(4, 6, requires_grad=True)
    decay = torch.tensor(0.97, dtype=torch.float32, requires_grad=True)
    rate = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    out = trail_chain(t0, decay, rate, 0.3, sim, 7, 3, np.zeros((5, 4), np.float32))
    assert sim.calls == [("agents", (5, 4)), ("record", 7, 3)]
    assert abs(sim.p.decay_factor - 0.97) < 1e-6 and sim.p.pheromone_deposition_amount == np.float32(0.3)
    out.sum().backward()
    assert np.array_equal(sim.g, np.ones((4, 6), np.float32))
    assert torch.equal(t0.grad, torch.full((4, 6), 3.0))
    assert decay.grad.dtype == torch.float32 and float(decay.grad) == 1.5
    assert rate.grad.dtype == torch.float64 and float(rate.grad) == -2.0


def test_no_trail_gradient_when_the_trail_needs_none():
    sim = FakeSim()
    t0 = torch.rand(4, 6)
    dep = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    out = trail_chain(t0, 0.97, 0.5, dep, sim, 2, 1, np.zeros((1, 4), np.float32))
    (out * 2).sum().backward()
    assert float(dep.grad) == 0.25 and t0.grad is None

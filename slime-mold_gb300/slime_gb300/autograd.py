"""torch.autograd.Function over the checkpointed adjoint of the C ABI.

TrailChain.apply(trail0, decay, rate, deposition, sim, n_steps, ckpt_every,
agents) runs n_steps of the simulation from (agents, trail0) on the GPU with
the three trail-chain parameters replaced, recording checkpoints, and returns
the final trail.  Its backward calls slime_backward: gradients of the loss
with respect to trail0, decay_factor, diffusion_rate and
pheromone_deposition_amount with the agent trajectories held fixed (steering
is piecewise constant in the trail, so its a.e. derivative is zero).

Tensors cross the ABI through host memory (CPU float32 tensors).
"""
import numpy as np
import torch


class TrailChain(torch.autograd.Function):
    @staticmethod
    def forward(ctx, trail0, decay, rate, deposition, sim, n_steps, ckpt_every, agents):
        p = sim.params()
        p.decay_factor = float(decay)
        p.diffusion_rate = float(rate)
        p.pheromone_deposition_amount = float(deposition)
        sim.set_params(p)
        sim.upload_agents(np.ascontiguousarray(agents, np.float32))
        sim.upload_trail(trail0.detach().to(torch.float32).cpu().numpy())
        sim.forward_record(int(n_steps), int(ckpt_every))
        out = torch.from_numpy(sim.download_trail().copy())
        ctx.sim = sim
        return out

    @staticmethod
    def backward(ctx, grad_out):
        g = grad_out.detach().to(torch.float32).cpu().contiguous().numpy()
        grads, d0 = ctx.sim.backward(g)
        f64 = torch.float64
        return (torch.from_numpy(d0), torch.tensor(grads.d_decay_factor, dtype=f64),
                torch.tensor(grads.d_diffusion_rate, dtype=f64), torch.tensor(grads.d_deposition_amount, dtype=f64),
                None, None, None, None)


def trail_chain(trail0, decay, rate, deposition, sim, n_steps, ckpt_every, agents):
    """Functional form of TrailChain.apply."""
    return TrailChain.apply(trail0, decay, rate, deposition, sim, n_steps, ckpt_every, agents)

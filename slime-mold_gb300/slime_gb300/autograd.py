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
        # a gradient goes back only to the parameters given as tensors, in
        # their own dtype (autograd refuses one for a plain number)
        ctx.param_dtypes = [x.dtype if torch.is_tensor(x) else None for x in (decay, rate, deposition)]
        return out

    @staticmethod
    def backward(ctx, grad_out):
        g = grad_out.detach().to(torch.float32).cpu().contiguous().numpy()
        grads, d0 = ctx.sim.backward(g, want_trail_grad=ctx.needs_input_grad[0])
        values = (grads.d_decay_factor, grads.d_diffusion_rate, grads.d_deposition_amount)
        dparams = [torch.tensor(v, dtype=dt) if dt is not None else None for v, dt in zip(values, ctx.param_dtypes)]
        return (torch.from_numpy(d0) if d0 is not None else None, *dparams, None, None, None, None)


def trail_chain(trail0, decay, rate, deposition, sim, n_steps, ckpt_every, agents):
    """Functional form of TrailChain.apply."""
    return TrailChain.apply(trail0, decay, rate, deposition, sim, n_steps, ckpt_every, agents)

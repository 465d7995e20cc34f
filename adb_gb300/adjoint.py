"""Differentiable rollouts of the GPU step (a torch.autograd.Function).

``rollout(sim, q0, v0, mu, n_steps, every)`` advances ``n_steps`` frames with
``ABD.implicit_euler`` and returns the final ``(q, v)``; gradients with respect to the
initial state, the initial velocities and the friction coefficient come from the adjoint
of each converged frame (``abd_adjoint_frame``: implicit differentiation on the GPU). Forward states are kept every ``every`` frames (every frame by
default: a state is 24 doubles per body); the backward pass recomputes the frames between
checkpoints from the one before them and walks each segment in reverse. The frame's velocity
update v_{t+1} = (q_{t+1} - q_t) / dt (model/abd.cpp:128-139) is differentiated here.

The adjoint system uses the exact Jacobian of the frame's optimality condition at its
solution: the Hessian without PSD projection (the ground barrier's full second
derivative), plus the dependence of every friction multiplier and tangent frame on the
configuration (ground, point-triangle and edge-edge; the reference recomputes them at
every Newton iterate, so the converged state carries them at its own positions). It is
solved by GMRES preconditioned with the forward step's Newton matrix. Gradients match
central differences of the reference step to the finite differences' resolution.
"""
from __future__ import annotations

import numpy as np
import torch

from .abd import ABD


class Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q0, v0, mu, sim: ABD, n_steps: int, every: int):
        sim.set_friction(float(mu))
        q = q0.detach().cpu().numpy().astype(np.float64).copy()
        v = v0.detach().cpu().numpy().astype(np.float64).copy()
        ckpt = {0: (q.copy(), v.copy())}
        sim.set_state(q, v)
        for t in range(n_steps):
            sim.step(1)
            if (t + 1) % every == 0 and t + 1 < n_steps:
                ckpt[t + 1] = sim.state()
        qT, vT = sim.state()
        ckpt[n_steps] = (qT.copy(), vT.copy())
        ctx.sim, ctx.n, ctx.ckpt, ctx.mu = sim, n_steps, ckpt, float(mu)
        return torch.from_numpy(qT.copy()), torch.from_numpy(vT.copy())

    @staticmethod
    def backward(ctx, gqT, gvT):
        sim, n, ckpt = ctx.sim, ctx.n, ctx.ckpt
        # The simulation may have run other rollouts (another mu, another state) since this
        # forward pass: recompute and differentiate with this rollout's friction, and hand
        # the simulation back as it was found.
        saved_state, saved_mu, saved_iter = sim.state(), sim.friction, sim.iter
        sim.set_friction(ctx.mu)
        try:
            return Rollout._backward(ctx, sim, n, ckpt, gqT, gvT)
        finally:
            sim.set_friction(saved_mu)
            sim.set_state(*saved_state)
            sim.iter = saved_iter

    @staticmethod
    def _backward(ctx, sim, n, ckpt, gqT, gvT):
        dt = sim.config.dt
        shape = ckpt[0][0].shape
        gq = np.zeros(shape) if gqT is None else gqT.detach().cpu().numpy().astype(np.float64).copy()
        gv = np.zeros(shape) if gvT is None else gvT.detach().cpu().numpy().astype(np.float64).copy()
        gmu = 0.0
        t_end = n
        for s0 in sorted((k for k in ckpt if k < n), reverse=True):
            # states s0 .. t_end of the segment: stored ones are reused, the rest recomputed
            states = [ckpt[s0]]
            stepped = False
            for t in range(s0, t_end):
                if t + 1 in ckpt:
                    states.append(ckpt[t + 1])
                    stepped = False
                    continue
                if not stepped:
                    sim.set_state(*states[-1])
                sim.step(1)
                states.append(sim.state())
                stepped = True
            for t in range(t_end - 1, s0 - 1, -1):
                (q_t, v_t), (q_n, _) = states[t - s0], states[t - s0 + 1]
                # v_{t+1} = (q_{t+1} - q_t) / dt
                gq_n = gq + gv / dt
                gq_t, gv_t, gm = sim.adjoint_frame(q_t, v_t, q_n, gq_n)
                gq, gv = gq_t - gv / dt, gv_t
                gmu += gm
            t_end = s0
        return torch.from_numpy(gq), torch.from_numpy(gv), torch.tensor(gmu, dtype=torch.float64), None, None, None


def rollout(sim: ABD, q0, v0, mu, n_steps: int, every: int = 1):
    """Differentiable (q_T, v_T) after n_steps frames from (q0, v0) with friction mu."""
    mu = mu if torch.is_tensor(mu) else torch.tensor(float(mu), dtype=torch.float64)
    return Rollout.apply(q0, v0, mu, sim, int(n_steps), int(every))

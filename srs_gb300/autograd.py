"""Thin optional torch binding of srs_adjoint, for gradient checks.

    prob = AdjointProblem(mesh_base, params, seeds, linescan, n_steps, tick_every)
    theta = prob.theta0().requires_grad_()          # float64 [N_ADJ], ADJ_PARAMS order
    loss = LinescanLoss.apply(theta, prob)          # sum over realizations
    loss.backward()                                 # theta.grad from srs_adjoint

The loss is the line-scan dF/F0 loss of srs_adjoint summed over the
realizations, or with mean_trace=True the misfit of the realizations' mean
dF/F0 trace against one shared target (SRS_ADJ_MEAN_TRACE); the initial state
of every realization is fixed (taken from a reset at the problem's own
parameters), so the gradient is the one of the explicit-step map conditioned
on the recorded gating path.  `loss_fp64` evaluates the same loss with the
FP64 engine from the same start (common random numbers), for finite
differences; `mean_trace_fp64` gives the mean trace itself (e.g. a target
from perturbed parameters).
"""
import numpy as np
import torch

import srs_gb300 as srs


class AdjointProblem:
    def __init__(self, mesh_base, params, seeds, linescan, n_steps, tick_every, target=None,
                 checkpoint_every=0, cluster_size=0, mean_trace=False, engine=None):
        self.mesh_base = str(mesh_base)
        self.params = params.copy()
        self.seeds = [int(s) for s in seeds]
        self.linescan = dict(linescan)
        self.n_steps, self.tick_every = int(n_steps), int(tick_every)
        self.checkpoint_every, self.cluster_size = int(checkpoint_every), int(cluster_size)
        # FP32 engine of the adjoint: resident, or plain for meshes too large for it
        self.engine = srs.ENGINE_RESIDENT if engine is None else int(engine)
        sim = self._sim(self.params, srs.FP32, self.engine, reset=True)
        _, self.f0 = sim.linescan()
        self.start = [sim.get_state(r) for r in range(len(self.seeds))]
        n_ticks = self.n_steps // self.tick_every
        self.mean_trace = bool(mean_trace)
        shape = ((n_ticks, len(self.f0)) if self.mean_trace
                 else (len(self.seeds), n_ticks, len(self.f0)))
        self.target = (np.zeros(shape) if target is None else np.broadcast_to(target, shape).copy())

    def theta0(self):
        return torch.tensor([self.params.reals[srs.R[n]] for n in srs.ADJ_PARAMS], dtype=torch.float64)

    def params_at(self, theta):
        p = self.params.copy()
        for k, name in enumerate(srs.ADJ_PARAMS):
            p.reals[srs.R[name]] = float(theta[k])
        return p

    def _sim(self, p, precision, engine, reset=False):
        g = srs.Grid(p, self.mesh_base)
        sim = srs.Simulation(g, p, len(self.seeds), precision, engine, seeds=self.seeds,
                             cluster_size=self.cluster_size if engine == srs.ENGINE_RESIDENT else 0)
        sim.reset()
        if not reset:
            for r, st in enumerate(self.start):
                sim.set_state(r, st["states"], st["ryr"], st["lcc"], st["lccv"], st["residuals"])
        sim.linescan_setup(**self.linescan)
        return sim

    def loss_and_grad(self, theta):
        sim = self._sim(self.params_at(theta), srs.FP32, self.engine)
        loss, grad, _ = sim.adjoint(self.n_steps, self.tick_every, self.f0, self.target,
                                    checkpoint_every=self.checkpoint_every,
                                    flags=srs.ADJ_MEAN_TRACE if self.mean_trace else 0)
        return float(loss.sum()), grad.sum(axis=0)

    def _traces_fp64(self, theta):
        """dF/F0 of every realization at every tick [R][n_ticks][n_samples]
        from the FP64 engine (same start, same seeds)."""
        sim = self._sim(self.params_at(theta), srs.FP64, srs.ENGINE_PLAIN)
        n_ticks = self.n_steps // self.tick_every
        out = np.zeros((len(self.seeds), n_ticks, len(self.f0)))
        for k in range(n_ticks):
            sim.explicit_step(self.tick_every)
            F, _ = sim.linescan()
            out[:, k, :] = F / self.f0[None, :] - 1.0
        return out

    def mean_trace_fp64(self, theta):
        """The realizations' mean dF/F0 trace [n_ticks][n_samples] (FP64)."""
        return self._traces_fp64(theta).mean(axis=0)

    def loss_fp64(self, theta):
        """The same loss from the FP64 engine (same start, same seeds)."""
        tr = self._traces_fp64(theta)
        if self.mean_trace:
            e = tr.mean(axis=0) - self.target
        else:
            e = tr - self.target
        return 0.5 * float((e * e).sum())


class LinescanLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, problem):
        loss, grad = problem.loss_and_grad(theta.detach().cpu().numpy())
        ctx.save_for_backward(torch.from_numpy(grad).to(theta.device))
        return torch.tensor(loss, dtype=torch.float64, device=theta.device)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out * g, None

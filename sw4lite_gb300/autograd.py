"""torch.autograd view of the receiver misfit, for checks only.

`misfit(rho, mu, la, problem)` returns J(rho, mu, lambda) for a fixed shot
(sources, receivers, observed records, time step count) and its backward pass
calls the library's discrete adjoint (sw4g_ew_gradient).  It exists so the
gradient can be checked with torch tooling against finite differences and an
FP64 reference gradient; the time loop and the adjoint themselves run in the
library's CUDA kernels, never in torch.
"""
from dataclasses import dataclass, field

import torch

import sw4lite_gb300 as sg


@dataclass
class Shot:
    grid: object                     # GridDesc (Dirichlet / supergrid sides)
    dt: float
    nsteps: int
    checkpoint_every: int
    receivers: list                  # 1-based (i, j, k) per receiver
    observed: torch.Tensor           # (nsteps + 1) x 3*len(receivers), float64
    sources: list = field(default_factory=list)


def _ew(rho, mu, la, shot: Shot):
    ew = sg.EW(shot.grid)
    ew.set_material(rho.contiguous(), mu.contiguous(), la.contiguous())
    for s in shot.sources:
        ew.add_source(s)
    ew.set_time_step(shot.dt, 0.0)
    ew.set_receivers(shot.receivers, [sg.REC_DISPLACEMENT] * len(shot.receivers), shot.nsteps + 1)
    return ew


class _Misfit(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho, mu, la, shot):
        ew = _ew(rho, mu, la, shot)
        g = [torch.zeros_like(rho) for _ in range(3)]
        J = ew.gradient(shot.nsteps, shot.checkpoint_every, shot.observed.contiguous(), *g)
        torch.cuda.synchronize()
        ew.close()
        ctx.save_for_backward(*g)
        return torch.tensor(J, dtype=torch.float64, device=rho.device)

    @staticmethod
    def backward(ctx, gJ):
        g = ctx.saved_tensors
        return g[0] * gJ, g[1] * gJ, g[2] * gJ, None


def misfit(rho, mu, la, shot: Shot) -> torch.Tensor:
    """J = 1/2 sum_n sum_r |u^n(x_r) - observed^n_r|^2 as a differentiable scalar."""
    return _Misfit.apply(rho, mu, la, shot)


def forward_misfit(rho, mu, la, shot: Shot) -> float:
    """J by a plain forward run (no adjoint), for finite differences."""
    ew = _ew(rho, mu, la, shot)
    ew.step(shot.nsteps, sg.MODE_FUSED)
    rec = torch.zeros_like(shot.observed)
    ew.records(rec)
    torch.cuda.synchronize()
    ew.close()
    return 0.5 * float(((rec - shot.observed) ** 2).sum())

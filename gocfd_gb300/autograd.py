"""torch.autograd.Function wrappers over the C ABI, used for gradchecks.

Forward goes through gcfd_rhs / gcfd_record_steps, backward through
gcfd_rhs_vjp / gcfd_step_vjp.  Tensors are float64 4 x Np x K arrays (the
solver's global state layout) and move through host memory; the solver is an
`Euler` on the FP64 path.
"""
import numpy as np
import torch


def _np(t: torch.Tensor) -> np.ndarray:
    return np.ascontiguousarray(t.detach().cpu().numpy().astype(np.float64))


class RHS(torch.autograd.Function):
    """RHS(Q) at a fixed solver time."""

    @staticmethod
    def forward(ctx, Q, solver, time=0.0):
        ctx.solver, ctx.time = solver, float(time)
        ctx.save_for_backward(Q)
        return torch.from_numpy(solver.rhs_global(_np(Q), ctx.time)).to(Q.device)

    @staticmethod
    def backward(ctx, gout):
        (Q,) = ctx.saved_tensors
        qb, _, _ = ctx.solver.rhs_vjp_global(_np(Q), _np(gout), ctx.time)
        return torch.from_numpy(qb).to(gout.device), None, None


class Steps(torch.autograd.Function):
    """nsteps SSP(5,4) steps from (Q0, t0).  Backward records the same window
    again (the forward map is deterministic) and runs its adjoint, so other
    forward calls in between (a gradcheck's perturbations) do not matter."""

    @staticmethod
    def forward(ctx, Q0, solver, nsteps, t0=0.0, checkpoint_every=1):
        ctx.solver, ctx.nsteps, ctx.t0, ctx.every = solver, int(nsteps), float(t0), int(checkpoint_every)
        ctx.save_for_backward(Q0)
        Steps._record(solver, _np(Q0), ctx.t0, ctx.nsteps, ctx.every)
        return torch.from_numpy(solver.get_global_state()).to(Q0.device)

    @staticmethod
    def _record(solver, q0, t0, nsteps, every):
        solver.set_global_state(q0)
        solver.time = t0
        solver.record(nsteps, every)

    @staticmethod
    def backward(ctx, gout):
        (Q0,) = ctx.saved_tensors
        Steps._record(ctx.solver, _np(Q0), ctx.t0, ctx.nsteps, ctx.every)
        qb, _, _ = ctx.solver.step_vjp(_np(gout))
        return torch.from_numpy(qb).to(gout.device), None, None, None, None

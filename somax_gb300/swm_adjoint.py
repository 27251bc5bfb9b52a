"""Reverse-mode differentiation of the multilayer shallow-water model over the hand-written
VJPs of libqgcore (what the reference takes with JAX autodiff through ``vector_field`` and
``integrate``: ``tests/models/test_swm_multilayer.py:239-252``).

* :class:`RHS`       -> ``qg_swm_rhs_vjp`` (the state's and the parameters' cotangents)
* :class:`Integrate` -> the state kept every ``checkpoint_every`` steps; the backward sweep runs
  each segment's adjoint in one C-ABI call (``qg_swm_segment_vjp``: the segment's states
  recomputed, then ``qg_swm_step_vjp``'s launches for every step in reverse, replayed as one
  graph), or, for steppers without it (the reparameterised model), one ``step_vjp`` per
  recomputed step; with ``apply_bc`` the boundary conditions applied to the initial state are
  transposed last (``qg_swm_bc_vjp``).

A step is ``y1 = y0 + dt sum_i b_i k_i``, ``k_i = F(B(y0 + dt sum_j a_ij k_j))`` with B the
boundary rules; its adjoint for the cotangent ``g`` of ``y1`` is ``k_bar_i = dt b_i g``, then
for the stages in reverse ``Y_bar_i = B^T F'(B Y_i)^T k_bar_i``, ``y0_bar += Y_bar_i``,
``k_bar_j += dt a_ij Y_bar_i``.  The parameters are (nu, kappa, tau0).
"""

from __future__ import annotations

import torch


def _f32(t: torch.Tensor) -> torch.Tensor:
    return t.detach().to(torch.float32).contiguous()


class RHS(torch.autograd.Function):
    """``dy = plan.rhs(y, params, apply_bc)`` with its VJP from ``qg_swm_rhs_vjp``."""

    @staticmethod
    def forward(ctx, y, params, plan, apply_bc):
        yc, pc = _f32(y), _f32(params)
        ctx.save_for_backward(yc, pc)
        ctx.plan, ctx.apply_bc = plan, bool(apply_bc)
        ctx.dtypes = (y.dtype, params.dtype)
        return plan.rhs(yc, pc, apply_bc=apply_bc)

    @staticmethod
    def backward(ctx, g):
        y, p = ctx.saved_tensors
        yb, pb = ctx.plan.rhs_vjp(y, p, _f32(g), ctx.apply_bc)
        return yb.to(ctx.dtypes[0]), pb.to(ctx.dtypes[1]), None, None


class Integrate(torch.autograd.Function):
    """``n_steps`` steps of ``scheme`` from ``y0`` (boundary rules applied first with
    ``apply_bc``), differentiable in ``y0`` and ``params`` by checkpointed recomputation."""

    @staticmethod
    def forward(ctx, y0, params, plan, dt, n_steps, scheme, apply_bc, checkpoint_every):
        every = max(1, int(checkpoint_every))
        p = _f32(params)
        y = _f32(y0).clone()
        if apply_bc:
            plan.apply_bc(y)
        cps = [y.clone()]
        done = 0
        while done < n_steps:
            k = min(every, n_steps - done)
            plan.step(y, p, dt, k, scheme, False)
            done += k
            if done < n_steps:
                cps.append(y.clone())
        ctx.save_for_backward(p, *cps)
        ctx.plan, ctx.dt, ctx.n, ctx.scheme = plan, float(dt), int(n_steps), scheme
        ctx.apply_bc, ctx.every = bool(apply_bc), every
        ctx.dtypes = (y0.dtype, params.dtype)
        return y

    @staticmethod
    def backward(ctx, g):
        p, *cps = ctx.saved_tensors
        plan, dt, scheme, every = ctx.plan, ctx.dt, ctx.scheme, ctx.every
        gy = _f32(g).clone()
        gp = torch.zeros_like(p)
        for s in reversed(range(len(cps))):
            k = min(every, ctx.n - s * every)
            if k <= 0:
                continue
            if hasattr(plan, "segment_vjp"):  # the whole segment's reverse sweep in one call
                gy, dp = plan.segment_vjp(cps[s], p, dt, k, scheme, gy)
                gp += dp
                continue
            ys = [cps[s]]
            for _ in range(k - 1):
                z = ys[-1].clone()
                plan.step(z, p, dt, 1, scheme, False)
                ys.append(z)
            for y in reversed(ys):
                gy, dp = plan.step_vjp(y, p, dt, scheme, gy)
                gp += dp
        if ctx.apply_bc:
            plan.bc_vjp(gy)
        return gy.view_as(g).to(ctx.dtypes[0]), gp.to(ctx.dtypes[1]), None, None, None, None, None, None


def rhs(plan, y, params, apply_bc=False):
    return RHS.apply(y, params, plan, apply_bc)


def integrate(plan, y0, params, dt, n_steps, scheme="tsit5", apply_bc=True, checkpoint_every=10):
    return Integrate.apply(y0, params, plan, dt, n_steps, scheme, apply_bc, checkpoint_every)

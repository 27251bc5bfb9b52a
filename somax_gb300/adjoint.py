"""Reverse-mode differentiation of the QG path over the hand-written VJPs of libqgcore.

The reference differentiates ``vector_field``, ``_invert_pv`` and ``integrate`` with JAX
autodiff through diffrax (``tests/models/test_qg_baroclinic.py:293-312``; diffrax's default
adjoint recomputes the forward from checkpoints).  Here the same derivatives come from
``torch.autograd.Function`` classes over the C ABI:

* :class:`RHS`       -> ``qg_rhs_vjp``    (q_bar and the parameter cotangents)
* :class:`Invert`    -> ``qg_invert_vjp`` (one adjoint DST-I solve; the solve is self-adjoint)
* :class:`Integrate` -> the adjoint of the explicit Runge-Kutta step (``qg_step_vjp``: the
  step's stage inputs recomputed with the fused right-hand side and the stages reversed with
  ``qg_rhs_vjp``'s kernels and fused linear-combination kernels, in one C-ABI call), with the
  state kept every ``checkpoint_every`` steps and each segment recomputed on the GPU during
  the backward sweep (memory: one state per checkpoint plus one segment).

A step is ``y1 = y0 + dt * sum_i b_i k_i``, ``k_i = F(B(y0 + dt * sum_j a_ij k_j))`` with B
the ring zeroing of the stage input (``core/model.py:47-49``); its adjoint for the cotangent
``g`` of ``y1`` is ``k_bar_i = dt b_i g``, then for the stages in reverse
``Y_bar_i = F_vjp(Y_i; k_bar_i)``, ``y0_bar += Y_bar_i``, ``k_bar_j += dt a_ij Y_bar_i``.
The fused ``qg_step`` kernels produce the same ring (``y0 + dt * wind``) as this form, so the
forward (every scheme) runs fused and only the recomputed stages of one step at a time run
unfused.  ``step_vjp_torch`` is the same algebra written with torch operations around
``qg_rhs`` / ``qg_rhs_vjp``; the tests compare the two.
"""

from __future__ import annotations

import torch

from .tableaus import rk_tableau


def _zero_ring(q: torch.Tensor) -> torch.Tensor:
    out = q.clone()
    out[..., 0, :] = 0
    out[..., -1, :] = 0
    out[..., :, 0] = 0
    out[..., :, -1] = 0
    return out


def _f32(t: torch.Tensor) -> torch.Tensor:
    return t.detach().to(torch.float32).contiguous()


class RHS(torch.autograd.Function):
    """``dq = plan.rhs(q, params, apply_bc)`` with its VJP from ``qg_rhs_vjp``."""

    @staticmethod
    def forward(ctx, q, params, plan, apply_bc):
        qc, pc = _f32(q), _f32(params)
        ctx.save_for_backward(qc, pc)
        ctx.plan, ctx.apply_bc, ctx.pshape = plan, bool(apply_bc), params.shape
        ctx.dtypes = (q.dtype, params.dtype)
        return plan.rhs(qc, pc, apply_bc=apply_bc)

    @staticmethod
    def backward(ctx, g):
        q, p = ctx.saved_tensors
        want_p = ctx.needs_input_grad[1]
        qb, pb = ctx.plan.rhs_vjp(q, p, _f32(g), ctx.apply_bc, want_params=want_p)
        qb = qb.view_as(q).to(ctx.dtypes[0])
        return qb, (pb.view(ctx.pshape).to(ctx.dtypes[1]) if want_p else None), None, None


class Invert(torch.autograd.Function):
    """``psi = plan.invert(q)`` with its VJP from ``qg_invert_vjp``."""

    @staticmethod
    def forward(ctx, q, plan):
        ctx.plan, ctx.dtype = plan, q.dtype
        return plan.invert(_f32(q))

    @staticmethod
    def backward(ctx, g):
        return ctx.plan.invert_vjp(_f32(g)).to(ctx.dtype), None


def _advance(plan, q, p, dt, n, scheme):
    """q <- n fused steps of ``scheme`` (in place; the ring of q is taken as it is)."""
    if n > 0:
        plan.step(q, p, dt, n, scheme, apply_bc=False)
    return q


def step_vjp(plan, y0, p, dt, scheme, g):
    """(y0_bar, params_bar) of one step from ``y0`` for the cotangent ``g`` of its result."""
    return plan.step_vjp(y0, p, dt, scheme, g)


def step_vjp_torch(plan, y0, p, dt, scheme, g):
    """``step_vjp`` with the stage algebra as torch operations around ``qg_rhs`` /
    ``qg_rhs_vjp`` (the reference form of the fused call)."""
    a, b = rk_tableau(scheme)
    s_n = len(b)
    # stage inputs of the step (recomputed)
    Y, ks = [], []
    for s in range(s_n):
        ys = y0
        if s:
            ys = y0.clone()
            for j, aij in enumerate(a[s]):
                if aij:
                    ys.add_(ks[j], alpha=dt * aij)
        Y.append(ys)
        if s < s_n - 1:
            ks.append(plan.rhs(ys, p, apply_bc=True))
    kbar = [g * (dt * bi) for bi in b]
    y0_bar = g.clone()
    p_bar = torch.zeros_like(p)
    for s in reversed(range(s_n)):
        Yb, pb = plan.rhs_vjp(Y[s], p, kbar[s].contiguous(), apply_bc=True)
        p_bar += pb
        y0_bar += Yb
        for j, aij in enumerate(a[s]):
            if aij:
                kbar[j].add_(Yb, alpha=dt * aij)
    return y0_bar, p_bar


class Integrate(torch.autograd.Function):
    """``n_steps`` steps of ``scheme`` from ``q0`` (ring zeroed first with ``apply_bc``),
    differentiable in ``q0`` and ``params`` by checkpointed recomputation."""

    @staticmethod
    def forward(ctx, q0, params, plan, dt, n_steps, scheme, apply_bc, checkpoint_every):
        every = max(1, int(checkpoint_every))
        p = _f32(params)
        q = _f32(q0).clone()
        if apply_bc:
            q = _zero_ring(q)
        cps = [q.clone()]
        done = 0
        while done < n_steps:
            k = min(every, n_steps - done)
            _advance(plan, q, p, dt, k, scheme)
            done += k
            if done < n_steps:
                cps.append(q.clone())
        ctx.save_for_backward(p, *cps)
        ctx.plan, ctx.dt, ctx.n, ctx.scheme = plan, float(dt), int(n_steps), scheme
        ctx.apply_bc, ctx.every, ctx.pshape = bool(apply_bc), every, params.shape
        ctx.dtypes = (q0.dtype, params.dtype)
        return q

    @staticmethod
    def backward(ctx, g):
        p, *cps = ctx.saved_tensors
        plan, dt, scheme, every = ctx.plan, ctx.dt, ctx.scheme, ctx.every
        gq = _f32(g).clone()
        gp = torch.zeros_like(p)
        for s in reversed(range(len(cps))):
            k = min(every, ctx.n - s * every)
            if k <= 0:
                continue
            ys = [cps[s]]
            for _ in range(k - 1):
                ys.append(_advance(plan, ys[-1].clone(), p, dt, 1, scheme))
            for y in reversed(ys):
                gq, dp = step_vjp(plan, y, p, dt, scheme, gq)
                gp += dp
        if ctx.apply_bc:
            gq = _zero_ring(gq)
        gq = gq.view_as(g).to(ctx.dtypes[0])
        return gq, gp.view(ctx.pshape).to(ctx.dtypes[1]), None, None, None, None, None, None


def rhs(plan, q, params, apply_bc=False):
    return RHS.apply(q, params, plan, apply_bc)


def invert(plan, q):
    return Invert.apply(q, plan)


def integrate(plan, q0, params, dt, n_steps, scheme="ssprk3", apply_bc=True, checkpoint_every=10):
    return Integrate.apply(q0, params, plan, dt, n_steps, scheme, apply_bc, checkpoint_every)

"""Differentiable substeps and checkpointed rollouts over the GB300 solver.

The contract is the reference's differentiable branch (``differentiation.py``):
the system matrix is a fixed input to each recorded substep (no dA/dq), every
solve starts from zero and runs to a tight tolerance (the reference uses tol
1e-8 with the solver's iteration budget), and the gradient is that of the
converged linear solve, not of truncated CG.  One substep is

    rhs = h*sum f(q, v, a, s) + h*ext - sum_j A_ij (v_j - v_i) + spring damping
    dv  = (PAP + I - P)^-1 P rhs,   v' = v + dv,   q' = q + h v'

with fixed nodes restored before the forces and after integration.  Its VJP
(``_Substep.backward``) runs, all on the GPU through the C ABI:

    vt = v'_bar + h q'_bar                    (outputs at fixed nodes carry no gradient)
    rhs_bar = (PAP + I - P)^-1 P vt           (fem_solve: A is symmetric)
    v_bar = vt + predictor VJP(rhs_bar)       (fem_predictor_vjp)
    (q_bar, v_bar, a_bar, s_bar) += force VJP(h rhs_bar)   (fem_force_vjp)
    ext_bar = h rhs_bar

Beyond the reference: fixed nodes are allowed (projected solve), and a
per-element shear scale ``s`` (``mu_scale``) is a differentiable control next
to the reference's additive activations.  ``checkpointed_gradient`` keeps
state checkpoints every K substeps and recomputes each segment in reverse,
the frame-checkpoint schedule of the reference's bear training
(``examples/diffsim/_bear_training.py:239-310``).  A segment may begin with a
tangent refresh (the step callback sees the substep index): each segment's
backward pass follows its recomputation directly, so it uses the matrix its
forward pass used; a backward pass after the matrix changed raises, as in the
reference (``differentiation.py:375-376``).
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from .solver import SolverFEM


class DifferentiableSolver:
    """Differentiable view of a ``SolverFEM`` (its assembled matrix is frozen while recording)."""

    def __init__(self, solver: SolverFEM, tolerance: float = 1.0e-8, maxiter: int | None = None):
        self.solver = solver
        self.model = solver.model
        self.device = solver.device
        self.tolerance = float(tolerance)
        self.maxiter = int(maxiter if maxiter is not None else solver.linear_solver_maxiter)
        self.lib = _lib.load()
        P = self.model.particle_count
        self.fixed = torch.zeros(P, dtype=torch.bool, device=self.device)
        if len(solver.fixed_particle_indices):
            self.fixed[torch.as_tensor(solver.fixed_particle_indices, device=self.device, dtype=torch.long)] = True
        self._scale = None
        self.last_iterations = []

    def _stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def set_mu_scale(self, scale: torch.Tensor | None) -> None:
        """Bind the per-tet shear scale read by the force kernels (None clears it)."""
        self._scale = None if scale is None else scale.detach().contiguous()
        ptr = None if self._scale is None else self._scale.data_ptr()
        _lib.check(self.lib.fem_set_mu_scale(self.solver._handle, ptr))

    def step(self, q, v, dt, *, external_forces=None, activations=None, mu_scale=None):
        """One differentiable substep: returns (q', v') tracked by autograd.

        The matrix is assembled for ``solver.dt`` and held fixed, so ``dt`` must
        equal it (differentiation.py:274-276).
        """
        if float(dt) != self.solver.dt:
            raise ValueError("Differentiable dt must match the fixed matrix assembly timestep")
        return _Substep.apply(self, q, v, float(dt), external_forces, activations, mu_scale)

    # -- primitives (no autograd) -------------------------------------------
    def forward_step(self, q, v, dt, ext, act, scale):
        s = self.solver
        P = self.model.particle_count
        q_in = q.detach().contiguous().clone()
        v_in = v.detach().contiguous().clone()
        q_out = torch.empty_like(q_in)
        v_out = torch.empty_like(v_in)
        f_ws = torch.empty_like(q_in)
        if scale is not None:
            self.set_mu_scale(scale)
        prev_tol, prev_it = s.linear_solver_tolerance, s.linear_solver_maxiter
        s.linear_solver_tolerance = self.tolerance
        s.linear_solver_maxiter = self.maxiter
        try:
            s.velocity_increment.zero_()  # every checked solve starts from zero (differentiation.py:199-205)
            ext_c = None if ext is None else ext.detach().contiguous()
            act_c = None if act is None else act.detach().contiguous()
            _lib.check(self.lib.fem_step(s._handle, q_in.data_ptr(), v_in.data_ptr(), q_out.data_ptr(),
                                         v_out.data_ptr(), f_ws.data_ptr(),
                                         None if ext_c is None else ext_c.data_ptr(),
                                         None if act_c is None else act_c.data_ptr(),
                                         self.model.gravity.data_ptr(), dt, self._stream()), "differentiable step")
        finally:
            s.linear_solver_tolerance = prev_tol
            s.linear_solver_maxiter = prev_it
        assert q_out.shape == (P, 3)
        return q_in, v_in, q_out, v_out

    def solve(self, rhs: torch.Tensor) -> torch.Tensor:
        x = torch.empty_like(rhs)
        _lib.check(self.lib.fem_solve(self.solver._handle, rhs.contiguous().data_ptr(), x.data_ptr(), self.tolerance,
                                      self.maxiter, self._stream()), "adjoint solve")
        return x


class _Substep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, diff, q, v, dt, ext, act, scale):
        q_in, v_in, q_out, v_out = diff.forward_step(q, v, dt, ext, act, scale)
        ctx.diff = diff
        ctx.dt = dt
        ctx.revision = diff.solver._revision  # the matrix this substep was recorded with
        ctx.has = (ext is not None, act is not None, scale is not None)
        ctx.save_for_backward(q_in, v_in, act if act is not None else q_in.new_empty(0),
                              scale if scale is not None else q_in.new_empty(0))
        return q_out, v_out

    @staticmethod
    def backward(ctx, q_out_bar, v_out_bar):
        diff: DifferentiableSolver = ctx.diff
        if diff.solver._revision != ctx.revision:  # differentiation.py:375-376
            raise RuntimeError("FEM model/matrix changed after recording; rerun the forward tape before backward")
        q_in, v_in, act, scale = ctx.saved_tensors
        has_ext, has_act, has_scale = ctx.has
        dt = ctx.dt
        lib = diff.lib
        handle = diff.solver._handle
        stream = diff._stream()
        qb = torch.zeros_like(q_in) if q_out_bar is None else q_out_bar.contiguous().clone()
        vb = torch.zeros_like(v_in) if v_out_bar is None else v_out_bar.contiguous().clone()
        qb[diff.fixed] = 0.0  # fixed outputs are overwritten by the restore
        vb[diff.fixed] = 0.0
        vt = vb + dt * qb
        rhs_bar = diff.solve(vt)
        v_bar = vt.clone()
        _lib.check(lib.fem_predictor_vjp(handle, rhs_bar.data_ptr(), dt, v_bar.data_ptr(), stream))
        q_bar = qb
        g = (dt * rhs_bar).contiguous()
        T = diff.model.tet_count
        act_bar = torch.zeros(T, dtype=torch.float32, device=q_in.device) if has_act else None
        scale_bar = torch.zeros(T, dtype=torch.float32, device=q_in.device) if has_scale else None
        if has_scale:
            diff.set_mu_scale(scale)
        _lib.check(lib.fem_force_vjp(handle, q_in.data_ptr(), v_in.data_ptr(),
                                     act.data_ptr() if has_act else None, diff.model.gravity.data_ptr(), g.data_ptr(),
                                     q_bar.data_ptr(), v_bar.data_ptr(),
                                     act_bar.data_ptr() if has_act else None,
                                     scale_bar.data_ptr() if has_scale else None, stream), "force VJP")
        q_bar[diff.fixed] = 0.0  # fixed inputs are overwritten by the restore
        v_bar[diff.fixed] = 0.0
        ext_bar = g if has_ext else None
        return None, q_bar, v_bar, None, ext_bar, act_bar, scale_bar


def checkpointed_gradient(step, q0, v0, steps: int, every: int, loss_fn, params=()):
    """Loss and gradients of a ``steps``-substep rollout with checkpoints every ``every`` substeps.

    ``step(q, v, k) -> (q, v)`` is one differentiable substep (it may read the
    leaf tensors in ``params``); ``loss_fn(q, v)`` maps the final state to a
    scalar.  The forward pass stores only the checkpoint states; the backward
    pass recomputes each segment with autograd, newest first, and carries the
    state adjoint into the previous segment.  Returns (loss, dL/dq0, dL/dv0,
    [dL/dp for p in params]).
    """
    ckpts = []
    with torch.no_grad():
        q, v = q0.detach(), v0.detach()
        for k in range(steps):
            if k % every == 0:
                ckpts.append((k, q.clone(), v.clone()))
            q, v = step(q, v, k)
    qf = q.detach().requires_grad_(True)
    vf = v.detach().requires_grad_(True)
    loss = loss_fn(qf, vf)
    qb, vb = torch.autograd.grad(loss, (qf, vf), allow_unused=True)
    qb = torch.zeros_like(qf) if qb is None else qb
    vb = torch.zeros_like(vf) if vb is None else vb
    grads = [torch.zeros_like(p) for p in params]
    for start, qc, vc in reversed(ckpts):
        end = min(start + every, steps)
        qs = qc.detach().requires_grad_(True)
        vs = vc.detach().requires_grad_(True)
        q, v = qs, vs
        for k in range(start, end):
            q, v = step(q, v, k)
        inputs = (qs, vs, *params)
        out = torch.autograd.grad((q, v), inputs, grad_outputs=(qb, vb), allow_unused=True)
        qb = torch.zeros_like(qs) if out[0] is None else out[0]
        vb = torch.zeros_like(vs) if out[1] is None else out[1]
        for i, gp in enumerate(out[2:]):
            if gp is not None:
                grads[i] += gp
    return loss.detach(), qb, vb, grads

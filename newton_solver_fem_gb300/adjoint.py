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
        self.after_backward_solve = None  # hook run after every adjoint solve (SolverFEM's residual check)

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
        if diff.after_backward_solve is not None:
            diff.after_backward_solve()
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


class DeviceRollout:
    """Checkpointed differentiable rollouts run segment by segment on the device.

    The forward pass and the reverse pass are whole segments of substeps enqueued
    by the library (``fem_rollout_segment``, ``fem_adjoint_segment``) on a
    stream, with no per-substep Python and no host synchronisation; full-length
    segments are replayed from captured CUDA graphs.  The contract is
    ``_Substep``'s: the matrix is held fixed within a segment, every forward
    solve starts from zero unless ``warm_start``, and the gradient is that of the
    linear solves.

    Memory: with ``store_all`` every substep's state is kept (steps + 1 states,
    no recomputation); otherwise only the checkpoint states every ``every``
    substeps are kept and each segment is recomputed once in the reverse pass
    (the reference's frame-checkpoint schedule, ``examples/diffsim/_bear_training.py:239-310``).
    ``refresh`` assembles the tangent at the start of every segment (a segment is
    then one frame of a frame loop), in the forward pass and again before the
    segment's reverse pass.

    ``overlap``: a ``DifferentiableSolver`` over a second handle with the same
    model and the same assembled matrix.  The reverse pass then recomputes
    segment i-1 on that handle, on its own stream, while segment i's reverse
    pass runs on the first (two state buffers alternate).  A small mesh leaves
    most SMs idle, so the recomputation comes almost for free; the two
    cooperative PCG grids together must fit on the device, which is checked.
    """

    def __init__(self, diff: DifferentiableSolver, steps: int, every: int, *, refresh: bool = False,
                 warm_start: bool = False, warm_adjoint: bool = False, store_all: bool = False, graphs: bool = True,
                 overlap: DifferentiableSolver | None = None):
        if steps < 1 or every < 1:
            raise ValueError("steps and every must be positive")
        self.diff, self.steps, self.every = diff, int(steps), int(every)
        self.refresh, self.warm_start, self.warm_adjoint = bool(refresh), bool(warm_start), bool(warm_adjoint)
        self.store_all, self.graphs = bool(store_all), bool(graphs) and not store_all
        self.overlap = None if store_all else overlap
        if self.overlap is not None:
            if self.overlap.solver is diff.solver or self.overlap.model.particle_count != diff.model.particle_count:
                raise ValueError("overlap needs a second solver over the same model")
            if (self.overlap.tolerance, self.overlap.maxiter, self.overlap.solver.dt) != \
                    (diff.tolerance, diff.maxiter, diff.solver.dt):
                raise ValueError("overlap needs the same tolerance, iteration cap and timestep")
            if not self.overlap_fits():
                self.overlap = None  # the two PCG grids would not be co-resident: recompute in line
        s = diff.solver
        P, dev = s.model.particle_count, s.device
        self.P, self.device = P, dev
        self.bounds = [(k, min(k + self.every, self.steps)) for k in range(0, self.steps, self.every)]
        nbuf = 2 if self.overlap is not None else 1
        n_states = self.steps + 1 if self.store_all else self.every + 1
        self.q_states = [torch.zeros((n_states, P, 3), dtype=torch.float32, device=dev) for _ in range(nbuf)]
        self.v_states = [torch.zeros_like(t) for t in self.q_states]
        self.dv_in = [torch.zeros((P, 3), dtype=torch.float32, device=dev) for _ in range(nbuf)]
        nck = len(self.bounds) + 1
        self.ck_q = None if self.store_all else torch.zeros((nck, P, 3), dtype=torch.float32, device=dev)
        self.ck_v = None if self.store_all else torch.zeros_like(self.ck_q)
        self.ck_dv = torch.zeros((nck, P, 3), dtype=torch.float32, device=dev) if self.warm_start else None
        self.q_bar = torch.zeros((P, 3), dtype=torch.float32, device=dev)
        self.v_bar = torch.zeros_like(self.q_bar)
        self.adj_start = torch.zeros_like(self.q_bar) if self.warm_adjoint else None
        self._graphs = {}
        self._primed = False

    def overlap_fits(self) -> bool:
        """Both handles' cooperative PCG grids fit on the device side by side (one CTA per SM each at most)."""
        lib = self.diff.lib
        total = 0
        for d in (self.diff, self.overlap):
            v = ctypes.c_int64()
            _lib.check(lib.fem_get_tuning(d.solver._handle, _lib.FEM_TUNE_GRID, ctypes.byref(v)))
            total += int(v.value)
        sms = torch.cuda.get_device_properties(self.diff.device).multi_processor_count
        return total <= sms

    # -- native calls ---------------------------------------------------------
    def _rollout(self, d, q0, v0, dv0, n, q_states, v_states, dv_out, ext, act):
        s = d.solver
        _lib.check(d.lib.fem_rollout_segment(
            s._handle, q0.data_ptr(), v0.data_ptr(), None if dv0 is None else dv0.data_ptr(), n,
            None if ext is None else ext.data_ptr(), None if act is None else act.data_ptr(),
            s.model.gravity.data_ptr(), s.dt, d.tolerance, d.maxiter, int(self.warm_start), int(self.refresh),
            q_states.data_ptr(), v_states.data_ptr(), None if dv_out is None else dv_out.data_ptr(), d._stream()),
            "rollout segment")

    def _adjoint(self, q_states, v_states, n, refresh, ext, act, acc):
        d, s = self.diff, self.diff.solver
        ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        _lib.check(d.lib.fem_adjoint_segment(
            s._handle, q_states.data_ptr(), v_states.data_ptr(), n, ptr(ext), ptr(act), s.model.gravity.data_ptr(),
            s.dt, d.tolerance, d.maxiter, int(refresh), ptr(self.adj_start), self.q_bar.data_ptr(),
            self.v_bar.data_ptr(), ptr(acc["ext"]), ptr(acc["act"]), ptr(acc["scale"]), ptr(acc["tet_mat"]),
            ptr(acc["hex_mat"]), d._stream()), "adjoint segment")

    def _prime(self, ext, act, acc):
        """First calls allocate the handles' rollout and adjoint scratch: make them outside any capture."""
        if self._primed:
            return
        for d in (self.diff, self.overlap):
            if d is None:
                continue
            if d is self.overlap and self.diff._scale is not None:
                d.set_mu_scale(self.diff._scale)
            _lib.check(d.lib.fem_rollout_segment(
                d.solver._handle, self.q_states[0].data_ptr(), self.v_states[0].data_ptr(), None, 0, None, None, None,
                d.solver.dt, d.tolerance, d.maxiter, 0, 0, self.q_states[0].data_ptr(), self.v_states[0].data_ptr(),
                None, d._stream()), "rollout segment")
        self._primed = True

    def _replay(self, key, stream, build):
        """Replay the graph `key` on `stream`, capturing it from `build()` on first use.  A graph holds
        the pointers it was captured with, so the key carries the control and shear-scale pointers."""
        key = key + (None if self.diff._scale is None else self.diff._scale.data_ptr(),)
        g = self._graphs.get(key)
        if g is None:
            cap = torch.cuda.Stream(self.device)
            cap.wait_stream(stream)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(cap):
                with torch.cuda.graph(g, stream=cap):
                    build()
            stream.wait_stream(cap)
            self._graphs[key] = g
        with torch.cuda.stream(stream):
            g.replay()

    @staticmethod
    def _ptrs(*tensors):
        return tuple(None if t is None else t.data_ptr() for t in tensors)

    # -- passes ----------------------------------------------------------------
    def forward(self, q0, v0, *, external_forces=None, activations=None):
        """Roll out from (q0, v0); returns the final state (q, v) (copies)."""
        ext = None if external_forces is None else external_forces.detach().contiguous()
        act = None if activations is None else activations.detach().contiguous()
        q0, v0 = q0.detach().contiguous(), v0.detach().contiguous()
        self._prime(ext, act, None)
        d = self.diff
        if self.ck_dv is not None:
            self.ck_dv[0].zero_()
        qs, vs = self.q_states[0], self.v_states[0]
        if self.store_all:
            qs[0].copy_(q0)
            vs[0].copy_(v0)
            for i, (a, b) in enumerate(self.bounds):
                dv0 = None if self.ck_dv is None else self.ck_dv[i]
                dv1 = None if self.ck_dv is None else self.ck_dv[i + 1]
                self._rollout(d, qs[a], vs[a], dv0, b - a, qs[a:], vs[a:], dv1, ext, act)
            return qs[self.steps].clone(), vs[self.steps].clone()
        self.ck_q[0].copy_(q0)
        self.ck_v[0].copy_(v0)
        stream = torch.cuda.current_stream(self.device)
        for i, (a, b) in enumerate(self.bounds):
            n = b - a
            qs[0].copy_(self.ck_q[i])
            vs[0].copy_(self.ck_v[i])
            if self.ck_dv is not None:
                self.dv_in[0].copy_(self.ck_dv[i])
            dv_in = None if self.ck_dv is None else self.dv_in[0]
            if self.graphs and n == self.every:
                self._replay(("fwd", self._ptrs(ext, act)), stream,
                             lambda: self._rollout(d, qs[0], vs[0], dv_in, n, qs, vs, dv_in, ext, act))
            else:
                self._rollout(d, qs[0], vs[0], dv_in, n, qs, vs, dv_in, ext, act)
            self.ck_q[i + 1].copy_(qs[n])
            self.ck_v[i + 1].copy_(vs[n])
            if self.ck_dv is not None:
                self.ck_dv[i + 1].copy_(self.dv_in[0])
        return self.ck_q[-1].clone(), self.ck_v[-1].clone()

    def _recompute(self, i, buf, stream, ext, act):
        """Segment i's states into buffer `buf`, on the recomputing handle and `stream`."""
        a, b = self.bounds[i]
        n = b - a
        d = self.overlap if self.overlap is not None else self.diff
        qs, vs, dv = self.q_states[buf], self.v_states[buf], self.dv_in[buf]
        with torch.cuda.stream(stream):
            qs[0].copy_(self.ck_q[i])
            vs[0].copy_(self.ck_v[i])
            if self.ck_dv is not None:
                dv.copy_(self.ck_dv[i])
        dv_in = None if self.ck_dv is None else dv
        if self.graphs and n == self.every:
            self._replay(("rec", buf, self._ptrs(ext, act)), stream,
                         lambda: self._rollout(d, qs[0], vs[0], dv_in, n, qs, vs, None, ext, act))
        else:
            with torch.cuda.stream(stream):
                self._rollout(d, qs[0], vs[0], dv_in, n, qs, vs, None, ext, act)

    def _reverse(self, i, buf, stream, ext, act, acc, key):
        """Segment i's reverse pass over buffer `buf` on the first handle and `stream`."""
        a, b = self.bounds[i]
        n = b - a
        qs, vs = self.q_states[buf], self.v_states[buf]
        # the matrix: refreshed by an in-line recomputation on this handle, else refreshed here
        refresh = self.refresh and self.overlap is not None
        if self.graphs and n == self.every:
            self._replay(("adj", buf, key), stream, lambda: self._adjoint(qs, vs, n, refresh, ext, act, acc))
        else:
            with torch.cuda.stream(stream):
                self._adjoint(qs, vs, n, refresh, ext, act, acc)

    def backward(self, q_bar, v_bar, *, external_forces=None, activations=None, mu_scale=None, materials=False):
        """Reverse pass from the final-state gradients; returns a dict of input gradients."""
        s = self.diff.solver
        dev = s.device
        ext = None if external_forces is None else external_forces.detach().contiguous()
        act = None if activations is None else activations.detach().contiguous()
        T, H = s.model.tet_count, s.hex_count
        acc = {
            "ext": torch.zeros((self.P, 3), dtype=torch.float32, device=dev) if ext is not None else None,
            "act": torch.zeros(T, dtype=torch.float32, device=dev) if act is not None and T else None,
            "scale": torch.zeros(T, dtype=torch.float32, device=dev) if mu_scale is not None and T else None,
            "tet_mat": torch.zeros((T, 3), dtype=torch.float32, device=dev) if materials and T else None,
            "hex_mat": torch.zeros((H, 3), dtype=torch.float32, device=dev) if materials and H else None,
        }
        self._prime(ext, act, acc)
        if self.overlap is not None and self.diff._scale is not None:
            self.overlap.set_mu_scale(self.diff._scale)
        self.q_bar.copy_(q_bar)
        self.v_bar.copy_(v_bar)
        if self.adj_start is not None:
            self.adj_start.zero_()
        # captured graphs bake in the accumulator pointers: one set of graphs per pointer set
        key = (None if ext is None else ext.data_ptr(), None if act is None else act.data_ptr(),
               tuple(None if t is None else t.data_ptr() for t in acc.values()))
        main = torch.cuda.current_stream(dev)
        nseg = len(self.bounds)
        if self.store_all:
            for i in reversed(range(nseg)):
                a, b = self.bounds[i]
                self._adjoint(self.q_states[0][a:], self.v_states[0][a:], b - a, self.refresh, ext, act, acc)
        elif self.overlap is None:
            for i in reversed(range(nseg)):
                self._recompute(i, 0, main, ext, act)
                self._reverse(i, 0, main, ext, act, acc, key)
        else:
            rec = torch.cuda.Stream(dev)
            adj = torch.cuda.Stream(dev)
            rec.wait_stream(main)
            adj.wait_stream(main)
            done_rec = [torch.cuda.Event(), torch.cuda.Event()]
            done_adj = [torch.cuda.Event(), torch.cuda.Event()]
            used = [False, False]
            self._recompute(nseg - 1, (nseg - 1) % 2, rec, ext, act)
            done_rec[(nseg - 1) % 2].record(rec)
            for i in reversed(range(nseg)):
                buf = i % 2
                if i > 0:  # recompute the previous segment while this one runs its reverse pass
                    nb = (i - 1) % 2
                    if used[nb]:
                        rec.wait_event(done_adj[nb])
                    self._recompute(i - 1, nb, rec, ext, act)
                    done_rec[nb].record(rec)
                adj.wait_event(done_rec[buf])
                self._reverse(i, buf, adj, ext, act, acc, key)
                done_adj[buf].record(adj)
                used[buf] = True
            main.wait_stream(adj)
            main.wait_stream(rec)
            for t in list(self.q_states) + list(self.v_states) + list(self.dv_in) + \
                    [self.q_bar, self.v_bar] + [t for t in acc.values() if t is not None]:
                t.record_stream(adj)
                t.record_stream(rec)
        out = {"q0": self.q_bar.clone(), "v0": self.v_bar.clone()}
        names = {"ext": "external_forces", "act": "activations", "scale": "mu_scale", "tet_mat": "tet_materials",
                 "hex_mat": "hex_materials"}
        for k, t in acc.items():
            if t is not None:
                out[names[k]] = t
        return out


def device_checkpointed_gradient(diff: DifferentiableSolver, q0, v0, steps: int, every: int, loss_fn, *,
                                 external_forces=None, activations=None, mu_scale=None, materials=False,
                                 refresh=False, warm_start=False, warm_adjoint=False, store_all=False, graphs=True,
                                 overlap: DifferentiableSolver | None = None, rollout: DeviceRollout | None = None):
    """Loss of a ``steps``-substep rollout and its gradients, computed on the device.

    ``loss_fn(q, v)`` maps the final state to a scalar (differentiated by torch).
    Returns (loss, grads) with grads keys ``q0``, ``v0`` and, when requested,
    ``external_forces`` (a load held over the rollout), ``activations``,
    ``mu_scale``, ``tet_materials``, ``hex_materials``.  Pass a ``DeviceRollout``
    to reuse its buffers and captured graphs across calls, and ``overlap`` (a
    second solver over the same model) to recompute segments concurrently with
    the reverse pass.
    """
    if mu_scale is not None:
        diff.set_mu_scale(mu_scale)
    ro = rollout or DeviceRollout(diff, steps, every, refresh=refresh, warm_start=warm_start,
                                  warm_adjoint=warm_adjoint, store_all=store_all, graphs=graphs, overlap=overlap)
    qf, vf = ro.forward(q0, v0, external_forces=external_forces, activations=activations)
    qf.requires_grad_(True)
    vf.requires_grad_(True)
    with torch.enable_grad():
        loss = loss_fn(qf, vf)
        qb, vb = torch.autograd.grad(loss, (qf, vf), allow_unused=True)
    qb = torch.zeros_like(qf) if qb is None else qb
    vb = torch.zeros_like(vf) if vb is None else vb
    grads = ro.backward(qb.detach(), vb.detach(), external_forces=external_forces, activations=activations,
                        mu_scale=mu_scale, materials=materials)
    return loss.detach(), grads

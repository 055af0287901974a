"""Prepared affine step over the GB300 solver (reference ``prepared_step.py:64-302``).

``SolverFEM.prepare_step`` evaluates the force terms of an accepted state once
and returns this workspace.  Its right-hand side, operator and preconditioner
actions, solve and reconstruction then run on the device through the C ABI
(``fem_prepare``, ``fem_prepared_rhs``, ``fem_apply_operator``,
``fem_apply_preconditioner``, ``fem_prepared_solve``,
``fem_prepared_reconstruct``), so they can be captured in CUDA graphs.

The workspace owns its arrays (``base_rhs``, ``velocity_increment``,
``diagonal_blocks`` and the copied state); one workspace is reused per solver.
Preparing again, or changing the solver's matrix (``refresh_tangent``,
``rebuild_element_blocks``, a new timestep), invalidates the previous
preparation, as in the reference.
"""

from __future__ import annotations

import ctypes
import math

import torch

from . import _lib


class PreparedFEMStep:
    """A prepared equation ``operator * delta_v = rhs(external_forces)``."""

    def __init__(self, solver):
        self.solver = solver
        self.model = solver.model
        self.device = solver.device
        P = self.model.particle_count
        f32 = dict(dtype=torch.float32, device=self.device)
        self._q = torch.zeros((P, 3), **f32)
        self._v = torch.zeros((P, 3), **f32)
        self._impulse = torch.zeros((P, 3), **f32)
        self._predictor = torch.zeros((P, 3), **f32)
        self._rhs = torch.zeros((P, 3), **f32)
        self.base_rhs = torch.zeros((P, 3), **f32)
        self.velocity_increment = torch.zeros((P, 3), **f32)
        self.diagonal_blocks = torch.zeros((P, 3, 3), **f32)
        self.fixed_mask = torch.zeros(P, dtype=torch.int32, device=self.device)
        if len(solver.fixed_particle_indices):
            idx = torch.as_tensor(solver.fixed_particle_indices, dtype=torch.long, device=self.device)
            self.fixed_mask[idx] = 1
        self._ws = _lib.FemPreparedWs(*(t.data_ptr() for t in (
            self._q, self._v, self._impulse, self._predictor, self.base_rhs, self.velocity_increment,
            self.diagonal_blocks)))
        self._revision = None
        self.dt = None

    # -- checks --------------------------------------------------------------
    def _check_current(self):
        if self._revision is None:
            raise RuntimeError("Prepare FEM mechanics before using this workspace")
        if self._revision != self.solver._revision or self.dt != self.solver.dt:
            raise RuntimeError("FEM mechanics changed; prepare the step again")

    def _vectors(self, t, name):
        P = self.model.particle_count
        if not isinstance(t, torch.Tensor) or tuple(t.shape) != (P, 3) or t.dtype != torch.float32 or \
                t.device != torch.device(self.device) or not t.is_contiguous():
            raise ValueError(f"{name} must be a particle-sized vec3 array on the model device")

    def _call(self, fn, *args):
        _lib.check(fn(self.solver._handle, *args), "prepared step")

    # -- API -----------------------------------------------------------------
    def prepare(self, state_in, control, contacts, dt, external_forces=None):
        """Copy the accepted state and evaluate its force terms once (prepared_step.py:126-183)."""
        if torch.cuda.is_current_stream_capturing():
            raise RuntimeError("Prepare FEM mechanics before CUDA graph capture")
        dt = float(dt)
        if not math.isfinite(dt) or dt <= 0 or dt != self.solver.dt:
            raise ValueError("Prepared timestep must be finite, positive and match the assembled tangent timestep")
        self._vectors(state_in.particle_q, "particle_q")
        self._vectors(state_in.particle_qd, "particle_qd")
        if external_forces is not None:
            self._vectors(external_forces, "external_forces")
        act = self.solver._activations(control)
        self.solver._register_contacts(contacts)
        self._revision = None
        lib = self.solver._lib
        self._call(lib.fem_prepare, ctypes.byref(self._ws), state_in.particle_q.data_ptr(),
                   state_in.particle_qd.data_ptr(), None if external_forces is None else external_forces.data_ptr(),
                   None if act is None else act.data_ptr(), self.model.gravity.data_ptr(), dt,
                   self.solver._stream())
        self.dt, self._revision = dt, self.solver._revision
        return self

    def rhs(self, external_forces=None, out=None):
        """The constrained impulse with an additional nodal load in newtons (prepared_step.py:185-213)."""
        self._check_current()
        out = self._rhs if out is None else out
        self._vectors(out, "out")
        if external_forces is not None:
            self._vectors(external_forces, "external_forces")
            if external_forces.data_ptr() == out.data_ptr():
                raise ValueError("RHS output must not alias its external-force input")
        self._call(self.solver._lib.fem_prepared_rhs, ctypes.byref(self._ws),
                   None if external_forces is None else external_forces.data_ptr(), self.dt, out.data_ptr(),
                   self.solver._stream())
        return out

    def apply_operator(self, vector, out):
        """out = (PAP + I - P) vector, without a solve (prepared_step.py:215-224)."""
        self._check_current()
        self._vectors(vector, "vector")
        self._vectors(out, "out")
        if vector.data_ptr() == out.data_ptr():
            raise ValueError("Operator action requires distinct input and output storage")
        self._call(self.solver._lib.fem_apply_operator, vector.data_ptr(), out.data_ptr(), self.solver._stream())
        return out

    def apply_preconditioner(self, vector, out):
        """out = M vector with the solver's preconditioner (prepared_step.py:226-235)."""
        self._check_current()
        self._vectors(vector, "vector")
        self._vectors(out, "out")
        if vector.data_ptr() == out.data_ptr():
            raise ValueError("Preconditioner action requires distinct input and output storage")
        self._call(self.solver._lib.fem_apply_preconditioner, vector.data_ptr(), out.data_ptr(),
                   self.solver._stream())
        return out

    def prepare_solve(self, tolerance=None):
        """Validate a solve tolerance (the handle's scratch is allocated once, so nothing else is needed)."""
        self._check_current()
        tol = self.solver.linear_solver_tolerance if tolerance is None else float(tolerance)
        if not math.isfinite(tol) or tol <= 0:
            raise ValueError("linear solver tolerance must be finite and positive")
        return tol

    def solve(self, rhs, out=None, *, tolerance=None):
        """Normalised PCG from this workspace's increment; updates only that guess (prepared_step.py:252-275)."""
        self._vectors(rhs, "rhs")
        tol = self.prepare_solve(tolerance)
        self._call(self.solver._lib.fem_prepared_solve, ctypes.byref(self._ws), rhs.data_ptr(), tol,
                   int(self.solver.linear_solver_maxiter), self.dt, self.solver._stream())
        if out is not None:
            self._vectors(out, "out")
            out.copy_(self.velocity_increment)
            return out
        return self.velocity_increment

    def reconstruct(self, delta_v, state_out):
        """state_out from the prepared state and delta_v, fixed supports restored (prepared_step.py:277-302)."""
        self._check_current()
        self._vectors(delta_v, "delta_v")
        self._vectors(state_out.particle_q, "particle_q")
        self._vectors(state_out.particle_qd, "particle_qd")
        if state_out.particle_q.data_ptr() == self._q.data_ptr() or \
                state_out.particle_qd.data_ptr() == self._v.data_ptr():
            raise ValueError("Reconstruction must not overwrite the prepared input")
        self._call(self.solver._lib.fem_prepared_reconstruct, ctypes.byref(self._ws), delta_v.data_ptr(), self.dt,
                   state_out.particle_q.data_ptr(), state_out.particle_qd.data_ptr(), self.solver._stream())
        return state_out

"""``SolverFEM``: the reference's solver interface over the GB300 C-ABI library.

Keeps the reference constructor (``solver.py:212-240``), its validation
(``solver.py:241-262``), ``step(state_in, state_out, control, contacts, dt, *,
external_forces=)`` (``solver.py:942-1002``), the tangent-refresh calls
(``refresh_tangent`` ``solver.py:769-857``, ``rebuild_element_blocks``
``solver.py:506-508``, ``refresh_preconditioner`` ``solver.py:502-504``), the
mutable ``linear_solver_tolerance`` / ``linear_solver_maxiter``, ``reset``,
``velocity_increment``, ``last_cg_iters``, the per-term force evaluators and the
volume telemetry.  Every numerical operation runs in ``libfemgb300.so`` on the
model's CUDA device, enqueued on the current torch stream; tensors are only
buffers.  There is no CPU path: a CPU model is rejected.

Implemented hot-path options: ``solver_type="cg"`` with ``preconditioner_type``
``"block_diag"`` or ``"diag"``; Tet4, Hex8, triangle membranes, springs with
the optional bend torque, hash-grid particle-particle contact, soft-rigid
contacts (``contacts.soft_contact_*``), analytic ground, gravity, linear
damping, tet activations, fixed nodes, batched independent scenes
(``model.scene_offsets``), soft-body surface contacts
(``set_soft_surface_contacts``).  Other Krylov types are outside this path.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from .builder import Model, State


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _f32(t: torch.Tensor, shape, name: str, device) -> torch.Tensor:
    if not isinstance(t, torch.Tensor) or t.dtype != torch.float32 or tuple(t.shape) != tuple(shape) or \
            t.device != device or not t.is_contiguous():
        raise ValueError(f"{name} must be a contiguous float32 tensor of shape {tuple(shape)} on {device}")
    return t


class BsrMatrix:
    """Exported 3x3-block CSR matrix in the reference's Warp ``BsrMatrix`` layout."""

    def __init__(self, offsets: torch.Tensor, columns: torch.Tensor, values: torch.Tensor, nrow: int):
        self.offsets = offsets
        self.columns = columns
        self.values = values
        self.nrow = nrow
        self.ncol = nrow
        self.nnz = int(columns.shape[0])

    def dense(self) -> np.ndarray:
        offsets, columns, values = self.offsets.cpu().numpy(), self.columns.cpu().numpy(), self.values.cpu().numpy()
        out = np.zeros((3 * self.nrow, 3 * self.ncol))
        rows = np.repeat(np.arange(self.nrow), np.diff(offsets))
        for k in range(len(columns)):
            r, c = rows[k], columns[k]
            out[3 * r:3 * r + 3, 3 * c:3 * c + 3] += values[k]
        return out


class SoftBodySurfaceContacts:
    """Registered surface-contact geometry (reference ``soft_surface_contacts.py``).

    The surfaces and their BVHs live in the library handle; ``update`` refits
    them at new positions, ``eval_forces`` evaluates the surface term alone."""

    def __init__(self, solver, particle_ranges, surface_triangles_list, ke: float, kd: float):
        self._solver = solver
        self.ke, self.kd = float(ke), float(kd)
        self.n_bodies = len(particle_ranges)
        self.particle_ranges = [(int(a), int(b)) for a, b in particle_ranges]

    def update(self, particle_q: torch.Tensor) -> None:
        """Refit every body's surface at particle_q (SoftBodySurfaceContacts.update)."""
        sv = self._solver
        _f32(particle_q, (sv.model.particle_count, 3), "particle_q", sv.device)
        _lib.check(sv._lib.fem_update_surface_contacts(sv._handle, particle_q.data_ptr(), sv._stream()),
                   "surface contacts")

    def eval_forces(self, particle_q, particle_v, particle_radius=None, particle_flags=None, particle_count=None):
        """Surface contact force per particle at (particle_q, particle_v), with the model's radii and flags."""
        sv = self._solver

        class _S:
            pass

        st = _S()
        st.particle_q, st.particle_qd = particle_q, particle_v
        return sv._forces(st, _lib.FEM_TERM_SURFACE)


class StreamingTetAssembly:
    """State of prepared tetrahedral updates (reference ``streaming.py`` ``StreamingTetAssembly``).

    The reserved pattern and every update live in the library handle; this
    object keeps the pool layout and the counters of the last update."""

    def __init__(self, original_node_count: int, node_count: int, element_count: int):
        self.original_node_count = int(original_node_count)
        self.copies = node_count // self.original_node_count
        self.node_count, self.element_count = node_count, element_count
        self.last_update: dict = {}


class SolverFEM:
    """Linearly implicit Backward-Euler FEM solver (reference ``SolverFEM``) on one GB300."""

    def __init__(
        self,
        model: Model,
        dt: float = 1.0 / 60.0,
        mass: float = 1.0,
        preconditioner_type: str = "diag",
        solver_type: str = "bicgstab",
        linear_solver_maxiter: int = 50,
        min_stretch: float = 0.05,
        max_stretch: float = 20.0,
        ground_plane=None,
        ground_ke: float = 1.0e5,
        ground_kd: float = 1.0e2,
        ground_kf: float = 1.0e3,
        ground_mu: float = 0.5,
        torque_stiffness: float = 0.0,
        torque_damping: float = 0.0,
        spring_rest_direction=None,
        self_contact_ke: float = 1.0e3,
        self_contact_kd: float = 1.0e2,
        linear_damping: float = 0.0,
        differentiable: bool = False,
        enable_tet_activations: bool = False,
        defer_differentiation_checks: bool = False,
        tet_volume_weights=None,
        fixed_particle_indices=None,
        linear_solver_tolerance: float = 1.0e-2,
        linear_solver_use_cuda_graph: bool = True,
    ):
        if not math.isfinite(linear_solver_tolerance) or linear_solver_tolerance <= 0:
            raise ValueError("linear_solver_tolerance must be finite and positive")
        fixed = np.asarray([] if fixed_particle_indices is None else fixed_particle_indices)
        if fixed.ndim != 1 or (fixed.size and fixed.dtype.kind not in "iu"):
            raise ValueError("fixed_particle_indices must be a one-dimensional integer sequence")
        if fixed.size and (fixed.min() < 0 or fixed.max() >= model.particle_count):
            raise ValueError("fixed_particle_indices contains an out-of-range node")
        fixed = np.unique(fixed).astype(np.int32)
        if fixed.size and differentiable:
            raise ValueError("fixed_particle_indices is not supported with differentiable=True")
        if not isinstance(model.particle_q, torch.Tensor) or model.particle_q.device.type != "cuda":
            raise RuntimeError("SolverFEM on GB300 requires a model on a CUDA device (no CPU path)")
        if solver_type not in ("cg", "bicgstab", "gmres", "cr"):
            raise ValueError(f"Invalid solver type: {solver_type}")
        if solver_type != "cg":
            raise NotImplementedError(
                f"solver_type={solver_type!r} is not implemented on GB300; pass solver_type='cg' (the reference's "
                f"default is 'bicgstab', but its hot path and every shipped configuration use 'cg')")
        if preconditioner_type not in ("block_diag", "diag"):
            raise NotImplementedError(f"preconditioner_type={preconditioner_type!r} is not implemented")
        self.torque_stiffness = float(torque_stiffness)
        self.torque_damping = float(torque_damping)
        if spring_rest_direction is None:
            self.spring_rest_direction = np.zeros((model.spring_count, 3), np.float32)
        else:
            srd = spring_rest_direction
            srd = srd.detach().cpu().numpy() if isinstance(srd, torch.Tensor) else np.asarray(srd)
            if srd.shape != (model.spring_count, 3):
                raise ValueError(f"spring_rest_direction shape {srd.shape} != (spring_count={model.spring_count}, 3)")
            self.spring_rest_direction = np.ascontiguousarray(srd, dtype=np.float32)
        self._torque = self.torque_stiffness > 0.0 and spring_rest_direction is not None and model.spring_count > 0
        if tet_volume_weights is not None:
            w = torch.as_tensor(tet_volume_weights)
            if tuple(w.shape) != (model.tet_count,) or not torch.isfinite(w).all() or (w < 0).any():
                raise ValueError("tet_volume_weights must be finite and nonnegative with shape (tet_count,)")
        self.model = model
        self.device = model.particle_q.device
        self.mass = float(mass)
        self.preconditioner_type = preconditioner_type
        self.solver_type = solver_type
        self.min_stretch = float(min_stretch)
        self.max_stretch = float(max_stretch)
        self.linear_damping = float(linear_damping)
        self.differentiable = bool(differentiable)
        self.defer_differentiation_checks = bool(defer_differentiation_checks)
        self.last_differentiation_residuals = None
        self._diff = None
        self.enable_tet_activations = bool(enable_tet_activations)
        self.linear_solver_use_cuda_graph = bool(linear_solver_use_cuda_graph)
        self.linear_solver_check_every = 0
        self.dt = float(dt)
        self.hex_count = int(model.fem.hex_count) if getattr(model, "fem", None) is not None else 0
        self.fixed_particle_indices = fixed
        self._tet_volume_weights = tet_volume_weights
        self._ground_plane = None if ground_plane is None else tuple(float(v) for v in ground_plane)
        model.particle_ke = float(self_contact_ke)
        model.particle_kd = float(self_contact_kd)
        # solver.py:1477-1488: the hash-grid contact runs only with a positive stiffness,
        # more than one particle, a positive maximum radius and a model particle grid
        self._particle_contact = (model.particle_ke > 0.0 and model.particle_count > 1 and
                                  model.particle_max_radius > 0.0 and getattr(model, "particle_grid", None) is not None)
        self._contacts_key = None
        self._lib = _lib.load()
        self._handle = ctypes.c_void_p()
        self._revision = 0  # matrix revision (refresh_tangent, rebuild_element_blocks, model changes)
        self._prepared_step = None
        self._streaming = None
        self._stepped = False
        self._soft_surface_contacts = None
        P = model.particle_count
        # persistent velocity increment, owned here so it is visible as a tensor
        self.dv = torch.zeros((P, 3), dtype=torch.float32, device=self.device)
        self._create(model, fixed, linear_solver_maxiter, linear_solver_tolerance, ground_ke, ground_kd, ground_kf,
                     ground_mu)
        self._tolerance = float(linear_solver_tolerance)
        self._maxiter = int(linear_solver_maxiter)
        self._initial_volume = self._compute_volume(model.particle_q)

    # ------------------------------------------------------------------ setup
    def _create(self, model, fixed, maxiter, tolerance, gke, gkd, gkf, gmu):
        self._ground_params = (gke, gkd, gkf, gmu)
        self._topology_storage = self._topology_signature()
        d, keep = self._descriptor(model, fixed, maxiter, tolerance)
        with torch.cuda.device(self.device):
            torch.cuda.current_stream(self.device).synchronize()
            _lib.check(self._lib.fem_create(ctypes.byref(d), ctypes.byref(self._handle)), "SolverFEM")
        del keep

    def _topology_signature(self):
        """Capacities and storage of the arrays a topology refresh may rewrite in place."""
        m = self.model
        arrays = (m.particle_mass, m.particle_inv_mass, m.particle_flags, m.tet_indices, m.tet_poses, m.tet_materials,
                  m.tri_indices, m.tri_poses, m.tri_materials)
        counts = (m.particle_count, m.tet_count, self.hex_count, m.spring_count, m.tri_count)
        return counts, tuple(None if a is None else (a.data_ptr(), tuple(a.shape)) for a in arrays)

    def _descriptor(self, model, fixed, maxiter, tolerance):
        """The FemDesc of the model's current arrays (and the host copies it points into)."""
        gke, gkd, gkf, gmu = self._ground_params
        keep = []

        def host(t, dtype):
            if t is None:
                return None
            a = np.ascontiguousarray(t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else t, dtype=dtype)
            keep.append(a)
            return a.ctypes.data

        d = _lib.FemDesc()
        P = model.particle_count
        fem = getattr(model, "fem", None)
        H = self.hex_count
        d.particle_count = P
        d.tet_count = model.tet_count
        d.hex_count = H
        d.spring_count = model.spring_count
        d.particle_q = host(model.particle_q, np.float32)
        d.particle_mass = host(model.particle_mass, np.float32)
        d.particle_inv_mass = host(model.particle_inv_mass, np.float32)
        d.particle_radius = host(model.particle_radius, np.float32)
        d.particle_flags = host(model.particle_flags, np.int32)
        if model.tet_count:
            d.tet_indices = host(model.tet_indices, np.int32)
            d.tet_poses = host(model.tet_poses, np.float32)
            d.tet_materials = host(model.tet_materials, np.float32)
        if H:
            d.hex_indices = host(fem.hex_indices, np.int32)
            d.hex_materials = host(fem.hex_materials, np.float32)
            d.hex_inv_J0 = host(fem.hex_inv_J0, np.float32)
            d.hex_det_J0_w = host(fem.hex_det_J0_w, np.float32)
        if model.spring_count:
            d.spring_indices = host(model.spring_indices, np.int32)
            d.spring_rest_length = host(model.spring_rest_length, np.float32)
            d.spring_stiffness = host(model.spring_stiffness, np.float32)
            d.spring_damping = host(model.spring_damping, np.float32)
        if model.tri_count:
            d.tri_count = model.tri_count
            d.tri_indices = host(model.tri_indices, np.int32)
            d.tri_poses = host(model.tri_poses, np.float32)
            d.tri_materials = host(model.tri_materials, np.float32)
        if self._torque:
            d.spring_rest_direction = host(self.spring_rest_direction, np.float32)
            d.torque_stiffness = self.torque_stiffness
            d.torque_damping = self.torque_damping
        d.particle_contact = int(self._particle_contact)
        d.particle_ke, d.particle_kd = float(model.particle_ke), float(model.particle_kd)
        d.particle_kf, d.particle_mu = float(model.particle_kf), float(model.particle_mu)
        d.particle_cohesion = float(model.particle_cohesion)
        d.particle_max_radius = float(model.particle_max_radius)
        d.soft_contact_ke, d.soft_contact_kd = float(model.soft_contact_ke), float(model.soft_contact_kd)
        d.soft_contact_kf, d.soft_contact_mu = float(model.soft_contact_kf), float(model.soft_contact_mu)
        d.fixed_indices = host(fixed, np.int32) if fixed.size else None
        d.fixed_count = int(fixed.size)
        offsets = getattr(model, "scene_offsets", None)
        if offsets is not None:
            d.scene_offsets = host(offsets, np.int64)
            d.scene_count = len(offsets) - 1
        g = model.gravity.detach().cpu().numpy().astype(np.float32)
        d.gravity[:] = list(g)
        d.dt = self.dt
        d.min_stretch = self.min_stretch
        d.max_stretch = self.max_stretch
        d.has_ground = 1 if self._ground_plane is not None else 0
        if self._ground_plane is not None:
            d.ground_plane[:] = list(self._ground_plane)
        d.ground_ke, d.ground_kd, d.ground_kf, d.ground_mu = gke, gkd, gkf, gmu
        d.linear_damping = self.linear_damping
        d.enable_tet_activations = int(self.enable_tet_activations)
        d.preconditioner = _lib.FEM_PRECOND_BLOCK_DIAG if self.preconditioner_type == "block_diag" else \
            _lib.FEM_PRECOND_DIAG
        d.maxiter = int(maxiter)
        d.tolerance = float(tolerance)
        d.velocity_increment = self.dv.data_ptr()
        return d, keep

    def refresh_topology(self, particle_q: torch.Tensor, dt: float | None = None, *, element_sources=None) -> None:
        """Rebuild the pattern after in-place edits of tet connectivity and masses (reference ``solver.py:872-940``).

        Particle and element capacities and the model's array storage must be
        unchanged; unused tet slots carry zero materials and valid node
        indices.  The constant matrix, the sparsity pattern, the slot map and
        the preconditioner are rebuilt and the tangent is assembled at
        ``particle_q`` (fixed nodes restored in place); the warm start is
        cleared.  The handle's storage is rebuilt, so CUDA graphs captured
        before the call must be captured again.

        After :meth:`prepare_tetrahedral_updates` the edit is applied instead
        to the reserved pattern in fixed device storage (captured graphs stay
        valid), validated before anything changes, with ``element_sources`` (a
        device int32 array of previous element ids per slot, -1 for new
        elements; default: equal slot ids) for the lineage counters in
        ``self._streaming.last_update``.  Without prepared updates
        ``element_sources`` is ignored, as in the reference.
        """
        dt = self.dt if dt is None else float(dt)
        if torch.cuda.is_current_stream_capturing():
            raise RuntimeError("refresh_topology must run outside CUDA graph capture")
        if self.preconditioner_type != "block_diag":
            raise ValueError("Persistent topology updates require the block_diag preconditioner")
        if dt != self.dt:
            raise ValueError("refresh_topology requires the solver's currently assembled timestep")
        if self._topology_signature() != self._topology_storage:
            raise ValueError("Topology updates must preserve model capacities and array storage")
        _f32(particle_q, (self.model.particle_count, 3), "particle_q", self.device)
        self._revision += 1
        d, keep = self._descriptor(self.model, self.fixed_particle_indices, self.linear_solver_maxiter,
                                   self.linear_solver_tolerance)
        if self._streaming is not None:
            T = self.model.tet_count
            if element_sources is not None:
                src = element_sources
                if not isinstance(src, torch.Tensor) or src.dtype != torch.int32 or src.ndim != 1 or \
                        src.numel() < T:
                    raise ValueError("Element sources must be a capacity-sized int32 array")
                if src.device != self.device:
                    raise ValueError("Element sources must reside on the solver device")
                src = src.contiguous()
            u = _lib.FemTopologyUpdate()
            with torch.cuda.device(self.device):
                _lib.check(self._lib.fem_update_tet_topology(
                    self._handle, ctypes.byref(d), particle_q.data_ptr(), dt,
                    None if element_sources is None else src.data_ptr(), ctypes.byref(u), self._stream()),
                    "refresh_topology")
            del keep
            self._streaming.last_update = {name: int(getattr(u, name)) for name, _ in u._fields_}
            self._streaming.last_update["full_numeric_refresh"] = bool(u.full_numeric_refresh)
            return
        with torch.cuda.device(self.device):
            _lib.check(self._lib.fem_refresh_topology(self._handle, ctypes.byref(d), particle_q.data_ptr(), dt,
                                                      self._stream()), "refresh_topology")
        del keep

    def set_soft_surface_contacts(self, particle_ranges, surface_triangles_list, ke: float = 1.0e3,
                                  kd: float = 1.0e2) -> None:
        """Register per-body surface meshes for soft-soft contacts (reference ``solver.py:510-540``).

        ``particle_ranges`` lists ``(start, count)`` particle slices, one per
        body; ``surface_triangles_list`` the per-body ``(T_i, 3)`` triangles with
        body-local indices (``None`` for a body without surface).  Each surface
        vertex is pushed out of the other bodies' surfaces (penalty ``ke``,
        damping ``kd``).  The surfaces take the current model positions now and
        are refitted by the first ``refresh_tangent``, by every
        ``rebuild_element_blocks`` and by ``soft_surface_contacts.update``.
        Call before capturing graphs.
        """
        if torch.cuda.is_current_stream_capturing():
            raise RuntimeError("Register surface contacts before CUDA graph capture")
        if len(particle_ranges) != len(surface_triangles_list):
            raise ValueError("particle_ranges and surface_triangles_list must have one entry per body")
        starts, sizes, offsets, tris = [], [], [0], []
        for (start, count), t in zip(particle_ranges, surface_triangles_list):
            starts.append(int(start))
            sizes.append(int(count))
            t = np.zeros((0, 3), np.int32) if t is None else np.asarray(t, np.int32).reshape(-1, 3)
            tris.append(t)
            offsets.append(offsets[-1] + len(t))
        starts = np.asarray(starts, np.int32)
        sizes = np.asarray(sizes, np.int32)
        offsets = np.asarray(offsets, np.int32)
        tris = np.ascontiguousarray(np.concatenate(tris) if tris else np.zeros((0, 3), np.int32), np.int32)
        with torch.cuda.device(self.device):
            _lib.check(self._lib.fem_set_surface_contacts(
                self._handle, len(starts), starts.ctypes.data, sizes.ctypes.data, offsets.ctypes.data,
                tris.ctypes.data if len(tris) else None, float(ke), float(kd), self.model.particle_q.data_ptr(),
                self._stream()), "set_soft_surface_contacts")
        self._soft_surface_contacts = SoftBodySurfaceContacts(self, particle_ranges, surface_triangles_list, ke, kd)

    @property
    def soft_surface_contacts(self):
        """Registered surface contact geometry, or None."""
        return self._soft_surface_contacts

    def prepare_tetrahedral_updates(self, original_node_count: int) -> None:
        """Reserve persistent sparse connections for duplicated Tet4 basis nodes (reference ``solver.py:693-719``).

        Pool node ``i`` represents original node ``i % original_node_count``;
        later tetrahedra may use any copy of their original corners.  Needs
        tetrahedra only, ``block_diag`` and no fixed nodes; call before
        capturing graphs or stepping.  Afterwards ``refresh_topology`` applies
        edits to fixed device storage (graphs captured earlier stay valid) and
        accepts ``element_sources``.
        """
        if self.fixed_particle_indices.size:
            raise ValueError("Streaming topology is not supported with fixed_particle_indices")
        if torch.cuda.is_current_stream_capturing() or self._stepped:
            raise RuntimeError("Prepare tetrahedral updates before capturing or stepping the solver")
        if self._streaming is not None:
            raise RuntimeError("Tetrahedral updates are already prepared")
        d, keep = self._descriptor(self.model, self.fixed_particle_indices, self.linear_solver_maxiter,
                                   self.linear_solver_tolerance)
        with torch.cuda.device(self.device):
            _lib.check(self._lib.fem_prepare_tet_updates(self._handle, ctypes.byref(d), int(original_node_count),
                                                         self._stream()), "prepare_tetrahedral_updates")
        del keep
        self._revision += 1
        self._streaming = StreamingTetAssembly(original_node_count, self.model.particle_count, self.model.tet_count)

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle is not None and handle.value:
            try:
                torch.cuda.synchronize(self.device)
                self._lib.fem_destroy(handle)
            except Exception:
                pass
            self._handle = ctypes.c_void_p()

    def _stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    # ------------------------------------------------------------------ settings
    @property
    def linear_solver_tolerance(self) -> float:
        return self._tolerance

    @linear_solver_tolerance.setter
    def linear_solver_tolerance(self, value: float) -> None:
        value = float(value)
        _lib.check(self._lib.fem_set_tolerance(self._handle, value), "linear_solver_tolerance")
        self._tolerance = value

    @property
    def linear_solver_maxiter(self) -> int:
        return self._maxiter

    @linear_solver_maxiter.setter
    def linear_solver_maxiter(self, value: int) -> None:
        _lib.check(self._lib.fem_set_maxiter(self._handle, int(value)), "linear_solver_maxiter")
        self._maxiter = int(value)

    @property
    def velocity_increment(self) -> torch.Tensor:
        """Persistent solved velocity increment (also the next solve's warm start)."""
        return self.dv

    # ------------------------------------------------------------------ step
    def step(self, state_in: State, state_out: State, control, contacts, dt: float, *, external_forces=None,
             observables=None):
        """Advance one linearly implicit substep (reference ``solver.py:942-1002``).

        ``state_in.particle_f`` is overwritten with the final right-hand side
        ``h*sum(f) - h^2 K v`` (projected); fixed nodes of ``state_in`` are
        restored in place, as in the reference.
        """
        if self.differentiable:
            return self._differentiable_step(state_in, state_out, control, contacts, dt, external_forces)
        P = self.model.particle_count
        dev = self.device
        ext = None
        if external_forces is not None:
            if not isinstance(external_forces, torch.Tensor) or tuple(external_forces.shape) != (P, 3) or \
                    external_forces.dtype != torch.float32 or external_forces.device != dev:
                raise ValueError("external_forces must be a model-sized wp.vec3 array on the model device")
            ext = external_forces.contiguous()
        for name, t in (("state_in.particle_q", state_in.particle_q), ("state_in.particle_qd", state_in.particle_qd),
                        ("state_out.particle_q", state_out.particle_q),
                        ("state_out.particle_qd", state_out.particle_qd), ("state_in.particle_f", state_in.particle_f)):
            _f32(t, (P, 3), name, dev)
        act = self._activations(control)
        self._register_contacts(contacts)
        self._stepped = True
        code = self._lib.fem_step(
            self._handle, state_in.particle_q.data_ptr(), state_in.particle_qd.data_ptr(),
            state_out.particle_q.data_ptr(), state_out.particle_qd.data_ptr(), state_in.particle_f.data_ptr(),
            _ptr(ext), _ptr(act), self.model.gravity.data_ptr(), float(dt), self._stream())
        _lib.check(code, "step")
        if self.linear_solver_check_every > 0:
            stats = self.stats()
            self.last_cg_iters = stats["max_iterations"]
        return state_out

    # ------------------------------------------------------------------ differentiable mode
    # Reference differentiation.step (differentiation.py:287-394): the matrix is held fixed, every solve
    # is a checked solve from zero at tolerance 1e-8 within linear_solver_maxiter, and the step is
    # recorded on the tape -- here torch autograd: outputs are attached to state_out.
    DIFF_RESIDUAL_BUDGET = 2.0e-5  # differentiation.py:162-166: residual <= 2e-5 ||b|| (+ 1e-10)

    def _differentiation(self):
        if self._diff is None:
            if self._streaming is not None:
                raise NotImplementedError("Differentiation requires fixed topology without streaming/component "
                                          "scaling")
            if self._soft_surface_contacts is not None or self.model.particle_ke > 0.0:
                raise NotImplementedError("Differentiation supports analytic ground contact; disable "
                                          "particle/surface contacts")
            for name in ("particle_mass", "particle_inv_mass", "particle_radius", "tet_poses", "tet_materials",
                         "tri_poses", "tri_materials", "spring_stiffness", "spring_damping", "spring_rest_length",
                         "gravity"):
                value = getattr(self.model, name, None)
                if isinstance(value, torch.Tensor) and value.requires_grad:
                    raise ValueError(f"{name} is fixed: finalize the model without gradients and enable "
                                     f"state/control gradients")
            if torch.cuda.is_current_stream_capturing():
                raise RuntimeError("Call prepare_differentiation() before CUDA graph capture")
            from .adjoint import DifferentiableSolver

            self._diff = DifferentiableSolver(self, tolerance=1.0e-8, maxiter=self.linear_solver_maxiter)
            self._diff.after_backward_solve = self._after_adjoint_solve
        return self._diff

    def prepare_differentiation(self):
        """Set up the differentiable mode before capture (reference ``prepare``, differentiation.py:236-270)."""
        return self._differentiation()

    def _after_adjoint_solve(self):
        if not self.defer_differentiation_checks:
            self.check()

    def check(self, *, reset: bool = True) -> dict:
        """Largest forward / adjoint relative residuals since the last check; raises when either exceeds
        the reference's budget (``differentiation.check``, differentiation.py:263-272)."""
        if torch.cuda.is_current_stream_capturing():
            raise RuntimeError("Check differentiable residuals after launching the CUDA graph")
        out = (ctypes.c_float * 2)()
        _lib.check(self._lib.fem_get_solve_residuals(self._handle, out, int(reset), self._stream()))
        result = {"forward_relative_residual": float(out[0]), "backward_relative_residual": float(out[1])}
        self.last_differentiation_residuals = result
        if not all(math.isfinite(v) for v in result.values()) or \
                max(result.values()) > self.DIFF_RESIDUAL_BUDGET:
            raise RuntimeError(f"FEM differentiable linear solve did not converge: {result}")
        return result

    def _differentiable_step(self, state_in, state_out, control, contacts, dt, external_forces):
        if float(dt) != self.dt:
            raise ValueError("Differentiable dt must match the fixed matrix assembly timestep")
        if contacts is not None:
            raise NotImplementedError("Differentiation supports only the analytic ground contact law")
        if state_in.particle_q is state_out.particle_q or state_in.particle_qd is state_out.particle_qd or \
                state_in.particle_q.data_ptr() == state_out.particle_q.data_ptr() or \
                state_in.particle_qd.data_ptr() == state_out.particle_qd.data_ptr():
            raise ValueError("Use unique input/output states for every taped step")
        P = self.model.particle_count
        if external_forces is not None and (not isinstance(external_forces, torch.Tensor) or
                                            tuple(external_forces.shape) != (P, 3) or
                                            external_forces.device != self.device):
            raise ValueError("external_forces must be a model-sized wp.vec3 array on the model device")
        diff = self._differentiation()
        act = None
        if self.enable_tet_activations and self.model.tet_count:
            act = control.tet_activations if control is not None else self.model.tet_activations
        from .adjoint import _Substep

        q_out, v_out = _Substep.apply(diff, state_in.particle_q, state_in.particle_qd, float(dt), external_forces,
                                      act, None)
        if torch.is_grad_enabled() and (q_out.requires_grad or v_out.requires_grad):
            state_out.particle_q, state_out.particle_qd = q_out, v_out  # the taped outputs
        else:
            state_out.particle_q.copy_(q_out)
            state_out.particle_qd.copy_(v_out)
        self._stepped = True
        if not self.defer_differentiation_checks:
            self.check()
        return state_out

    def _register_contacts(self, contacts) -> None:
        """Point the library at ``contacts.soft_contact_*`` (or clear it) for the following launches.

        Re-registers only when the arrays change; a larger capacity than any
        registered before allocates scratch, which cannot happen under capture.
        """
        if contacts is None or not hasattr(contacts, "soft_contact_count"):
            key = None
        else:
            cap = int(contacts.soft_contact_max)
            arrays = (contacts.soft_contact_count, contacts.soft_contact_particle, contacts.soft_contact_body_pos,
                      contacts.soft_contact_body_vel, contacts.soft_contact_normal)
            shapes = ((1,), (cap,), (cap, 3), (cap, 3), (cap, 3))
            dtypes = (torch.int32, torch.int32, torch.float32, torch.float32, torch.float32)
            for a, shape, dtype in zip(arrays, shapes, dtypes):
                if not isinstance(a, torch.Tensor) or a.dtype != dtype or tuple(a.shape) != shape or \
                        a.device != self.device or not a.is_contiguous():
                    raise ValueError("contacts.soft_contact_* must be contiguous device arrays of soft_contact_max "
                                     "entries (count int32[1], particle int32, body_pos/body_vel/normal float32 [.,3])")
            key = (cap,) + tuple(a.data_ptr() for a in arrays)
        if key == self._contacts_key:
            return
        if key is not None and key[0] > getattr(self, "_contacts_capacity", 0) and \
                torch.cuda.is_current_stream_capturing():
            raise RuntimeError("register soft contacts of this capacity before CUDA graph capture")
        if key is None:
            code = self._lib.fem_set_soft_contacts(self._handle, None, None, None, None, None, 0)
        else:
            code = self._lib.fem_set_soft_contacts(self._handle, *key[1:], key[0])
        _lib.check(code, "soft contacts")
        if key is not None:
            self._contacts_capacity = max(key[0], getattr(self, "_contacts_capacity", 0))
        self._contacts_key = key

    def _activations(self, control):
        """The per-tet activations the force kernels read (None unless enabled)."""
        if not (self.enable_tet_activations and self.model.tet_count):
            return None
        act = control.tet_activations if control is not None else self.model.tet_activations
        _f32(act, (self.model.tet_count,), "tet_activations", self.device)
        return act

    def prepare_step(self, state_in, control, contacts, dt, *, external_forces=None):
        """Prepare reusable affine mechanics without integrating (reference ``solver.py:483-500``).

        Returns the solver's persistent :class:`PreparedFEMStep` with the
        constrained operator, the preconditioner, the base impulse and trial
        reconstruction.  The caller owns tangent refresh and must prepare again
        for every new accepted state, control or matrix revision.
        """
        from .prepared_step import PreparedFEMStep

        if torch.cuda.is_current_stream_capturing():
            raise RuntimeError("Prepare FEM mechanics before CUDA graph capture")
        if getattr(self, "_prepared_step", None) is None:
            self._prepared_step = PreparedFEMStep(self)
        return self._prepared_step.prepare(state_in, control, contacts, dt, external_forces)

    def stats(self) -> dict:
        """Synchronise and return the last solve's statistics (raises on a device timeout / NaN)."""
        s = _lib.FemStats()
        iters = (ctypes.c_int32 * max(1, self.model.scene_count))()
        code = self._lib.fem_get_stats(self._handle, ctypes.byref(s), iters, self._stream())
        _lib.check(code, "linear solve")
        return {
            "status": s.status,
            "max_iterations": s.max_iterations,
            "min_iterations": s.min_iterations,
            "max_relative_residual": s.max_relative_residual,
            "unconverged_scenes": s.unconverged_scenes,
            "total_iterations": s.total_iterations,
            "scene_iterations": list(iters)[: self.model.scene_count],
        }

    @property
    def last_cg_iters(self) -> int:
        return self.stats()["max_iterations"]

    @last_cg_iters.setter
    def last_cg_iters(self, value) -> None:
        pass

    # ------------------------------------------------------------------ tangent
    def refresh_tangent(self, particle_q: torch.Tensor, dt: float | None = None) -> None:
        """Refresh the element stiffness in place; a changed dt rebuilds all blocks and clears dv."""
        dt = self.dt if dt is None else float(dt)
        if not math.isfinite(dt) or dt <= 0:
            raise ValueError("refresh_tangent dt must be finite and positive")
        _f32(particle_q, (self.model.particle_count, 3), "particle_q", self.device)
        _lib.check(self._lib.fem_refresh_tangent(self._handle, particle_q.data_ptr(), dt, self._stream()),
                   "refresh_tangent")
        self.dt = dt
        self._revision += 1  # a new matrix revision invalidates prepared steps (solver.py:466-471)

    def rebuild_element_blocks(self, particle_q: torch.Tensor, dt: float, *, update_preconditioner=True) -> None:
        """Reassemble the Tet4/Hex8 blocks at particle_q and dt (the preconditioner refreshes in place)."""
        _f32(particle_q, (self.model.particle_count, 3), "particle_q", self.device)
        _lib.check(self._lib.fem_rebuild_element_blocks(self._handle, particle_q.data_ptr(), float(dt),
                                                        self._stream()), "rebuild_element_blocks")
        self._revision += 1

    def refresh_preconditioner(self) -> None:
        _lib.check(self._lib.fem_refresh_preconditioner(self._handle, self._stream()), "refresh_preconditioner")

    def reset(self, state=None, world_mask=None, flags=None) -> None:
        """Clear the warm start and the sticky device status."""
        _lib.check(self._lib.fem_reset(self._handle, self._stream()), "reset")

    def notify_model_changed(self, flags) -> None:
        """Gravity is read live from ``model.gravity``; topology edits need a new solver."""
        self._revision += 1

    # ------------------------------------------------------------------ matrix views
    def matrix_info(self) -> dict:
        nnzb, ntrip, stored = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(self._lib.fem_matrix_info(self._handle, ctypes.byref(nnzb), ctypes.byref(ntrip),
                                             ctypes.byref(stored)))
        return {"nnzb": nnzb.value, "triplets": ntrip.value, "stored_blocks": stored.value}

    @property
    def A_bsr(self) -> BsrMatrix:
        """Copy of the assembled A in BSR form (offsets [P+1], columns [nnzb], values [nnzb,3,3])."""
        info = self.matrix_info()
        P = self.model.particle_count
        offsets = torch.empty(P + 1, dtype=torch.int32, device=self.device)
        columns = torch.empty(info["nnzb"], dtype=torch.int32, device=self.device)
        values = torch.empty((info["nnzb"], 3, 3), dtype=torch.float32, device=self.device)
        _lib.check(self._lib.fem_export_bsr(self._handle, offsets.data_ptr(), columns.data_ptr(), values.data_ptr(),
                                            self._stream()))
        return BsrMatrix(offsets, columns, values, P)

    @property
    def _pc_inv_diag(self) -> torch.Tensor:
        out = torch.empty((self.model.particle_count, 3, 3), dtype=torch.float32, device=self.device)
        _lib.check(self._lib.fem_export_preconditioner(self._handle, out.data_ptr(), self._stream()))
        return out

    def _triplets(self):
        n = self.matrix_info()["triplets"]
        rows = torch.empty(n, dtype=torch.int32, device=self.device)
        cols = torch.empty(n, dtype=torch.int32, device=self.device)
        vals = torch.empty((n, 3, 3), dtype=torch.float32, device=self.device)
        _lib.check(self._lib.fem_export_triplets(self._handle, rows.data_ptr(), cols.data_ptr(), vals.data_ptr(),
                                                 self._stream()))
        return rows, cols, vals

    @property
    def bsr_values(self) -> torch.Tensor:
        return self._triplets()[2]

    @property
    def bsr_rows(self) -> torch.Tensor:
        return self._triplets()[0]

    @property
    def bsr_cols(self) -> torch.Tensor:
        return self._triplets()[1]

    # ------------------------------------------------------------------ force evaluators
    def _forces(self, state, terms: int, activations=None) -> torch.Tensor:
        P = self.model.particle_count
        out = torch.empty((P, 3), dtype=torch.float32, device=self.device)
        q = state.particle_q.detach().contiguous()
        v = state.particle_qd.detach().contiguous()
        _lib.check(self._lib.fem_eval_forces(self._handle, q.data_ptr(), v.data_ptr(), _ptr(activations),
                                             self.model.gravity.data_ptr(), terms, out.data_ptr(), self._stream()))
        return out

    def eval_tetrahedral_forces(self, model, control, state) -> torch.Tensor:
        act = None
        if self.enable_tet_activations and model.tet_count:
            act = (control.tet_activations if control is not None else model.tet_activations).contiguous()
        return self._forces(state, _lib.FEM_TERM_TET, act)

    def eval_hexahedral_forces(self, model, control, state) -> torch.Tensor:
        return self._forces(state, _lib.FEM_TERM_HEX)

    def eval_spring_forces(self, model, state) -> torch.Tensor:
        return self._forces(state, _lib.FEM_TERM_SPRING)

    def eval_triangle_forces(self, model, control, state) -> torch.Tensor:
        return self._forces(state, _lib.FEM_TERM_TRI)

    def eval_particle_particle_forces(self, model, control, state) -> torch.Tensor:
        return self._forces(state, _lib.FEM_TERM_PARTICLE)

    def eval_soft_contact_forces(self, model, state, contacts) -> torch.Tensor:
        self._register_contacts(contacts)
        return self._forces(state, _lib.FEM_TERM_SOFT_CONTACT)

    def eval_particle_ground_contact_forces(self, model, control, state) -> torch.Tensor:
        return self._forces(state, _lib.FEM_TERM_GROUND)

    def eval_gravity_forces(self, model) -> torch.Tensor:
        st = model.state()
        return self._forces(st, _lib.FEM_TERM_GRAVITY)

    def eval_linear_damping_forces(self, model, state) -> torch.Tensor:
        return self._forces(state, _lib.FEM_TERM_DAMPING)

    # ------------------------------------------------------------------ volume telemetry (not on the hot path)
    def _compute_volume(self, positions: torch.Tensor | None) -> float:
        total = 0.0
        m = self.model
        if m.tet_count and positions is not None:
            idx = m.tet_indices.long()
            p = positions.detach().double()
            e = p[idx[:, 1:]] - p[idx[:, :1]]  # [T, 3 edges, 3]
            # |e1 . (e2 x e3)| / 6, written out (no dependence on torch's linear-algebra backend)
            vol = (e[:, 0] * torch.cross(e[:, 1], e[:, 2], dim=1)).sum(dim=1).abs() / 6.0
            if self._tet_volume_weights is not None:
                vol = vol * torch.as_tensor(self._tet_volume_weights, device=vol.device).double()
            total += float(vol.sum())
        if self.hex_count:
            total += float(m.fem.hex_det_J0_w.double().sum())
        return total

    def compute_volume(self, state=None) -> float:
        return self._compute_volume(None if state is None else state.particle_q)

    def get_initial_volume(self, state=None) -> float:
        return self._initial_volume if self._initial_volume > 1e-12 else 1.0

    def get_volume_ratio(self, state=None) -> float:
        initial = self.get_initial_volume(state)
        current = self.compute_volume(state)
        if not math.isfinite(current) or current <= 0.0:
            return 1.0
        ratio = current / initial
        return ratio if math.isfinite(ratio) else 1.0


SolverLinearFEM = SolverFEM

"""Topology refresh and reassembly on the GPU (``-m gpu``).

``refresh_topology`` (reference ``solver.py:872-940``, sorted path) rebuilds
the pattern after in-place edits of tet connectivity and masses: the result
equals a solver built fresh on the edited model.  All three reassembly calls
restore fixed positions in the caller's array and assemble the same matrix as
an undisplaced state (reference ``tests/test_fixed_particles.py:122-140``).
"""

import numpy as np
import pytest
import torch
from gpu_helpers import DEVICE, rounded, tensor, to_np

from newton_solver_fem_gb300 import SolverFEM, model_from_arrays, scenes

pytestmark = pytest.mark.gpu

DT = 1.0 / 600.0


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def tet_model():
    x, tets, mats, mass = scenes.tet_block(4, 2, 2, 0.05, (0.0, 0.0, 0.0), 1.0e5, 0.45, 1000.0)
    model = model_from_arrays(rounded(x), rounded(mass), tets=tets, tet_materials=mats, gravity=(0.0, 0.0, -9.81),
                              device=DEVICE)
    fixed = np.nonzero(np.isclose(x[:, 0], 0.0))[0].astype(np.int32)
    return model, fixed


def make(model, fixed):
    return SolverFEM(model, dt=DT, solver_type="cg", preconditioner_type="block_diag", self_contact_ke=0.0,
                     linear_solver_tolerance=1.0e-6, linear_solver_maxiter=500, fixed_particle_indices=fixed)


def deformed(model, seed=0):
    rng = np.random.default_rng(seed)
    s = model.state()
    s.particle_q.add_(tensor(rng.normal(0, 1.0e-3, tuple(s.particle_q.shape))))
    return s


def test_refresh_topology_equals_a_fresh_solver_on_the_edited_model():
    model, fixed = tet_model()
    solver = make(model, fixed)
    state = deformed(model)
    solver.refresh_tangent(state.particle_q)
    nnzb_before = solver.matrix_info()["nnzb"]
    solver.velocity_increment.fill_(0.01)
    # edit in place: empty the last cube's six tets (zero materials, valid indices) and double some masses
    model.tet_materials[-6:] = 0.0
    heavy = torch.arange(0, model.particle_count, 7, device=DEVICE)
    model.particle_mass[heavy] *= 2.0
    model.particle_inv_mass[heavy] *= 0.5
    solver.refresh_topology(state.particle_q)
    fresh = make(model, fixed)
    fresh.refresh_tangent(state.particle_q)
    assert solver.matrix_info()["nnzb"] == fresh.matrix_info()["nnzb"] < nnzb_before
    np.testing.assert_array_equal(to_np(solver.velocity_increment), 0.0)
    np.testing.assert_allclose(solver.A_bsr.dense(), fresh.A_bsr.dense(), rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(to_np(solver._pc_inv_diag), to_np(fresh._pc_inv_diag), rtol=1e-6, atol=1e-6)
    outs = []
    for s in (solver, fresh):
        a, b = model.state(), model.state()
        a.particle_q.copy_(state.particle_q)
        s.step(a, b, None, None, DT)
        outs.append((to_np(b.particle_q), to_np(b.particle_qd)))
    np.testing.assert_allclose(outs[0][0], outs[1][0], rtol=0, atol=1e-8)
    np.testing.assert_allclose(outs[0][1], outs[1][1], rtol=0, atol=1e-6 * np.abs(outs[1][1]).max())


@pytest.mark.parametrize("method", ["refresh_tangent", "refresh_topology", "rebuild_element_blocks"])
def test_reassembly_uses_the_fixed_positions(method):
    model, fixed = tet_model()
    expected, actual = make(model, fixed), make(model, fixed)
    reference, changed = model.state(), model.state()
    positions = to_np(model.particle_q).copy()
    positions[fixed[-1]] += 0.0  # fixed nodes stay at rest in the reference
    positions[10] += (0.002, 0.001, -0.001)
    reference.particle_q.copy_(tensor(positions))
    positions[fixed] += (0.03, -0.02, 0.04)  # displaced supports in the changed input
    changed.particle_q.copy_(tensor(positions))
    getattr(expected, method)(reference.particle_q, DT)
    getattr(actual, method)(changed.particle_q, DT)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(to_np(changed.particle_q), to_np(reference.particle_q))
    np.testing.assert_array_equal(actual.A_bsr.dense(), expected.A_bsr.dense())
    e_out, a_out = model.state(), model.state()
    expected.step(reference, e_out, None, None, DT)
    actual.step(changed, a_out, None, None, DT)
    np.testing.assert_allclose(to_np(a_out.particle_qd), to_np(e_out.particle_qd), rtol=0, atol=1e-7)


def test_refresh_topology_rejections():
    model, fixed = tet_model()
    solver = make(model, fixed)
    with pytest.raises(ValueError, match="currently assembled timestep"):
        solver.refresh_topology(model.particle_q, DT / 2)
    # element lineage only matters to prepared (streaming) updates; the sorted path ignores it
    solver.refresh_topology(model.particle_q, element_sources=torch.zeros(1, dtype=torch.int32, device=DEVICE))
    model.tet_materials = model.tet_materials.clone()  # new storage: not an in-place edit
    with pytest.raises(ValueError, match="capacities and array storage"):
        solver.refresh_topology(model.particle_q)
